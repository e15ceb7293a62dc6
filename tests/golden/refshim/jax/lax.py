"""``jax.lax`` stand-in: sequential scan and map."""

from __future__ import annotations

import numpy as _np

from .numpy import _wrap


def scan(f, init, xs=None, length=None):
    n = length if xs is None else len(xs)
    carry = init
    ys = []
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    if ys and ys[0] is not None:
        return carry, _wrap(_np.stack([_np.asarray(y) for y in ys]))
    return carry, None


def map(f, xs):
    from . import _index_tree, _stack_tree, _leading_len

    n = _leading_len((xs,), (0,))
    return _stack_tree([f(_index_tree(xs, i)) for i in range(n)])
