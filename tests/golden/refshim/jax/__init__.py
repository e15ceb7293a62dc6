"""NumPy stand-in for the ``jax`` package, used ONLY to execute the
unmodified NHQG reference source in a container without JAX.

Test infrastructure: it lets ``tests/golden/make_golden.py`` import the
reference's ``nhqg`` package and record golden input/output vectors.  It is
never imported by the product package, the tests that run on the GPU host, or
``bench.py``.

Semantics covered (what the reference's hot path touches):
  * ``jax.numpy`` ~ numpy, with arrays that carry ``.at[idx].set/add/multiply``
  * ``jit`` (identity, with or without static_argnums), ``vmap`` (loop over
    axis 0 and stack), ``lax.scan`` / ``lax.map``
  * ``scipy.linalg.lu_factor`` / ``lu_solve`` (SciPy LAPACK)
  * ``device_put`` / ``devices`` / ``default_backend`` as host no-ops
  * ``random``: NOT JAX's threefry stream -- a NumPy PCG64 stream keyed by the
    seed, sufficient for finite-value smoke tests only.
"""

from __future__ import annotations

import functools as _ft

import numpy as _np

from . import numpy  # noqa: F401  (jax.numpy)
from . import lax  # noqa: F401
from . import random  # noqa: F401
from . import scipy  # noqa: F401
from . import sharding  # noqa: F401
from .numpy import _wrap, _JArray

Array = _JArray


class _Config:
    def update(self, *args, **kwargs):
        return None

    jax_enable_x64 = True


config = _Config()


def jit(fun=None, **kwargs):
    """Identity decorator (tracing/compilation has no NumPy analogue)."""
    if fun is None:
        return lambda f: f
    return fun


def _index_tree(x, i):
    if isinstance(x, tuple) and not hasattr(x, "_fields"):
        return tuple(_index_tree(e, i) for e in x)
    if hasattr(x, "_fields"):
        return type(x)(*(_index_tree(e, i) for e in x))
    if isinstance(x, list):
        return [_index_tree(e, i) for e in x]
    if x is None:
        return None
    return x[i]


def _stack_tree(items):
    first = items[0]
    if isinstance(first, tuple) and not hasattr(first, "_fields"):
        return tuple(_stack_tree([it[j] for it in items]) for j in range(len(first)))
    if hasattr(first, "_fields"):
        return type(first)(*(_stack_tree([it[j] for it in items]) for j in range(len(first))))
    if isinstance(first, list):
        return [_stack_tree([it[j] for it in items]) for j in range(len(first))]
    return _wrap(_np.stack([_np.asarray(it) for it in items]))


def _leading_len(args, in_axes):
    for a, ax in zip(args, in_axes):
        if ax is None:
            continue
        leaf = a
        while isinstance(leaf, (tuple, list)):
            leaf = leaf[0]
        return _np.asarray(leaf).shape[0]
    raise ValueError("vmap needs at least one mapped argument")


def vmap(fun, in_axes=0, out_axes=0):
    """Loop over axis 0 of each mapped argument and stack the results."""

    @_ft.wraps(fun)
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        for ax in axes:
            if ax not in (0, None):
                raise NotImplementedError("stand-in vmap supports in_axes 0/None")
        n = _leading_len(args, axes)
        outs = []
        for i in range(n):
            call = [a if ax is None else _index_tree(a, i) for a, ax in zip(args, axes)]
            outs.append(fun(*call))
        return _stack_tree(outs)

    return mapped


def device_put(x, *args, **kwargs):
    return x


def devices(*args, **kwargs):
    return ["cpu:0"]


def default_backend():
    return "cpu"


def block_until_ready(x):
    return x
