"""``jax.random`` stand-in.

NOT JAX's threefry stream: keys are (seed, counter) pairs and ``normal`` draws
from NumPy's PCG64.  Only good for finite-value smoke runs of the reference;
golden vectors built by this repo never depend on it.
"""

from __future__ import annotations

import numpy as _np

from .numpy import _wrap


def PRNGKey(seed):
    return _np.array([0, int(seed)], dtype=_np.uint32)


def split(key, num=2):
    base = int(key[1]) * 1000003 + int(key[0])
    return [_np.array([i + 1, base % (2 ** 32)], dtype=_np.uint32) for i in range(num)]


def normal(key, shape=(), dtype=_np.float64):
    rng = _np.random.default_rng([int(key[0]), int(key[1])])
    return _wrap(rng.standard_normal(shape).astype(dtype))
