"""``jax.scipy.linalg`` stand-in over SciPy LAPACK."""

from __future__ import annotations

import numpy as _np
import scipy.linalg as _sla

from ..numpy import _wrap


def lu_factor(a, **kwargs):
    lu, piv = _sla.lu_factor(_np.asarray(a))
    return _wrap(lu), piv


def lu_solve(lu_and_piv, b, **kwargs):
    lu, piv = lu_and_piv
    return _wrap(_sla.lu_solve((_np.asarray(lu), piv), _np.asarray(b)))


def solve(a, b, **kwargs):
    return _wrap(_sla.solve(_np.asarray(a), _np.asarray(b)))
