"""Scalar diagnostics of a state on the GB300 engine.

``compute_diagnostics(state, grid)`` returns the depth-integrated energies,
rms values and Nusselt numbers of the reference's ``compute_diagnostics``
(nhqg/diagnostics.py:597-690) under the same keys: KE_bt, KE_bc, KE_tot,
enstrophy, Nusselt, Nusselt_dealiased, vol_avg_tw, vol_avg_tw_dealiased,
q_rms, w_rms, th_rms, th_bar_max.  The reference's shell spectra and budget
terms are not computed.  The reduction runs on the device
(``nhqg_diagnostics``); the call synchronises to return host floats.
"""

from __future__ import annotations

from . import _native as nat
from .engine import engine_for
from .grid import Grid
from .solver import to_device

DIAG_KEYS = nat.DIAG_KEYS


def compute_diagnostics_device(state, grid: Grid):
    """The diagnostics as a float64 CUDA tensor in ``DIAG_KEYS`` order
    (stream-ordered, no host synchronisation)."""
    s = to_device(state)
    return engine_for(grid).diagnostics(*s)


def compute_diagnostics(state, grid: Grid) -> dict[str, float]:
    vals = compute_diagnostics_device(state, grid).cpu().tolist()
    return dict(zip(DIAG_KEYS, vals))
