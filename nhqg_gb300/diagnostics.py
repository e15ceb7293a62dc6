"""Diagnostics of a state on the GB300 engine.

``compute_diagnostics(state, grid)`` returns the depth-integrated energies,
rms values and Nusselt numbers of the reference's ``compute_diagnostics``
(nhqg/diagnostics.py:597-690) under the same keys: KE_bt, KE_bc, KE_tot,
enstrophy, Nusselt, Nusselt_dealiased, vol_avg_tw, vol_avg_tw_dealiased,
q_rms, w_rms, th_rms, th_bar_max, the physical-space maxima over the Nx grid
at every CGL node max_speed, max_w, max_theta, max_tw (:631-641) and
heat_flux_mismatch.  The reference's budget terms are not computed.  The
reductions and the transforms to physical space run on the device
(``nhqg_diagnostics``); the call synchronises to return host floats.

``spectra(state, grid)`` returns the reference's ``energy_spectrum`` of psi
(nhqg/diagnostics.py:80-101), the q, w, theta horizontal shell spectra of
``compute_diagnostics`` (:104-111, 667-669) and ``vertical_mode_energy``
(:583-585) of q, w and theta, plus the psi kinetic energy per Chebyshev
index; the sums run on the device (``nhqg_spectra``).  ``high_mode_fraction`` (:588-594) and
``tail_fraction`` read a vertical spectrum.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .engine import engine_for
from .grid import Grid, compact_layout
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


_SHELLS: dict = {}


def shell_table(grid: Grid, n_bins: int | None = None):
    """(bin centres, shell index of every compact mode) under the reference's
    test i dk <= |k| < (i+1) dk with dk = 2 pi / L and n_bins = int(k_max / dk)
    + 1 by default, k_max over the whole rfft grid (nhqg/diagnostics.py:56-77).
    Compact mode m = r Mc + c holds kx row rows[r] and ky column c, with
    (rows, Mc) the engine's compact layout (grid.compact_layout)."""
    key = (id(grid), n_bins)
    if key not in _SHELLS:
        ksq = np.asarray(grid.ksq, dtype=np.float64)
        k_mag = np.sqrt(ksq)
        dk = 2.0 * np.pi / float(grid.L)
        k_max = np.sqrt(np.max(ksq))
        nb = int(float(k_max / dk)) + 1 if n_bins is None else int(n_bins)
        idx = np.full(ksq.shape, -1, dtype=np.int32)
        for i in range(nb):
            idx[(k_mag >= i * dk) & (k_mag < (i + 1) * dk)] = i
        rows, ncol = compact_layout(grid)
        compact = np.ascontiguousarray(idx[rows][:, :ncol].reshape(-1))
        _SHELLS[key] = (np.arange(nb) * dk + dk / 2, compact, grid)
    k_bins, compact, _ = _SHELLS[key]
    return k_bins, compact


def spectra(state, grid: Grid, n_bins: int | None = None) -> dict:
    """Shell energy spectrum of psi (k_bins, E_bt, E_bc, E_tot), vertical
    spectra (q, w, th: sum of |f_n|^2 over the modes; psi_ke: sum of
    w_k |k|^2 |psi_n|^2) and the horizontal shell spectra of q, w, theta at
    the CGL nodes (q_shell, w_shell, th_shell), as host float64 arrays;
    unnormalised like the reference."""
    s = to_device(state)
    k_bins, compact = shell_table(grid, n_bins)
    nb = len(k_bins)
    bins = torch.from_numpy(compact).to(s.q_hat.device)
    out = engine_for(grid).spectra(*s, bins, nb).cpu().numpy()
    P, G = grid.Nz + 1, grid.Nz - 1
    o = 3 * nb
    f = o + 2 * P + 2 * G
    return dict(k_bins=k_bins, E_bt=out[:nb], E_bc=out[nb:2 * nb], E_tot=out[2 * nb:o],
                q=out[o:o + P], w=out[o + P:o + P + G], th=out[o + P + G:o + P + 2 * G],
                psi_ke=out[o + P + 2 * G:f], q_shell=out[f:f + nb], w_shell=out[f + nb:f + 2 * nb],
                th_shell=out[f + 2 * nb:f + 3 * nb])


def high_mode_fraction(spec, frac: float = 0.25) -> float:
    """Share of a vertical spectrum in its top max(1, int(n frac)) entries
    (nhqg/diagnostics.py:588-594)."""
    spec = np.asarray(spec)
    n_tail = max(1, int(spec.shape[0] * frac))
    total = float(np.sum(spec))
    return float(np.sum(spec[-n_tail:]) / total) if total > 0 else 0.0


def tail_fraction(spec, n0: int) -> float:
    """Share of a vertical spectrum above Chebyshev index n0."""
    spec = np.asarray(spec)
    total = float(np.sum(spec))
    return float(np.sum(spec[n0 + 1:]) / total) if total > 0 else 0.0
