"""Seeded initial states (host NumPy; transferred with ``solver.to_device``).

``theta_perturbation_state`` is the start of the benchmark configurations:
theta' = amplitude * N(0,1) * sin(pi Z) at the CGL nodes, drawn from NumPy's
PCG64 ``default_rng(seed)`` with shape (Nz+1, Nx, Nx); rfft2 per level, then
V^-1 and the Dirichlet pinv to Galerkin coefficients; q' = w = 0 and
Theta_bar = 0; finally the Hermitian projection of the ky=0 column and the
2/3 band limit (``sanitize_state`` semantics, nhqg/solver.py:128-146).
"""

from __future__ import annotations

import numpy as np

from .grid import Grid


def _sanitize_host(f: np.ndarray, Nx: int, mask: np.ndarray) -> np.ndarray:
    neg = (-np.arange(Nx)) % Nx
    f = f.copy()
    col = f[:, :, 0]
    f[:, :, 0] = 0.5 * (col + np.conj(col[:, neg]))
    col = f[:, :, -1]
    f[:, :, -1] = 0.5 * (col + np.conj(col[:, neg]))
    return f * mask[None]


def theta_perturbation_state(grid: Grid, seed: int = 0, amplitude: float = 1e-3):
    P, Nx = grid.Nz + 1, grid.Nx
    rng = np.random.default_rng(seed)
    th = amplitude * rng.standard_normal((P, Nx, Nx)) * np.sin(np.pi * grid.Z)[:, None, None]
    th_nodal = np.fft.rfft2(th)
    cols = th_nodal.reshape(P, -1)
    th_cheb = (grid.V_inv @ cols.view(np.float64)).view(np.complex128)
    th_gal = (grid.dirichlet_pinv @ th_cheb.view(np.float64)).view(np.complex128)
    th_gal = th_gal.reshape(P - 2, Nx, Nx // 2 + 1)
    q = np.zeros((P, Nx, Nx // 2 + 1), dtype=np.complex128)
    w = np.zeros_like(th_gal)
    return (q, w, _sanitize_host(th_gal, Nx, grid.mask_23), np.zeros(P))
