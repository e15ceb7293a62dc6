"""Checkpoint files in the reference's npz schema (nhqg/io.py:107-153).

``save_checkpoint`` writes ``checkpoint_<step:08d>.npz`` with the keys
q_hat_real/q_hat_imag, w_hat_real/w_hat_imag, th_hat_real/th_hat_imag,
th_bar, step and t = step * dt, so a GPU run can be resumed by the reference
and the reverse.  ``load_checkpoint`` applies the reference's load-time
Hermitian projection of the ky = 0 and Nyquist columns; with
``band_limit=True`` it also applies the 2/3 band limit (``sanitize_state``
semantics), which the GPU step requires of its input.
"""

from __future__ import annotations

import os
from pathlib import Path

import numpy as np


def _host(a) -> np.ndarray:
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(a)


def save_checkpoint(state, step: int, cfg, output_dir: str | None = None) -> str:
    if output_dir is None:
        output_dir = cfg.output_dir
    Path(output_dir).mkdir(parents=True, exist_ok=True)
    fname = os.path.join(output_dir, f"checkpoint_{step:08d}.npz")
    q, w, th, tb = (_host(x) for x in state)
    np.savez(fname, q_hat_real=q.real, q_hat_imag=q.imag, w_hat_real=w.real, w_hat_imag=w.imag,
             th_hat_real=th.real, th_hat_imag=th.imag, th_bar=tb, step=step, t=step * cfg.dt)
    return fname


def _hermitian_project(f: np.ndarray) -> np.ndarray:
    Nx = f.shape[1]
    neg = (-np.arange(Nx)) % Nx
    f = np.array(f)
    f[:, :, 0] = 0.5 * (f[:, :, 0] + np.conj(f[:, neg, 0]))
    if Nx % 2 == 0:
        f[:, :, -1] = 0.5 * (f[:, :, -1] + np.conj(f[:, neg, -1]))
    return f


def _band_limit(f: np.ndarray) -> np.ndarray:
    Nx, Nk = f.shape[1], f.shape[2]
    K = Nx // 3
    ii = np.arange(Nx)
    kint = np.where(ii <= Nx // 2, ii, ii - Nx)
    mask = (np.abs(kint)[:, None] <= K) & (np.arange(Nk)[None, :] <= K)
    return f * mask[None]


def load_checkpoint(path: str, to_device: bool = True, band_limit: bool = False):
    """Returns (state, step, t); the state is a solver.State of CUDA tensors
    (``to_device``) or a tuple of NumPy arrays."""
    data = np.load(path)
    fields = []
    for name in ("q_hat", "w_hat", "th_hat"):
        f = _hermitian_project(data[f"{name}_real"] + 1j * data[f"{name}_imag"])
        fields.append(_band_limit(f) if band_limit else f)
    th_bar = (np.asarray(data["th_bar"], dtype=np.float64) if "th_bar" in data
              else np.zeros(fields[0].shape[0]))
    state = (*fields, th_bar)
    if to_device:
        from .solver import to_device as _dev
        state = _dev(state)
    return state, int(data["step"]), float(data["t"])
