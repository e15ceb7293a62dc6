"""Dealiased horizontal products on the GB300 engine (2/3 and 3/2 rules).

Mirrors the reference's ``nhqg.spectral`` entry points used by the time step
(nhqg/spectral.py:53-75, 219-253, 331-358): same names and arguments, inputs
of shape (levels, Nx, Nx//2+1) complex (CUDA tensors or NumPy), outputs CUDA
tensors.  The 3/2-rule products run on the zero-padded Npad = 3Nx/2 grid.
"""

from __future__ import annotations

import hashlib

import numpy as np
import torch

from .config import NHQGConfig
from .engine import Engine
from .grid import make_grid

_SPECTRAL: dict[tuple, Engine] = {}


def _digest(a) -> str:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return hashlib.sha1(a.tobytes()).hexdigest()


def _engine(Nx: int, kx, ky, sponge_phys=None, rule: str = "23_rule") -> Engine:
    """A context with these wavenumbers (and sponge: sponge_phys on the Nx
    grid for the 2/3 rule, the padded sponge_phys_pad for the 3/2 rule)."""
    kx = np.asarray(kx, dtype=np.float64).reshape(Nx, 1)
    ky = np.asarray(ky, dtype=np.float64).reshape(1, Nx // 2 + 1)
    key = (Nx, rule, _digest(kx), _digest(ky), None if sponge_phys is None else _digest(sponge_phys))
    e = _SPECTRAL.get(key)
    if e is None:
        L = 2.0 * np.pi / ky[0, 1] if ky.shape[1] > 1 and ky[0, 1] != 0 else 2.0 * np.pi
        cfg = NHQGConfig(Nx=Nx, Nz=4, L=float(L), float_dtype="float64",
                         horizontal_dealiasing=rule, nonlinear_advection="flux")
        g = make_grid(cfg)
        sp = None if sponge_phys is None else np.ascontiguousarray(np.asarray(sponge_phys, dtype=np.float64))
        if rule == "32_rule":
            # the engine reads sponge_phys_pad; sponge_phys only marks "present"
            g = g._replace(kx=kx, ky=ky, sponge_phys_pad=sp,
                           sponge_phys=None if sp is None else np.zeros((Nx, Nx)))
        else:
            g = g._replace(kx=kx, ky=ky, sponge_phys=sp)
        e = Engine(g)
        _SPECTRAL[key] = e
    return e


def _check_mask(mask, Nx):
    K = Nx // 3
    ii = np.arange(Nx)
    kint = np.where(ii <= Nx // 2, ii, ii - Nx)
    ref = ((np.abs(kint)[:, None] <= K) & (np.arange(Nx // 2 + 1)[None, :] <= K))
    m = np.asarray(mask.cpu() if isinstance(mask, torch.Tensor) else mask)
    if m.shape != ref.shape or not np.array_equal(m != 0, ref):
        raise ValueError("mask must be the 2/3-rule keep-mask (|kx|, ky <= Nx//3)")


def _planes(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.to(device="cuda", dtype=torch.complex128)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.complex128))).to("cuda")
    if t.dim() == 2:
        t = t.unsqueeze(0)
    return t.contiguous()


def _host(a):
    return np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a)


def _check_npad(Nx, Npad):
    if int(Npad) != 3 * int(Nx) // 2:
        raise ValueError(f"Npad must be 3*Nx//2 = {3 * int(Nx) // 2} (nhqg/config.py:76-78), got {Npad}")


def _triple(form, psi, q, w, th, kx, ky, mask, Nx, rule="23_rule"):
    if rule == "23_rule":
        _check_mask(mask, Nx)
    e = _engine(Nx, _host(kx), _host(ky), rule=rule)
    ps, qq, ww, tt = (_planes(a) for a in (psi, q, w, th))
    outs = [torch.empty_like(qq) for _ in range(3)]
    e.triple_advection(form, ps, qq, ww, tt, *outs)
    return tuple(outs)


def triple_conservative_flux_divergence_23(psi_hat, q_hat, w_hat, th_hat, kx, ky, mask, Nx):
    """div(u f, v f), u = -psi_y, v = psi_x, f in (q, w, th), 2/3-masked."""
    return _triple("flux", psi_hat, q_hat, w_hat, th_hat, kx, ky, mask, Nx)


def triple_jacobian_23(psi_hat, q_hat, w_hat, th_hat, kx, ky, mask, Nx):
    """J[psi, f] = psi_x f_y - psi_y f_x for f in (q, w, th), 2/3-masked."""
    return _triple("jacobian", psi_hat, q_hat, w_hat, th_hat, kx, ky, mask, Nx)


def triple_conservative_flux_divergence(psi_hat, q_hat, w_hat, th_hat, kx, ky, Nx, Npad):
    """div(u f, v f) under the 3/2 rule: zero-padded to Npad = 3Nx/2,
    products on the padded grid, truncated (nhqg/spectral.py:190-216, 237-253)."""
    _check_npad(Nx, Npad)
    return _triple("flux", psi_hat, q_hat, w_hat, th_hat, kx, ky, None, Nx, rule="32_rule")


def triple_jacobian(psi_hat, q_hat, w_hat, th_hat, kx, ky, Nx, Npad):
    """J[psi, f] for f in (q, w, th) under the 3/2 rule (nhqg/spectral.py:147-180, 219-234)."""
    _check_npad(Nx, Npad)
    return _triple("jacobian", psi_hat, q_hat, w_hat, th_hat, kx, ky, None, Nx, rule="32_rule")


def sponge_product_32(f_hat, sponge_phys_pad, Nx, Npad):
    """truncate(rfft2(sigma_pad * irfft2(pad f))) per level, sigma_pad the
    pre-attenuated padded sponge (nhqg/spectral.py:63-75)."""
    _check_npad(Nx, Npad)
    L = 2.0 * np.pi
    kx = 2.0 * np.pi * np.fft.fftfreq(Nx, d=L / Nx)
    ky = 2.0 * np.pi * np.arange(Nx // 2 + 1) / L
    sp = _host(sponge_phys_pad)
    if sp.shape != (int(Npad), int(Npad)):
        raise ValueError(f"sponge_phys_pad must be ({Npad}, {Npad}), got {sp.shape}")
    e = _engine(Nx, kx, ky, sponge_phys=sp, rule="32_rule")
    f = _planes(f_hat)
    out = torch.empty_like(f)
    e.sponge_product(f, out)
    return out


def sponge_product_23(f_hat, sponge_phys, mask, Nx):
    """mask * rfft2(sigma * irfft2(f)) per level."""
    _check_mask(mask, Nx)
    L = 2.0 * np.pi
    kx = 2.0 * np.pi * np.fft.fftfreq(Nx, d=L / Nx)
    ky = 2.0 * np.pi * np.arange(Nx // 2 + 1) / L
    sp = np.asarray(sponge_phys.cpu() if isinstance(sponge_phys, torch.Tensor) else sponge_phys)
    e = _engine(Nx, kx, ky, sponge_phys=sp)
    f = _planes(f_hat)
    out = torch.empty_like(f)
    e.sponge_product(f, out)
    return out
