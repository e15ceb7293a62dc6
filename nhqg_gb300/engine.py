"""One native engine context per Grid: table upload and typed entry points.

PyTorch supplies device memory and the current CUDA stream; every compute
call goes through the C ABI of ``libnhqg_gpu.so`` (include/nhqg_gpu.h).
"""

from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _native as nat
from .grid import Grid, _zero_pad

_ENGINES: dict[tuple, "Engine"] = {}


def _dptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(nat.c_double_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _stream_handle() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def require_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("the NHQG GB300 engine needs a CUDA device (no CPU fallback)")


class Engine:
    """Native context built from a Grid; ``closure``/``exchange`` flags of the
    Grid select the stepper, per-operator calls pass them explicitly."""

    def __init__(self, grid: Grid):
        require_cuda()
        self.lib = nat.load()
        self.grid = grid
        g = grid
        self.P, self.G, self.Nx, self.Nk = g.Nz + 1, g.Nz - 1, g.Nx, g.Nk
        keep = {}

        def arr(name, a):
            keep[name] = _f64(a)
            return _dptr(keep[name])

        d = nat.GridDesc()
        d.Nx, d.Nz = g.Nx, g.Nz
        d.advection = nat.ADV[g.nonlinear_advection]
        d.thermal_closure = nat.CLOSURE[g.thermal_closure]
        d.exchange = nat.EXCHANGE[g.mean_exchange_discretization]
        d.w_bc_top = nat.WBC[g.w_bc_top]
        d.substeps = max(1, int(g.sbp_corrector_substeps))
        d.n_shells = int(g.imex_inv.shape[0])
        d.dt, d.gamma_imex, d.Ra_sigma = g.dt, g.gamma_imex, g.Ra_sigma
        d.sigma, d.beta, d.eps_sq = g.sigma, g.beta, g.mean_temp_eps_sq
        d.kx = arr("kx", np.ravel(g.kx))
        d.ky = arr("ky", np.ravel(g.ky))
        for name in ("inv_denom", "diss_rate_q", "diss_rate_w", "diss_rate_th", "inv_alpha_q",
                     "inv_alpha_th", "V", "V_inv", "w_stencil", "G_Z", "proj_dirichlet", "sbp_D1",
                     "sbp_L", "cgl_to_sbp", "sbp_to_cgl"):
            setattr(d, name, arr(name, getattr(g, name)))
        rows = np.ascontiguousarray(np.where(g.imex_shell_row >= 0, g.imex_shell_row, 0), dtype=np.int32)
        keep["rows"] = rows
        d.shell_of_mode = rows.ctypes.data_as(nat.c_int_p)
        keep["shell_inv"] = np.ascontiguousarray(g.imex_inv, dtype=np.float64)
        d.shell_inv = _dptr(keep["shell_inv"])
        self.pad32 = g.horizontal_dealiasing == "32_rule"
        d.horizontal_dealiasing = nat.DEALIAS[g.horizontal_dealiasing]
        if g.eta_hat is not None:
            e = np.ascontiguousarray(np.asarray(g.eta_hat, dtype=np.complex128))
            keep["eta"] = e
            d.eta_hat = ctypes.cast(e.ctypes.data, nat.c_double_p)
            # physical eta on the products' grid, derived from eta_hat so that a
            # replaced eta_hat cannot disagree with it
            kx = np.asarray(g.kx, dtype=np.float64).reshape(-1)[:, None]
            ky = np.asarray(g.ky, dtype=np.float64).reshape(-1)[None, :g.Nk]
            parts = {"eta_phys": e, "eta_x_phys": 1j * kx * e, "eta_y_phys": 1j * ky * e}
            for name, spec in parts.items():
                if self.pad32:
                    phys = np.fft.irfft2(_zero_pad(spec, g.Nx, g.Npad), s=(g.Npad, g.Npad))
                else:
                    phys = np.fft.irfft2(spec, s=(g.Nx, g.Nx))
                setattr(d, name, arr(name, phys))
        sponge = g.sponge_phys_pad if self.pad32 else g.sponge_phys
        if g.sponge_phys is not None and sponge is None:
            raise ValueError("a 3/2-rule grid with a sponge needs sponge_phys_pad")
        if sponge is not None:
            d.sponge_phys = arr("sponge", sponge)
        if g.mean_solve is not None:
            d.mean_solve = arr("mean_solve", g.mean_solve)
        if getattr(g, "imex_shell_coef", None) is not None:
            d.shell_coef = arr("shell_coef", np.ravel(g.imex_shell_coef))
        d.cc_weights = arr("cc_weights", g.cc_weights)
        d.imex_scheme = nat.SCHEME[g.imex_scheme]
        self._desc = d
        handle = ctypes.c_void_p()
        nat.check(self.lib.nhqg_ctx_create(ctypes.byref(d), ctypes.byref(handle)), "nhqg_ctx_create")
        self.handle = handle
        self.precision = "fp64"
        self._finalizer = weakref.finalize(self, Engine._destroy, self.lib, handle.value)

    @staticmethod
    def _destroy(lib, h):
        if h:
            lib.nhqg_ctx_destroy(ctypes.c_void_p(h))

    # ------------------------------------------------------------- helpers
    def state_desc(self, q, w, th, tb) -> nat.StateDesc:
        for t, n, nl in ((q, "q_hat", self.P), (w, "w_hat", self.G), (th, "th_hat", self.G)):
            if t.dtype != torch.complex128 or not t.is_cuda or not t.is_contiguous():
                raise ValueError(f"{n} must be a contiguous complex128 CUDA tensor")
            if tuple(t.shape) != (nl, self.Nx, self.Nk):
                raise ValueError(f"{n} has shape {tuple(t.shape)}, expected {(nl, self.Nx, self.Nk)}")
        if tb.dtype != torch.float64 or not tb.is_cuda or tuple(tb.shape) != (self.P,):
            raise ValueError("th_bar must be a float64 CUDA tensor of shape (Nz+1,)")
        return nat.StateDesc(q.data_ptr(), w.data_ptr(), th.data_ptr(), tb.data_ptr())

    def device_status(self, reset: bool = True) -> int:
        return int(self.lib.nhqg_get_device_status(self.handle, 1 if reset else 0))

    def profile(self, on: bool) -> None:
        nat.check(self.lib.nhqg_profile_enable(self.handle, 1 if on else 0), "nhqg_profile_enable")

    def profile_report(self) -> dict[str, tuple[int, float]]:
        """{kernel class: (launches, total ms)} since profile(True)."""
        buf = ctypes.create_string_buffer(1 << 16)
        nat.check(self.lib.nhqg_profile_report(self.handle, buf, len(buf)), "nhqg_profile_report")
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split()
            out[name] = (int(n), float(ms))
        return out

    def launches(self) -> int:
        return int(self.lib.nhqg_last_launch_count(self.handle))

    def set_precision(self, precision: str) -> None:
        """'fp64' (plain path) or 'mixed' (FP32 products and transforms,
        double-float column algebra and corrector transforms, FP64 solves) for
        the following step / RHS / solve calls."""
        if precision not in nat.PRECISION:
            raise ValueError(f"precision must be one of {sorted(nat.PRECISION)}, got {precision!r}")
        if precision != self.precision:
            nat.check(self.lib.nhqg_set_precision(self.handle, nat.PRECISION[precision]),
                      f"nhqg_set_precision({precision!r})")
            self.precision = precision

    @property
    def tensor_core_vertical(self) -> bool:
        """True if the mixed path's Chebyshev <-> nodal transforms run on the
        tensor cores (else the FP32 fast DCT)."""
        return bool(self.lib.nhqg_get_mixed_vertical(self.handle))

    @tensor_core_vertical.setter
    def tensor_core_vertical(self, on: bool) -> None:
        nat.check(self.lib.nhqg_set_mixed_vertical(self.handle, int(bool(on))),
                  "nhqg_set_mixed_vertical")

    def tc_to_nodal(self, field: int, coef: torch.Tensor, nodal: torch.Tensor) -> None:
        """Tensor-core _to_nodal of compact coefficients (complex128, field 0 q
        (Nz+1, M), 1 w / 2 theta (Nz-1, M)) into nodal (Nz+1, M) complex64."""
        nat.check(self.lib.nhqg_tc_to_nodal(self.handle, int(field), ctypes.c_void_p(coef.data_ptr()),
                                            ctypes.c_void_p(nodal.data_ptr()), _stream_handle()),
                  "nhqg_tc_to_nodal")

    def tc_to_coef(self, nodal: torch.Tensor) -> None:
        """Tensor-core _to_coeffs of compact nodal values (Nz+1, M) complex64, in place."""
        nat.check(self.lib.nhqg_tc_to_coef(self.handle, ctypes.c_void_p(nodal.data_ptr()),
                                           _stream_handle()), "nhqg_tc_to_coef")

    # ------------------------------------------------------------- entry points
    def step(self, q, w, th, tb, n_steps: int = 1, precision: str = "fp64") -> None:
        self.set_precision(precision)
        s = self.state_desc(q, w, th, tb)
        nat.check(self.lib.nhqg_step(self.handle, ctypes.byref(s), int(n_steps), _stream_handle()),
                  "nhqg_step")

    def explicit_rhs(self, src, dst, closure: str, exchange: str, precision: str = "fp64") -> None:
        self.set_precision(precision)
        a, b = self.state_desc(*src), self.state_desc(*dst)
        nat.check(self.lib.nhqg_explicit_rhs(self.handle, ctypes.byref(a), ctypes.byref(b),
                                             nat.CLOSURE[closure], nat.EXCHANGE[exchange],
                                             _stream_handle()), "nhqg_explicit_rhs")

    def implicit_tendency(self, src, dst, closure: str) -> None:
        a, b = self.state_desc(*src), self.state_desc(*dst)
        nat.check(self.lib.nhqg_implicit_tendency(self.handle, ctypes.byref(a), ctypes.byref(b),
                                                  nat.CLOSURE[closure], _stream_handle()),
                  "nhqg_implicit_tendency")

    def implicit_solve(self, src, dst, closure: str, precision: str = "fp64") -> None:
        self.set_precision(precision)
        a, b = self.state_desc(*src), self.state_desc(*dst)
        nat.check(self.lib.nhqg_implicit_solve(self.handle, ctypes.byref(a), ctypes.byref(b),
                                               nat.CLOSURE[closure], _stream_handle()),
                  "nhqg_implicit_solve")

    def mean_temp_solve(self, R, out, closure: str) -> None:
        nat.check(self.lib.nhqg_mean_temp_solve(self.handle, R.data_ptr(), out.data_ptr(),
                                                nat.CLOSURE[closure], _stream_handle()),
                  "nhqg_mean_temp_solve")

    def corrector(self, src, dst, total_dt: float) -> None:
        a, b = self.state_desc(*src), self.state_desc(*dst)
        nat.check(self.lib.nhqg_sbp2_corrector(self.handle, ctypes.byref(a), ctypes.byref(b),
                                               float(total_dt), _stream_handle()),
                  "nhqg_sbp2_corrector")

    def sanitize(self, q, w, th, tb) -> None:
        s = self.state_desc(q, w, th, tb)
        nat.check(self.lib.nhqg_sanitize(self.handle, ctypes.byref(s), _stream_handle()), "nhqg_sanitize")

    def triple_advection(self, advection: str, psi, q, w, th, Aq, Aw, Ath) -> None:
        """The grid's products (2/3 or 3/2 rule) of (levels, Nx, Nk) planes."""
        levels = int(q.shape[0])
        name = "nhqg_triple_advection_32" if self.pad32 else "nhqg_triple_advection_23"
        nat.check(getattr(self.lib, name)(
            self.handle, nat.ADV[advection], levels, psi.data_ptr(), q.data_ptr(), w.data_ptr(),
            th.data_ptr(), Aq.data_ptr(), Aw.data_ptr(), Ath.data_ptr(), _stream_handle()), name)

    def diagnostics(self, q, w, th, tb) -> torch.Tensor:
        """NHQG_DIAG_COUNT doubles on the device (order of _native.DIAG_KEYS)."""
        s = self.state_desc(q, w, th, tb)
        out = torch.empty(len(nat.DIAG_KEYS), dtype=torch.float64, device=q.device)
        nat.check(self.lib.nhqg_diagnostics(self.handle, ctypes.byref(s), ctypes.c_void_p(out.data_ptr()),
                                            _stream_handle()), "nhqg_diagnostics")
        return out

    def spectra(self, q, w, th, tb, mode_bin: torch.Tensor, n_bins: int) -> torch.Tensor:
        """3 n_bins shell energies, the vertical spectra of q, w, theta and
        the psi kinetic energy, then the q, w, theta shell spectra (3 n_bins),
        on the device (layout of nhqg_spectra)."""
        s = self.state_desc(q, w, th, tb)
        P, G = int(q.shape[0]), int(w.shape[0])
        out = torch.empty(6 * n_bins + 2 * P + 2 * G, dtype=torch.float64, device=q.device)
        nat.check(self.lib.nhqg_spectra(self.handle, ctypes.byref(s), ctypes.c_void_p(mode_bin.data_ptr()),
                                        int(n_bins), ctypes.c_void_p(out.data_ptr()), _stream_handle()),
                  "nhqg_spectra")
        return out

    def tiles(self) -> tuple[int, int, int, int]:
        """Horizontal-product tile budgets in KiB (FP64 col, FP64 row, FP32 col,
        FP32 row); 0 = built-in default."""
        t = (ctypes.c_int * 4)()
        nat.check(self.lib.nhqg_get_tiles(self.handle, t), "nhqg_get_tiles")
        return tuple(t)

    def set_tiles(self, tiles) -> None:
        t = (ctypes.c_int * 4)(*[int(v) for v in tiles])
        nat.check(self.lib.nhqg_set_tiles(self.handle, t), "nhqg_set_tiles")

    def autotune(self) -> tuple[int, int, int, int]:
        """Time candidate tiles on this context's buffers (both precisions once
        the mixed path is enabled), keep the fastest, return them."""
        nat.check(self.lib.nhqg_autotune(self.handle, _stream_handle()), "nhqg_autotune")
        return self.tiles()

    def sponge_product(self, f, out) -> None:
        name = "nhqg_sponge_product_32" if self.pad32 else "nhqg_sponge_product_23"
        nat.check(getattr(self.lib, name)(self.handle, int(f.shape[0]), f.data_ptr(),
                                          out.data_ptr(), _stream_handle()), name)


def _key(grid: Grid) -> tuple:
    return (id(grid.imex_inv), id(grid.V), id(grid.eta_hat), id(grid.sponge_phys),
            id(grid.sponge_phys_pad), grid.horizontal_dealiasing,
            id(grid.cgl_to_sbp), grid.thermal_closure, grid.mean_exchange_discretization,
            grid.nonlinear_advection, grid.w_bc_top, int(grid.sbp_corrector_substeps),
            float(grid.dt), float(grid.beta), float(grid.mean_temp_eps_sq))


def engine_for(grid: Grid) -> Engine:
    """Cached Engine of a Grid (one native context per Grid contents)."""
    k = _key(grid)
    e = _ENGINES.get(k)
    if e is None:
        e = Engine(grid)
        _ENGINES[k] = e
        weakref.finalize(grid.imex_inv, _ENGINES.pop, k, None)
    return e
