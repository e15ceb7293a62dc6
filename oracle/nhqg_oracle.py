"""NumPy restatement of the NHQG ARS(2,2,2) IMEX step (test oracle).

TEST INFRASTRUCTURE -- see ``oracle/__init__.py``.  Fields are NumPy arrays in
the reference layout: spectral ``(levels, Nx, Nx//2+1)`` complex128 with ky
contiguous and kx in fftfreq order; ``th_bar`` is ``(Nz+1,)`` float64.

Covered branches (the time-step hot path and its documented variants):
horizontal products under the 2/3 rule or the 3/2 rule (zero-padded) in flux
or Jacobian form, polar trap
eta, Rayleigh sponge, Dirichlet or open-top (Neumann) w basis,
``q_boundary='none'``, thermal closures ``fixed_conduction`` and
``evolve_mean`` with ``legacy`` / ``balanced_sbp2`` / ``balanced_sbp2_pc``
exchange, ``imex_scheme='ars222'`` and (legacy exchange) ``'rk443'``.
"""

from __future__ import annotations

import dataclasses
import os
from typing import NamedTuple

import numpy as np
import scipy.fft as sfft
import scipy.linalg as sla

_WORKERS = int(os.environ.get("NHQG_ORACLE_THREADS", "0")) or (os.cpu_count() or 1)


def set_threads(n: int) -> None:
    """FFT worker threads used by the oracle (BLAS threads follow the env)."""
    global _WORKERS
    _WORKERS = max(1, int(n))


# ---------------------------------------------------------------------------
# Configuration -- field names and defaults of nhqg/config.py:16-68
# ---------------------------------------------------------------------------

@dataclasses.dataclass(frozen=True)
class OracleConfig:
    Nx: int = 256
    Nz: int = 32
    Ra_tilde: float = 100.0
    sigma: float = 1.0
    beta: float = 0.0
    gamma: float = 0.0
    trap_r_star: float | None = None
    trap_sharpness: float = 20.0
    sponge_rate: float = 0.0
    sponge_r_start: float | None = None
    sponge_sharpness: float = 20.0
    Ld: float = float("inf")
    L: float = 20.0
    thermal_closure: str = "fixed_conduction"
    mean_temp_eps_sq: float = 1.0
    q_boundary: str = "none"
    w_bc_top: str = "dirichlet"
    nonlinear_advection: str = "jacobian"
    dt: float = 1e-3
    t_final: float = 100.0
    imex_scheme: str = "ars222"
    nu_q: float = 0.0
    hyper_order: int = 4
    nu_w: float = 0.0
    nu_theta: float = 0.0
    drag: float = 0.0
    save_interval: int = 100
    output_dir: str = "output"
    float_dtype: str = "float32"
    vertical_cutoff_n: int | None = None
    vertical_dealiasing: str = "none"
    horizontal_dealiasing: str = "32_rule"
    mean_exchange_discretization: str = "legacy"
    sbp_transfer_mode: str = "interp"
    sbp_corrector_substeps: int = 1
    imex_matmul_chunk: int = 0

    @property
    def Nk(self) -> int:
        return self.Nx // 2 + 1

    @property
    def Npad(self) -> int:
        return 3 * self.Nx // 2

    @property
    def Ld_inv_sq(self) -> float:
        return 0.0 if self.Ld == float("inf") else 1.0 / self.Ld ** 2


class OracleState(NamedTuple):
    """nhqg/solver.py:33-38."""
    q_hat: np.ndarray
    w_hat: np.ndarray
    th_hat: np.ndarray
    th_bar: np.ndarray


# ---------------------------------------------------------------------------
# Vertical operators -- nhqg/grid.py
# ---------------------------------------------------------------------------

def cheb_diff_matrix(N: int) -> np.ndarray:
    """d/dxi on Chebyshev coefficients via the backward recurrence
    b_{N-1} = 2N a_N, b_k = b_{k+2} + 2(k+1) a_{k+1}, b_0 = b_2/2 + a_1
    (nhqg/grid.py:148-169), applied to each unit vector."""
    G = np.zeros((N + 1, N + 1))
    for n in range(N + 1):
        a = np.zeros(N + 1)
        a[n] = 1.0
        b = np.zeros(N + 1)
        if N >= 1:
            b[N - 1] = 2.0 * N * a[N]
            for k in range(N - 2, 0, -1):
                b[k] = b[k + 2] + 2.0 * (k + 1) * a[k + 1]
            b[0] = (0.5 * b[2] if N >= 2 else 0.0) + a[1]
        G[:, n] = b
    return G


def cc_weights(N: int) -> np.ndarray:
    """Clenshaw-Curtis weights on [0,1] (nhqg/grid.py:176-189)."""
    theta = np.pi * np.arange(N + 1) / N
    w = np.zeros(N + 1)
    for j in range(N + 1):
        s = 0.0
        for k in range(1, N // 2 + 1):
            b = 1.0 if k == N // 2 else 2.0
            s += b * np.cos(2.0 * k * theta[j]) / (4.0 * k * k - 1.0)
        c_j = 2.0 if j in (0, N) else 1.0
        w[j] = (1.0 - s) / (N * c_j)
    return w


def cheb_vandermonde(N: int) -> tuple[np.ndarray, np.ndarray]:
    """V[j,n] = cos(pi j n / N) and its DCT-I inverse (nhqg/grid.py:192-201)."""
    j = np.arange(N + 1, dtype=np.float64)
    V = np.cos(np.outer(j, j) * (np.pi / N))
    c = np.ones(N + 1)
    c[0] = c[N] = 2.0
    inv_c = 1.0 / c
    V_inv = (2.0 / N) * np.outer(inv_c, inv_c) * V.T
    return V, V_inv


def piecewise_linear_interp(x_src: np.ndarray, x_dst: np.ndarray) -> np.ndarray:
    """Row-stochastic linear interpolation matrix (nhqg/grid.py:229-258)."""
    reverse = bool(x_src[0] > x_src[-1])
    xs = x_src[::-1] if reverse else x_src
    M = np.zeros((x_dst.size, xs.size))
    for i, x in enumerate(x_dst):
        if x <= xs[0]:
            M[i, 0] = 1.0
            continue
        if x >= xs[-1]:
            M[i, -1] = 1.0
            continue
        j = int(np.searchsorted(xs, x, side="right") - 1)
        t = (x - xs[j]) / (xs[j + 1] - xs[j])
        M[i, j] = 1.0 - t
        M[i, j + 1] = t
    return M[:, ::-1] if reverse else M


def sbp2_operators(N: int):
    """Uniform-grid SBP2 norm H, first derivative D1, Laplacian L with zero
    boundary rows (nhqg/grid.py:261-286)."""
    dz = 1.0 / N
    n = N + 1
    h = np.ones(n)
    h[0] = h[-1] = 0.5
    H = dz * np.diag(h)
    D1 = np.zeros((n, n))
    D1[0, 0], D1[0, 1] = -1.0 / dz, 1.0 / dz
    for i in range(1, N):
        D1[i, i - 1], D1[i, i + 1] = -0.5 / dz, 0.5 / dz
    D1[N, N - 1], D1[N, N] = -1.0 / dz, 1.0 / dz
    L = np.zeros((n, n))
    for i in range(1, N):
        L[i, i - 1], L[i, i], L[i, i + 1] = 1.0 / dz ** 2, -2.0 / dz ** 2, 1.0 / dz ** 2
    return H, D1, L


def tau_projection(tau_rows: np.ndarray, N: int) -> np.ndarray:
    """Projection that rewrites a_{N-1}, a_N to satisfy two tau rows
    (nhqg/grid.py:293-319)."""
    M_inv = np.linalg.inv(tau_rows[:, N - 1:N + 1])
    R = tau_rows[:, :N - 1]
    MR = M_inv @ R
    P = np.eye(N + 1)
    P[N - 1, :N - 1] = -MR[0]
    P[N - 1, N - 1] = P[N - 1, N] = 0.0
    P[N, :N - 1] = -MR[1]
    P[N, N - 1] = P[N, N] = 0.0
    return P


def mixed_stencil(N: int) -> np.ndarray:
    """Shen basis T_n + a_n T_{n+1} + b_n T_{n+2}: Dirichlet bottom, Neumann top
    (nhqg/grid.py:322-342)."""
    S = np.zeros((N + 1, N - 1))
    for n in range(N - 1):
        b = -(n ** 2 + (n + 1) ** 2) / ((n + 1) ** 2 + (n + 2) ** 2)
        S[n, n], S[n + 1, n], S[n + 2, n] = 1.0, 1.0 + b, b
    return S


def build_shell_inverses(G_Z, w_stencil, w_pinv, ksq_flat, Ld_inv_sq, dt, gamma,
                         Nz, nu_q, nu_w, nu_theta, sigma, Ra_sigma, drag, p,
                         buoyancy_K):
    """Per-|k|^2-shell inverse of the eliminated w operator
    A' = alpha_w_eff I - (gamma dt)^2 c_k pinv_w G_Z q_solve G_Z S_w,
    q_boundary='none' (nhqg/grid.py:349-432)."""
    N = Nz
    ksq_rounded = np.round(ksq_flat, decimals=8)
    unique_ksq, inverse_idx = np.unique(ksq_rounded, return_inverse=True)
    Ng = N - 1
    inv = np.zeros((len(unique_ksq), Ng, Ng))
    I = np.eye(N + 1)
    GG = w_pinv @ G_Z
    for s, kv in enumerate(unique_ksq):
        kp = kv ** p
        alpha_q = 1.0 + gamma * dt * (nu_q * kp + drag)
        alpha_w = 1.0 + gamma * dt * nu_w * kp
        alpha_th = 1.0 + gamma * dt * (nu_theta / sigma) * kp
        alpha_w_eff = alpha_w - (gamma * dt) ** 2 * Ra_sigma / alpha_th
        q_solve = (1.0 / alpha_q) * I
        if buoyancy_K is None:
            couple = alpha_w_eff * np.eye(Ng)
        else:
            couple = alpha_w * np.eye(Ng) - (gamma * dt) ** 2 * (Ra_sigma / alpha_th) * buoyancy_K
        denom = kv + Ld_inv_sq
        if denom == 0.0:
            inv[s] = np.linalg.inv(couple)
        else:
            B = GG @ q_solve @ G_Z @ w_stencil
            inv[s] = np.linalg.inv(couple - (gamma * dt) ** 2 * (1.0 / denom) * B)
    return inv, inverse_idx.astype(np.int32)


@dataclasses.dataclass
class OracleGrid:
    cfg: OracleConfig
    Nx: int
    Nk: int
    Nz: int
    Npad: int
    Z: np.ndarray
    cc_weights: np.ndarray
    G_Z: np.ndarray
    G_Z2: np.ndarray
    V: np.ndarray
    V_inv: np.ndarray
    dirichlet_stencil: np.ndarray
    dirichlet_pinv: np.ndarray
    w_stencil: np.ndarray
    w_pinv: np.ndarray
    map_w_to_th: np.ndarray | None
    map_th_to_w: np.ndarray | None
    proj_dirichlet: np.ndarray
    proj_neumann: np.ndarray
    proj_w: np.ndarray
    sbp_D1: np.ndarray
    sbp_L: np.ndarray
    cgl_to_sbp: np.ndarray
    sbp_to_cgl: np.ndarray
    kx: np.ndarray
    ky: np.ndarray
    ksq: np.ndarray
    inv_denom: np.ndarray
    mask_23: np.ndarray
    eta_hat: np.ndarray | None
    sponge_phys: np.ndarray | None
    sponge_phys_pad: np.ndarray | None
    diss_rate_q: np.ndarray
    diss_rate_w: np.ndarray
    diss_rate_th: np.ndarray
    inv_alpha_q: np.ndarray
    inv_alpha_th: np.ndarray
    imex_inv: np.ndarray | None
    ksq_idx: np.ndarray
    beta: float
    Ra_sigma: float
    sigma: float
    dt: float
    gamma_imex: float
    imex_scheme: str
    mean_temp_eps_sq: float
    thermal_closure: str
    mean_exchange_discretization: str
    horizontal_dealiasing: str
    nonlinear_advection: str
    sbp_corrector_substeps: int

    def replace(self, **kw) -> "OracleGrid":
        return dataclasses.replace(self, **kw)


def make_grid(cfg: OracleConfig, with_shell_inverses: bool = True) -> OracleGrid:
    """Host precompute of every table the step reads (nhqg/grid.py:439-698).

    ``with_shell_inverses=False`` skips the per-shell A'^-1 table (the only
    table whose build is minutes at 256^2 x 256); ``imex_implicit_solve`` then
    builds just the shells it meets, lazily."""
    if cfg.q_boundary != "none":
        raise NotImplementedError("oracle covers q_boundary='none' (production)")
    if cfg.vertical_dealiasing != "none" or cfg.vertical_cutoff_n is not None:
        raise NotImplementedError("oracle covers vertical_dealiasing='none', no cutoff")
    Nx, Nz, L = cfg.Nx, cfg.Nz, cfg.L
    N, Nk = Nz, cfg.Nk
    dt = cfg.dt
    j = np.arange(N + 1, dtype=np.float64)
    xi = np.cos(np.pi * j / N)
    Z = 0.5 * (1.0 + xi)
    cc_w = cc_weights(N)
    G_Z = 2.0 * cheb_diff_matrix(N)
    G_Z2 = G_Z @ G_Z
    V, V_inv = cheb_vandermonde(N)

    S = np.zeros((N + 1, N - 1))
    for i in range(N - 1):
        S[i, i], S[i + 2, i] = -1.0, 1.0
    S_pinv = np.zeros((N - 1, N + 1))
    S_pinv[:, :N - 1] = np.linalg.inv(S[:N - 1, :])

    e_plus = np.ones(N + 1)
    e_minus = np.array([(-1.0) ** n for n in range(N + 1)])
    tau_dir = np.stack([e_plus, e_minus])
    tau_neu = np.stack([e_plus @ G_Z, e_minus @ G_Z])
    proj_dir = tau_projection(tau_dir, N)
    proj_neu = tau_projection(tau_neu, N)

    if cfg.w_bc_top == "dirichlet":
        w_stencil, w_pinv, proj_w = S, S_pinv, proj_dir
        map_w_to_th = map_th_to_w = buoyancy_K = None
    elif cfg.w_bc_top == "neumann":
        w_stencil = mixed_stencil(N)
        w_pinv = np.zeros((N - 1, N + 1))
        w_pinv[:, :N - 1] = np.linalg.inv(w_stencil[:N - 1, :])
        proj_w = tau_projection(np.stack([tau_neu[0], tau_dir[1]]), N)
        map_w_to_th = S_pinv @ w_stencil
        map_th_to_w = w_pinv @ S
        buoyancy_K = map_th_to_w @ map_w_to_th
    else:
        raise ValueError(f"Unsupported w_bc_top={cfg.w_bc_top!r}")

    Z_sbp = np.linspace(0.0, 1.0, N + 1)
    H, D1, Lap = sbp2_operators(N)
    c2s_lin = piecewise_linear_interp(Z, Z_sbp)
    M_cc = np.diag(cc_w)
    if cfg.sbp_transfer_mode == "interp":
        c2s, s2c = c2s_lin, piecewise_linear_interp(Z_sbp, Z)
    elif cfg.sbp_transfer_mode == "mass_adjoint":
        c2s = c2s_lin
        s2c = np.linalg.solve(M_cc, c2s.T @ H)
    elif cfg.sbp_transfer_mode == "weighted_polar":
        h = np.diag(H)
        A_t = np.diag(np.sqrt(h)) @ c2s_lin @ np.diag(1.0 / np.sqrt(cc_w))
        U, _, Vt = np.linalg.svd(A_t, full_matrices=False)
        c2s = np.diag(1.0 / np.sqrt(h)) @ (U @ Vt) @ np.diag(np.sqrt(cc_w))
        s2c = np.linalg.solve(M_cc, c2s.T @ H)
    else:
        raise ValueError(f"Unsupported sbp_transfer_mode={cfg.sbp_transfer_mode!r}")

    # horizontal wavenumbers, evaluated in the reference's operation order
    kx1 = 2.0 * np.pi * np.fft.fftfreq(Nx, d=L / Nx)
    ky1 = 2.0 * np.pi * np.arange(Nk) / L
    kx, ky = kx1[:, None], ky1[None, :]
    ksq = kx ** 2 + ky ** 2
    denom = ksq + cfg.Ld_inv_sq
    inv_denom = np.zeros_like(denom)
    np.divide(1.0, denom, out=inv_denom, where=denom > 0)

    K = Nx // 3
    ii = np.arange(Nx)
    kx_int = np.where(ii <= Nx // 2, ii, ii - Nx)
    mask = ((np.abs(kx_int)[:, None] <= K) & (np.arange(Nk)[None, :] <= K)).astype(np.float64)

    if cfg.gamma != 0.0 and cfg.beta != 0.0:
        raise ValueError("gamma (polar trap) and beta (flat beta-plane) are mutually exclusive")
    eta_hat = None
    r_star = None
    xy = np.arange(Nx) * (L / Nx)
    X, Y = np.meshgrid(xy, xy, indexing="ij")
    r = np.sqrt((X - L / 2.0) ** 2 + (Y - L / 2.0) ** 2)
    if cfg.gamma != 0.0:
        r_star = cfg.trap_r_star if cfg.trap_r_star is not None else 0.45 * (L / 2.0)
        sig_trap = 0.5 * (1.0 - np.tanh(cfg.trap_sharpness * (r - r_star) / r_star))
        eta_hat = np.fft.rfft2(-0.5 * cfg.gamma * r ** 2 * sig_trap)
        e_tot = np.sum(np.abs(eta_hat) ** 2)
        e_out = np.sum(np.abs(eta_hat * (1.0 - mask)) ** 2)
        if e_out > 1e-10 * e_tot:  # nhqg/grid.py:622-629
            raise ValueError(f"Trap background PV is under-resolved: {e_out / e_tot:.2e}")
        if cfg.horizontal_dealiasing == "23_rule":
            eta_hat = eta_hat * mask
    sponge_phys = sponge_phys_pad = None
    if cfg.sponge_rate < 0.0:
        raise ValueError("sponge_rate must be >= 0")
    if cfg.sponge_rate > 0.0:
        if cfg.sponge_r_start is not None:
            r_s = cfg.sponge_r_start
        elif cfg.gamma != 0.0:
            r_s = 1.18 * r_star
        else:
            raise ValueError("sponge_r_start is required when gamma == 0")
        sig = cfg.sponge_rate * 0.5 * (1.0 + np.tanh(cfg.sponge_sharpness * (r - r_s) / r_s))
        sig_hat = np.fft.rfft2(sig)
        s_tot = np.sum(np.abs(sig_hat) ** 2)
        s_out = np.sum(np.abs(sig_hat * (1.0 - mask)) ** 2)
        if s_out > 1e-10 * s_tot:  # nhqg/grid.py:652-659
            raise ValueError(f"Sponge profile is under-resolved: {s_out / s_tot:.2e}")
        if cfg.horizontal_dealiasing == "23_rule":
            sig_hat = sig_hat * mask
        sponge_phys = np.fft.irfft2(sig_hat, s=(Nx, Nx))
        # the padded-grid sigma of the 3/2 rule, without the (Npad/Nx)^2
        # rescale (nhqg/grid.py:663-667)
        sponge_phys_pad = np.fft.irfft2(_zero_pad(sig_hat, Nx, cfg.Npad), s=(cfg.Npad, cfg.Npad))

    if cfg.imex_scheme == "ars222":  # nhqg/grid.py:671-676
        gamma_imex = 1.0 - 1.0 / np.sqrt(2.0)
    elif cfg.imex_scheme == "rk443":
        gamma_imex = 0.5
    else:
        raise NotImplementedError(f"oracle covers imex_scheme 'ars222' and 'rk443', not {cfg.imex_scheme!r}")
    p = cfg.hyper_order
    drq = cfg.nu_q * ksq ** p + cfg.drag
    drw = cfg.nu_w * ksq ** p
    drt = (cfg.nu_theta / cfg.sigma) * ksq ** p
    inv_aq = 1.0 / (1.0 + gamma_imex * dt * drq)
    inv_at = 1.0 / (1.0 + gamma_imex * dt * drt)

    ksq_rounded = np.round(ksq.ravel(), decimals=8)
    _, inv_idx = np.unique(ksq_rounded, return_inverse=True)
    imex_inv = None
    if with_shell_inverses:
        imex_inv, inv_idx = build_shell_inverses(
            G_Z, w_stencil, w_pinv, ksq.ravel(), cfg.Ld_inv_sq, dt, gamma_imex, Nz,
            cfg.nu_q, cfg.nu_w, cfg.nu_theta, cfg.sigma, cfg.Ra_tilde / cfg.sigma,
            cfg.drag, p, buoyancy_K)

    return OracleGrid(
        cfg=cfg, Nx=Nx, Nk=Nk, Nz=Nz, Npad=cfg.Npad, Z=Z, cc_weights=cc_w,
        G_Z=G_Z, G_Z2=G_Z2, V=V, V_inv=V_inv, dirichlet_stencil=S,
        dirichlet_pinv=S_pinv, w_stencil=w_stencil, w_pinv=w_pinv,
        map_w_to_th=map_w_to_th, map_th_to_w=map_th_to_w, proj_dirichlet=proj_dir,
        proj_neumann=proj_neu, proj_w=proj_w, sbp_D1=D1, sbp_L=Lap,
        cgl_to_sbp=c2s, sbp_to_cgl=s2c, kx=kx, ky=ky, ksq=ksq, inv_denom=inv_denom,
        mask_23=mask, eta_hat=eta_hat, sponge_phys=sponge_phys, sponge_phys_pad=sponge_phys_pad,
        diss_rate_q=drq, diss_rate_w=drw, diss_rate_th=drt, inv_alpha_q=inv_aq,
        inv_alpha_th=inv_at, imex_inv=imex_inv,
        ksq_idx=np.asarray(inv_idx, dtype=np.int32).reshape(Nx, Nk),
        beta=cfg.beta, Ra_sigma=cfg.Ra_tilde / cfg.sigma, sigma=cfg.sigma, dt=dt,
        gamma_imex=gamma_imex, imex_scheme=cfg.imex_scheme, mean_temp_eps_sq=cfg.mean_temp_eps_sq,
        thermal_closure=cfg.thermal_closure,
        mean_exchange_discretization=cfg.mean_exchange_discretization,
        horizontal_dealiasing=cfg.horizontal_dealiasing,
        nonlinear_advection=cfg.nonlinear_advection,
        sbp_corrector_substeps=cfg.sbp_corrector_substeps,
    )


# ---------------------------------------------------------------------------
# Helpers -- nhqg/solver.py:45-160
# ---------------------------------------------------------------------------

def vmat(mat: np.ndarray, field: np.ndarray) -> np.ndarray:
    """einsum('ij,j...->i...') as one real GEMM over the flattened columns
    (nhqg/solver.py:45-82)."""
    f = np.ascontiguousarray(field)
    cols = f.reshape(f.shape[0], -1)
    if np.iscomplexobj(cols):
        re = cols.view(np.float64)  # interleaved real/imag columns
        out = (mat @ re).view(np.complex128)
    else:
        out = mat @ cols
    return out.reshape((mat.shape[0],) + f.shape[1:])


def _irfft2(a: np.ndarray, N: int) -> np.ndarray:
    return sfft.irfft2(a, s=(N, N), workers=_WORKERS)


def _rfft2(a: np.ndarray) -> np.ndarray:
    return sfft.rfft2(a, workers=_WORKERS)


def invert_psi(q_hat, inv_denom):
    """nhqg/solver.py:89-91."""
    return -q_hat * inv_denom[None]


def zero_mean(f):
    """nhqg/solver.py:98-100."""
    f = f.copy()
    f[:, 0, 0] = 0.0
    return f


def hermitian_project(f, Nx):
    """Hermitian part of the ky=0 (and Nyquist) columns (nhqg/solver.py:107-125)."""
    neg = (-np.arange(Nx)) % Nx
    f = f.copy()
    col = f[:, :, 0]
    f[:, :, 0] = 0.5 * (col + np.conj(col[:, neg]))
    if Nx % 2 == 0:
        col = f[:, :, -1]
        f[:, :, -1] = 0.5 * (col + np.conj(col[:, neg]))
    return f


def sanitize_state(state: OracleState, grid: OracleGrid) -> OracleState:
    """nhqg/solver.py:128-146."""
    q = hermitian_project(state.q_hat, grid.Nx)
    w = hermitian_project(state.w_hat, grid.Nx)
    th = hermitian_project(state.th_hat, grid.Nx)
    if grid.horizontal_dealiasing == "23_rule":
        m = grid.mask_23[None]
        q, w, th = q * m, w * m, th * m
    return OracleState(q, w, th, state.th_bar)


# ---------------------------------------------------------------------------
# Horizontal products under the 2/3 rule -- nhqg/spectral.py:53-60, 281-358
# ---------------------------------------------------------------------------

# Test hook, None in every parity check: a function applied to the
# physical-space factors of the 2/3-rule products before they are multiplied.
# A test sets it (e.g. to a BF16 rounding) to show that a precision gate on
# the mixed path would catch products computed at a lower precision.
PRODUCT_ROUNDING = None


def _factor(a):
    return a if PRODUCT_ROUNDING is None else PRODUCT_ROUNDING(a)


def triple_conservative_flux_divergence_23(psi, q, w, th, kx, ky, mask, Nx):
    """div(u f, v f), u=-psi_y, v=psi_x, for f in (q, w, th), every level
    (nhqg/spectral.py:307-328, 346-358)."""
    kx3, ky3 = kx[None], ky[None]
    u = _factor(_irfft2(-1j * ky3 * psi, Nx))
    v = _factor(_irfft2(1j * kx3 * psi, Nx))
    outs = []
    for f_hat in (q, w, th):
        f = _factor(_irfft2(f_hat, Nx))
        div = 1j * kx3 * _rfft2(u * f) + 1j * ky3 * _rfft2(v * f)
        outs.append(div * mask[None])
    return tuple(outs)


def triple_jacobian_23(psi, q, w, th, kx, ky, mask, Nx):
    """J[psi, f] = psi_x f_y - psi_y f_x (nhqg/spectral.py:281-304, 331-343)."""
    kx3, ky3 = kx[None], ky[None]
    psi_x = _irfft2(1j * kx3 * psi, Nx)
    psi_y = _irfft2(1j * ky3 * psi, Nx)
    outs = []
    for f_hat in (q, w, th):
        fx = _irfft2(1j * kx3 * f_hat, Nx)
        fy = _irfft2(1j * ky3 * f_hat, Nx)
        outs.append(_rfft2(psi_x * fy - psi_y * fx) * mask[None])
    return tuple(outs)


def sponge_product_23(f_hat, sponge_phys, mask, Nx):
    """mask * rfft2(sigma * irfft2(f)) per level (nhqg/spectral.py:53-60)."""
    return _rfft2(sponge_phys[None] * _irfft2(f_hat, Nx)) * mask[None]


def _zero_pad(f_hat, Nx, Npad):
    """Batched 3/2-rule zero pad (nhqg/spectral.py:18-34)."""
    Nk, Nkp = Nx // 2 + 1, Npad // 2 + 1
    out = np.zeros(f_hat.shape[:-2] + (Npad, Nkp), dtype=np.complex128)
    out[..., :Nx // 2, :Nk] = f_hat[..., :Nx // 2, :]
    out[..., Npad - Nx // 2:, :Nk] = f_hat[..., Nx // 2:, :]
    return out


def _truncate(f_pad, Nx, Npad):
    """Keep the Nx-grid modes of a padded spectrum and rescale by (Npad/Nx)^2
    (nhqg/spectral.py:37-50)."""
    out = np.concatenate([f_pad[..., :Nx // 2, :Nx // 2 + 1], f_pad[..., Npad - Nx // 2:, :Nx // 2 + 1]],
                         axis=-2)
    return out * (Npad / Nx) ** 2


def _pad_wavenumbers(ky, Npad):
    """kx, ky of the padded grid from the base grid's ky spacing
    (nhqg/spectral.py:79-87)."""
    k0 = ky[0, 1] if ky.shape[1] >= 2 else 0.0
    kxp = k0 * np.fft.fftfreq(Npad, d=1.0 / Npad)
    kyp = k0 * np.arange(Npad // 2 + 1)
    return kxp[:, None], kyp[None, :]


def _pad_irfft2(f_hat, Nx, Npad):
    return _irfft2(_zero_pad(f_hat, Nx, Npad), Npad)


def triple_conservative_flux_divergence_32(psi, q, w, th, kx, ky, Nx, Npad):
    """div(u f, v f) under the 3/2 rule: zero-pad, products on the Npad grid,
    padded-grid derivatives, truncate (nhqg/spectral.py:190-216, 237-253)."""
    kx3, ky3 = kx[None], ky[None]
    u = _pad_irfft2(-1j * ky3 * psi, Nx, Npad)
    v = _pad_irfft2(1j * kx3 * psi, Nx, Npad)
    kxp, kyp = _pad_wavenumbers(ky, Npad)
    outs = []
    for f_hat in (q, w, th):
        f = _pad_irfft2(f_hat, Nx, Npad)
        div = 1j * kxp[None] * _rfft2(u * f) + 1j * kyp[None] * _rfft2(v * f)
        outs.append(_truncate(div, Nx, Npad))
    return tuple(outs)


def triple_jacobian_32(psi, q, w, th, kx, ky, Nx, Npad):
    """J[psi, f] under the 3/2 rule (nhqg/spectral.py:147-180, 219-234)."""
    kx3, ky3 = kx[None], ky[None]
    psi_x = _pad_irfft2(1j * kx3 * psi, Nx, Npad)
    psi_y = _pad_irfft2(1j * ky3 * psi, Nx, Npad)
    outs = []
    for f_hat in (q, w, th):
        fx = _pad_irfft2(1j * kx3 * f_hat, Nx, Npad)
        fy = _pad_irfft2(1j * ky3 * f_hat, Nx, Npad)
        outs.append(_truncate(_rfft2(psi_x * fy - psi_y * fx), Nx, Npad))
    return tuple(outs)


def sponge_product_32(f_hat, sponge_phys_pad, Nx, Npad):
    """sigma * f under the 3/2 rule with the pre-attenuated padded sigma
    (nhqg/spectral.py:63-75)."""
    return _truncate(_rfft2(sponge_phys_pad[None] * _pad_irfft2(f_hat, Nx, Npad)), Nx, Npad)


def _mean_npad(grid):
    """Grid of the SBP2 corrector's horizontal means: Nx under the 2/3 rule,
    the padded grid under the 3/2 rule (nhqg/solver.py:836, 931)."""
    return None if grid.horizontal_dealiasing == "23_rule" else grid.Npad


def horizontal_mean(a_nodal, b_nodal, Nx, Npad=None):
    """<a b>_xy per level from spectral fields (nhqg/solver.py:204-245)."""
    if Npad is None or Npad == Nx:
        a, b = _irfft2(a_nodal, Nx), _irfft2(b_nodal, Nx)
    else:
        scale = (Npad / Nx) ** 2
        a = scale * _irfft2(_zero_pad(a_nodal, Nx, Npad), Npad)
        b = scale * _irfft2(_zero_pad(b_nodal, Nx, Npad), Npad)
    return np.mean(a * b, axis=(1, 2))


# ---------------------------------------------------------------------------
# Explicit RHS -- nhqg/solver.py:510-608
# ---------------------------------------------------------------------------

def _uses_split(grid):
    """nhqg/solver.py:310-316 (the midpoint/coral branches are not covered)."""
    m = grid.mean_exchange_discretization
    if m in ("balanced_sbp2", "balanced_sbp2_pc"):
        return True
    if m == "legacy":
        return False
    raise NotImplementedError(f"oracle does not cover mean_exchange_discretization={m!r}")


def explicit_rhs(state: OracleState, grid: OracleGrid) -> OracleState:
    """nhqg/solver.py:510-599."""
    q_hat, w_hat, th_hat, th_bar = state
    psi_hat = invert_psi(q_hat, grid.inv_denom)
    w_cheb = vmat(grid.w_stencil, w_hat)
    th_cheb = vmat(grid.dirichlet_stencil, th_hat)
    psi_n = vmat(grid.V, psi_hat)
    q_n = vmat(grid.V, q_hat)
    w_n = vmat(grid.V, w_cheb)
    th_n = vmat(grid.V, th_cheb)
    if grid.eta_hat is not None:  # nhqg/solver.py:534-535
        q_n = q_n + grid.eta_hat[None]
    # nhqg/solver.py:389-418
    if grid.nonlinear_advection not in ("flux", "jacobian"):
        raise ValueError(f"Unsupported nonlinear_advection={grid.nonlinear_advection!r}")
    if grid.horizontal_dealiasing == "23_rule":
        prod = (triple_conservative_flux_divergence_23 if grid.nonlinear_advection == "flux"
                else triple_jacobian_23)
        Aq_n, Aw_n, Ath_n = prod(psi_n, q_n, w_n, th_n, grid.kx, grid.ky, grid.mask_23, grid.Nx)
    elif grid.horizontal_dealiasing == "32_rule":
        prod = (triple_conservative_flux_divergence_32 if grid.nonlinear_advection == "flux"
                else triple_jacobian_32)
        Aq_n, Aw_n, Ath_n = prod(psi_n, q_n, w_n, th_n, grid.kx, grid.ky, grid.Nx, grid.Npad)
    else:
        raise ValueError(f"Unsupported horizontal_dealiasing={grid.horizontal_dealiasing!r}")
    Aq = vmat(grid.V_inv, Aq_n)
    Aw = vmat(grid.V_inv, Aw_n)
    Ath = vmat(grid.V_inv, Ath_n)
    E_q = -Aq - 1j * grid.beta * grid.kx[None] * psi_hat
    E_w = vmat(grid.w_pinv, vmat(grid.proj_w, -Aw))
    if grid.thermal_closure == "evolve_mean" and not _uses_split(grid):
        # legacy explicit exchange (nhqg/solver.py:571-586)
        dtb = grid.G_Z @ th_bar
        dtb_n = grid.V @ dtb
        prod = vmat(grid.V_inv, dtb_n[:, None, None] * w_n)
        E_th = vmat(grid.dirichlet_pinv, vmat(grid.proj_dirichlet, -Ath - prod))
        w_nod = vmat(grid.V, vmat(grid.w_stencil, w_hat))
        th_nod = vmat(grid.V, vmat(grid.dirichlet_stencil, th_hat))
        flux = horizontal_mean(w_nod, th_nod, grid.Nx, grid.Npad)
        E_th_bar = grid.mean_temp_eps_sq * (-grid.G_Z @ (grid.V_inv @ flux))
    else:
        E_th = vmat(grid.dirichlet_pinv, vmat(grid.proj_dirichlet, -Ath))
        E_th_bar = np.zeros_like(th_bar)
    if grid.sponge_phys is not None:  # nhqg/solver.py:421-424, 591-597
        if grid.horizontal_dealiasing == "23_rule":
            sp = lambda f: sponge_product_23(f, grid.sponge_phys, grid.mask_23, grid.Nx)  # noqa: E731
        else:
            sp = lambda f: sponge_product_32(f, grid.sponge_phys_pad, grid.Nx, grid.Npad)  # noqa: E731
        E_q = E_q - sp(q_hat)
        E_w = E_w - sp(w_hat)
        E_th = E_th - sp(th_hat)
    return OracleState(E_q, E_w, E_th, E_th_bar)


def explicit_rhs_dispatch(state, grid):
    """nhqg/solver.py:602-608 (vertical_dealiasing='none')."""
    return explicit_rhs(state, grid)


# ---------------------------------------------------------------------------
# Implicit tendency and solve -- nhqg/solver.py:615-758
# ---------------------------------------------------------------------------

def implicit_tendency(state: OracleState, grid: OracleGrid) -> OracleState:
    """nhqg/solver.py:615-641."""
    q_hat, w_hat, th_hat, th_bar = state
    w_cheb = vmat(grid.w_stencil, w_hat)
    th_cheb = vmat(grid.dirichlet_stencil, th_hat)
    dw = vmat(grid.G_Z, w_cheb)
    dq = vmat(grid.G_Z, q_hat)
    Iw_cheb = grid.inv_denom[None] * dq + grid.Ra_sigma * th_cheb
    I_w = vmat(grid.w_pinv, vmat(grid.proj_w, Iw_cheb))
    I_th = w_hat if grid.map_w_to_th is None else vmat(grid.map_w_to_th, w_hat)
    if grid.thermal_closure == "evolve_mean":
        I_tb = (grid.mean_temp_eps_sq / grid.sigma) * (grid.G_Z2 @ th_bar)
    else:
        I_tb = np.zeros_like(th_bar)
    return OracleState(dw, I_w, I_th, I_tb)


def _shell_inverse_lookup(grid: OracleGrid, shells: np.ndarray) -> np.ndarray:
    """A'^-1 for the given shell ids (built lazily when the grid was made
    without the table)."""
    if grid.imex_inv is not None:
        return grid.imex_inv[shells]
    cache = grid.__dict__.setdefault("_shell_cache", {})
    missing = [int(s) for s in np.unique(shells) if int(s) not in cache]
    if missing:
        c = grid.cfg
        uniq = np.unique(np.round(grid.ksq.ravel(), decimals=8))
        bK = None if grid.map_th_to_w is None else grid.map_th_to_w @ grid.map_w_to_th
        inv, _ = build_shell_inverses(
            grid.G_Z, grid.w_stencil, grid.w_pinv, uniq[missing], c.Ld_inv_sq, grid.dt,
            grid.gamma_imex, grid.Nz, c.nu_q, c.nu_w, c.nu_theta, c.sigma,
            grid.Ra_sigma, c.drag, c.hyper_order, bK)
        for s, m in zip(missing, inv):
            cache[s] = m
    flat = np.asarray(shells).ravel()
    out = np.stack([cache[int(s)] for s in flat])
    return out.reshape(np.shape(shells) + out.shape[1:])


def _shell_groups(grid: OracleGrid):
    """Modes grouped by shell: (shell ids, start offsets, flat mode order)."""
    g = grid.__dict__.get("_shell_groups")
    if g is None:
        idx = grid.ksq_idx.ravel()
        order = np.argsort(idx, kind="stable")
        shells, starts = np.unique(idx[order], return_index=True)
        g = (shells, np.append(starts, idx.size), order)
        grid.__dict__["_shell_groups"] = g
    return g


def per_shell_matmul(grid: OracleGrid, field: np.ndarray) -> np.ndarray:
    """Apply A'^-1[shell(k)] to each mode's column (nhqg/solver.py:648-675).
    Modes of one shell share the matrix, so each shell is one small GEMM
    instead of the reference's gathered (Nx, Nk, m, m) batch; the products
    are the same per mode."""
    m = field.shape[0]
    cols = np.ascontiguousarray(np.transpose(field, (1, 2, 0))).reshape(-1, m)
    out = np.empty_like(cols)
    shells, starts, order = _shell_groups(grid)
    if grid.imex_inv is None:
        _shell_inverse_lookup(grid, shells[:1])  # warm the lazy cache ...
        cache = grid.__dict__["_shell_cache"]
        if len(cache) < len(shells):             # ... for every shell at once
            _shell_inverse_lookup(grid, shells)
        table = [cache[int(s)] for s in shells]
    else:
        table = [grid.imex_inv[s] for s in shells]
    for i, A in enumerate(table):
        modes = order[starts[i]:starts[i + 1]]
        out[modes] = cols[modes] @ A.T
    return np.transpose(out.reshape(field.shape[1], field.shape[2], m), (2, 0, 1))


def imex_implicit_solve(R_q, R_w, R_th, grid: OracleGrid):
    """Block elimination at each k (nhqg/solver.py:691-738), q_boundary='none'."""
    gdt = grid.gamma_imex * grid.dt
    rth = R_th * grid.inv_alpha_th[None]
    if grid.map_th_to_w is not None:
        rth = vmat(grid.map_th_to_w, rth)
    R_w_eff = R_w + gdt * grid.Ra_sigma * rth
    temp = R_q * grid.inv_alpha_q[None]
    d_temp = vmat(grid.G_Z, temp)
    d_gal = vmat(grid.w_pinv, vmat(grid.proj_w, grid.inv_denom[None] * d_temp))
    rhs_w = R_w_eff + gdt * d_gal
    w_new = per_shell_matmul(grid, rhs_w)
    dw = vmat(grid.G_Z, vmat(grid.w_stencil, w_new))
    q_new = (R_q + gdt * dw) * grid.inv_alpha_q[None]
    w_th = w_new if grid.map_w_to_th is None else vmat(grid.map_w_to_th, w_new)
    th_new = (R_th + gdt * w_th) * grid.inv_alpha_th[None]
    return q_new, w_new, th_new


def imex_mean_temp_solve(R_th_bar, grid: OracleGrid):
    """nhqg/solver.py:741-758."""
    if grid.thermal_closure != "evolve_mean":
        return grid.proj_dirichlet @ R_th_bar
    N = grid.Nz
    alpha = grid.gamma_imex * grid.dt * grid.mean_temp_eps_sq / grid.sigma
    A = np.eye(N + 1) - alpha * grid.G_Z2
    A[N - 1, :] = 1.0
    A[N, :] = [(-1.0) ** n for n in range(N + 1)]
    rhs = R_th_bar.copy()
    rhs[N - 1] = rhs[N] = 0.0
    return np.linalg.solve(A, rhs)


# ---------------------------------------------------------------------------
# SBP2 thermal corrector -- nhqg/solver.py:346-358, 873-962
# ---------------------------------------------------------------------------

def apply_balanced_sbp2_corrector(state: OracleState, grid: OracleGrid, total_dt) -> OracleState:
    """Hoisted-invariant SBP2 corrector with ``sbp_corrector_substeps`` midpoint
    substeps (nhqg/solver.py:909-950 and substep :873-906)."""
    if grid.thermal_closure != "evolve_mean":
        return state
    n_sub = max(1, int(grid.sbp_corrector_substeps))
    sub_dt = float(total_dt) / n_sub
    mu = grid.mean_temp_eps_sq
    kappa = 1.0 / grid.sigma
    D1, Lap = grid.sbp_D1, grid.sbp_L
    c2s, s2c = grid.cgl_to_sbp, grid.sbp_to_cgl
    w_sbp = vmat(c2s, vmat(grid.V, vmat(grid.w_stencil, state.w_hat)))
    w2 = horizontal_mean(w_sbp, w_sbp, grid.Nx, _mean_npad(grid))
    I = np.eye(grid.Nz + 1)
    half = 0.5 * mu * kappa * sub_dt * Lap + 0.25 * mu * sub_dt ** 2 * (D1 @ np.diag(w2) @ D1)
    A = I - half
    B = I + half
    A[0, :] = 0.0
    A[-1, :] = 0.0
    A[0, 0] = A[-1, -1] = 1.0
    lu = sla.lu_factor(A)
    q_hat, w_hat, th_hat, th_bar = state
    for _ in range(n_sub):
        th_sbp = vmat(c2s, vmat(grid.V, vmat(grid.dirichlet_stencil, th_hat)))
        tb_sbp = c2s @ (grid.V @ th_bar)
        flux = horizontal_mean(w_sbp, th_sbp, grid.Nx, _mean_npad(grid))
        rhs = B @ tb_sbp - mu * sub_dt * (D1 @ flux)
        rhs[0] = rhs[-1] = 0.0
        tb_new = sla.lu_solve(lu, rhs)
        g_half = 0.5 * (D1 @ (tb_sbp + tb_new))
        th_new = th_sbp - sub_dt * w_sbp * g_half[:, None, None]
        th_new[0] = 0.0
        th_new[-1] = 0.0
        tb_new[0] = tb_new[-1] = 0.0
        th_cheb = vmat(grid.proj_dirichlet, vmat(grid.V_inv, vmat(s2c, th_new)))
        th_hat = vmat(grid.dirichlet_pinv, th_cheb)
        th_bar = grid.proj_dirichlet @ (grid.V_inv @ (s2c @ tb_new))
    return OracleState(q_hat, w_hat, th_hat, th_bar)


# ---------------------------------------------------------------------------
# Steppers -- nhqg/solver.py:993-1053, 1149-1242
# ---------------------------------------------------------------------------

def _finalize(state: OracleState) -> OracleState:
    """nhqg/solver.py:993-999 (no vertical cutoff)."""
    return OracleState(zero_mean(state.q_hat), zero_mean(state.w_hat),
                       zero_mean(state.th_hat), state.th_bar)


def _base_grid(grid: OracleGrid) -> OracleGrid:
    return grid.replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")


def imex_step_ars222(state: OracleState, grid: OracleGrid) -> OracleState:
    """nhqg/solver.py:1012-1053."""
    g = grid.gamma_imex
    delta = -np.sqrt(2.0) / 2.0
    dt = grid.dt
    q_n, w_n, th_n, tb_n = state
    E1 = explicit_rhs_dispatch(state, grid)
    q1, w1, th1 = imex_implicit_solve(q_n + g * dt * E1.q_hat, w_n + g * dt * E1.w_hat,
                                      th_n + g * dt * E1.th_hat, grid)
    tb1 = imex_mean_temp_solve(tb_n + g * dt * E1.th_bar, grid)
    s1 = OracleState(q1, w1, th1, tb1)
    E2 = explicit_rhs_dispatch(s1, grid)
    I1 = implicit_tendency(s1, grid)
    omg = dt * (1 - g)
    R_q = q_n + dt * (delta * E1.q_hat + (1 - delta) * E2.q_hat) + omg * I1.q_hat \
        - omg * grid.diss_rate_q[None] * q1
    R_w = w_n + dt * (delta * E1.w_hat + (1 - delta) * E2.w_hat) + omg * I1.w_hat \
        - omg * grid.diss_rate_w[None] * w1
    R_th = th_n + dt * (delta * E1.th_hat + (1 - delta) * E2.th_hat) + omg * I1.th_hat \
        - omg * grid.diss_rate_th[None] * th1
    R_tb = tb_n + dt * (delta * E1.th_bar + (1 - delta) * E2.th_bar) + omg * I1.th_bar
    q2, w2, th2 = imex_implicit_solve(R_q, R_w, R_th, grid)
    tb2 = imex_mean_temp_solve(R_tb, grid)
    return _finalize(OracleState(q2, w2, th2, tb2))


def _implicit_with_diss(state: OracleState, impl: OracleState, grid: OracleGrid) -> OracleState:
    """Implicit derivative including horizontal dissipation (nhqg/solver.py:1002-1009)."""
    return OracleState(impl.q_hat - grid.diss_rate_q[None] * state.q_hat,
                       impl.w_hat - grid.diss_rate_w[None] * state.w_hat,
                       impl.th_hat - grid.diss_rate_th[None] * state.th_hat, impl.th_bar)


# ARS(4,4,3) tableau rows as (coefficient, K_j or E_j) pairs, K_j the implicit
# derivative at stage j (1-based), E_j the explicit one at stage j (0 = y_n)
RK443_ROWS = (
    ((0.5, "E0"),),
    ((1.0 / 6.0, "K1"), (11.0 / 18.0, "E0"), (1.0 / 18.0, "E1")),
    ((-0.5, "K1"), (0.5, "K2"), (5.0 / 6.0, "E0"), (-5.0 / 6.0, "E1"), (0.5, "E2")),
    ((1.5, "K1"), (-1.5, "K2"), (0.5, "K3"), (0.25, "E0"), (1.75, "E1"), (0.75, "E2"), (-1.75, "E3")),
)
RK443_FINAL = ((1.5, "K1"), (-1.5, "K2"), (0.5, "K3"), (0.5, "K4"), (0.25, "E0"), (1.75, "E1"),
               (0.75, "E2"), (-1.75, "E3"))


def imex_step_rk443(state: OracleState, grid: OracleGrid) -> OracleState:
    """ARS(4,4,3) IMEX-RK step, gamma = 1/2 in every implicit stage
    (nhqg/solver.py:1056-1122): y0 + dt * sum(c X) per row, left to right."""
    dt = grid.dt
    d = {"E0": explicit_rhs_dispatch(state, grid)}

    def comb(row):
        return OracleState(*(state[f] + dt * sum(c * d[name][f] for c, name in row) for f in range(4)))

    for i, row in enumerate(RK443_ROWS, start=1):
        rhs = comb(row)
        q, w, th = imex_implicit_solve(rhs.q_hat, rhs.w_hat, rhs.th_hat, grid)
        Y = OracleState(q, w, th, imex_mean_temp_solve(rhs.th_bar, grid))
        d[f"K{i}"] = _implicit_with_diss(Y, implicit_tendency(Y, grid), grid)
        if i < 4:
            d[f"E{i}"] = explicit_rhs_dispatch(Y, grid)
    return _finalize(comb(RK443_FINAL))


def imex_step_balanced_sbp2_pc(state: OracleState, grid: OracleGrid) -> OracleState:
    """Stage-wise predictor/corrector (nhqg/solver.py:1167-1225)."""
    base = _base_grid(grid)
    g = grid.gamma_imex
    delta = -np.sqrt(2.0) / 2.0
    dt = grid.dt
    alpha = g * dt
    omg = dt * (1 - g)
    q_n, w_n, th_n, tb_n = state
    E1 = explicit_rhs_dispatch(state, base)
    q1p, w1p, th1p = imex_implicit_solve(q_n + alpha * E1.q_hat, w_n + alpha * E1.w_hat,
                                         th_n + alpha * E1.th_hat, base)
    tb1p = imex_mean_temp_solve(tb_n + alpha * E1.th_bar, base)
    pred1 = OracleState(q1p, w1p, th1p, tb1p)
    s1 = apply_balanced_sbp2_corrector(pred1, grid, alpha)
    C_th = (s1.th_hat - pred1.th_hat) / alpha
    C_tb = (s1.th_bar - pred1.th_bar) / alpha
    E2 = explicit_rhs_dispatch(s1, base)
    I1 = implicit_tendency(s1, base)
    R_q = q_n + dt * (delta * E1.q_hat + (1 - delta) * E2.q_hat) + omg * I1.q_hat \
        - omg * grid.diss_rate_q[None] * s1.q_hat
    R_w = w_n + dt * (delta * E1.w_hat + (1 - delta) * E2.w_hat) + omg * I1.w_hat \
        - omg * grid.diss_rate_w[None] * s1.w_hat
    R_th = th_n + dt * (delta * E1.th_hat + (1 - delta) * E2.th_hat) + omg * I1.th_hat \
        - omg * grid.diss_rate_th[None] * s1.th_hat + omg * C_th
    R_tb = tb_n + dt * (delta * E1.th_bar + (1 - delta) * E2.th_bar) + omg * I1.th_bar \
        + omg * C_tb
    q2, w2, th2 = imex_implicit_solve(R_q, R_w, R_th, base)
    tb2 = imex_mean_temp_solve(R_tb, base)
    out = apply_balanced_sbp2_corrector(OracleState(q2, w2, th2, tb2), grid, alpha)
    return _finalize(out)


def imex_step(state: OracleState, grid: OracleGrid) -> OracleState:
    """Dispatch (nhqg/solver.py:1228-1242) + sanitize."""
    m = grid.mean_exchange_discretization
    if m == "balanced_sbp2_pc":
        new = imex_step_balanced_sbp2_pc(state, grid)
    elif m == "balanced_sbp2":  # nhqg/solver.py:1149-1164
        new = _finalize(apply_balanced_sbp2_corrector(
            imex_step_ars222(state, _base_grid(grid)), grid, grid.dt))
    elif m == "legacy":
        new = imex_step_rk443(state, grid) if grid.imex_scheme == "rk443" else imex_step_ars222(state, grid)
    else:
        raise NotImplementedError(f"oracle does not cover {m!r}")
    return sanitize_state(new, grid)


# ---------------------------------------------------------------------------
# Seeded theta' initial state (the benchmark configurations' start)
# ---------------------------------------------------------------------------

def theta_perturbation_state(grid: OracleGrid, seed: int = 0, amplitude: float = 1e-3) -> OracleState:
    """theta' = amplitude * N(0,1) * sin(pi Z) at the CGL nodes (PCG64
    ``default_rng(seed)``, shape (Nz+1, Nx, Nx)); rfft2 per level -> V^-1 ->
    Dirichlet pinv; q' = w = 0, Theta_bar = 0; then ``sanitize_state``."""
    P, Nx = grid.Nz + 1, grid.Nx
    rng = np.random.default_rng(seed)
    th = amplitude * rng.standard_normal((P, Nx, Nx)) * np.sin(np.pi * grid.Z)[:, None, None]
    th_gal = vmat(grid.dirichlet_pinv, vmat(grid.V_inv, np.fft.rfft2(th)))
    q = np.zeros((P, Nx, Nx // 2 + 1), dtype=np.complex128)
    w = np.zeros_like(th_gal)
    return sanitize_state(OracleState(q, w, th_gal, np.zeros(P)), grid)


# ---------------------------------------------------------------------------
# Scalar diagnostics -- nhqg/diagnostics.py:597-690 (the subset without the
# shell spectra and budgets)
# ---------------------------------------------------------------------------

DIAG_KEYS = ("KE_bt", "KE_bc", "KE_tot", "enstrophy", "Nusselt", "Nusselt_dealiased",
             "vol_avg_tw", "vol_avg_tw_dealiased", "q_rms", "w_rms", "th_rms", "th_bar_max")


def compute_diagnostics(state: OracleState, grid: OracleGrid) -> dict:
    """Depth-integrated (Clenshaw-Curtis) energies, rms values and Nusselt
    numbers of ``state``.  Half-plane Parseval weights 1 at ky = 0 and the
    Nyquist column, 2 elsewhere (nhqg/diagnostics.py:45-51), normalised by
    Nx^4; the dealiased heat flux is the mean-equation's flux profile: on
    the SBP grid mapped back to CGL for the balanced SBP2 exchange
    (nhqg/diagnostics.py:232-248, nhqg/solver.py:370-374), on the CGL grid
    otherwise (nhqg/diagnostics.py:272-281)."""
    q, w, th, tb = state
    Nx, Nk = grid.Nx, grid.Nk
    cc = grid.cc_weights
    psi_n = vmat(grid.V, invert_psi(q, grid.inv_denom))
    q_n = vmat(grid.V, q)
    w_n = vmat(grid.V, vmat(grid.w_stencil, w))
    th_n = vmat(grid.V, vmat(grid.dirichlet_stencil, th))
    wr = np.ones((Nx, Nk))
    if Nk > 2:
        wr[:, 1:Nk - 1] = 2.0
    norm = float(Nx) ** 4
    dint = lambda a: np.einsum("j,j...->...", cc, a)  # noqa: E731
    psi_bt = dint(psi_n)
    ksq = grid.ksq
    KE_bt = 0.5 * np.sum(ksq * np.abs(psi_bt) ** 2 * wr) / norm
    KE_tot = 0.5 * np.sum(ksq * dint(np.abs(psi_n) ** 2) * wr) / norm
    q_sq = np.sum(dint(np.abs(q_n) ** 2) * wr) / norm
    w_sq = np.sum(dint(np.abs(w_n) ** 2) * wr) / norm
    th_sq = np.sum(dint(np.abs(th_n) ** 2) * wr) / norm
    vol_tw = np.sum(dint(np.real(w_n * np.conj(th_n))) * wr) / norm
    if grid.mean_exchange_discretization in ("balanced_sbp2", "balanced_sbp2_pc"):
        c2s = grid.cgl_to_sbp
        flux = grid.sbp_to_cgl @ horizontal_mean(vmat(c2s, w_n), vmat(c2s, th_n), Nx, grid.Npad)
    else:
        flux = horizontal_mean(w_n, th_n, Nx, grid.Npad)
    vol_tw_d = float(np.sum(cc * flux))
    out = dict(KE_bt=KE_bt, KE_bc=KE_tot - KE_bt, KE_tot=KE_tot, enstrophy=0.5 * q_sq,
               Nusselt=1.0 + vol_tw, Nusselt_dealiased=1.0 + vol_tw_d, vol_avg_tw=vol_tw,
               vol_avg_tw_dealiased=vol_tw_d, q_rms=np.sqrt(q_sq), w_rms=np.sqrt(w_sq),
               th_rms=np.sqrt(th_sq), th_bar_max=float(np.max(np.abs(tb))),
               heat_flux_mismatch=vol_tw_d - vol_tw)
    # physical-space maxima over the Nx grid at every CGL level
    # (nhqg/diagnostics.py:631-641)
    kx3, ky3 = grid.kx[None], grid.ky[None]
    u = _irfft2(-1j * ky3 * psi_n, Nx)
    v = _irfft2(1j * kx3 * psi_n, Nx)
    wp = _irfft2(w_n, Nx)
    tp = _irfft2(th_n, Nx)
    out.update(max_speed=np.max(np.sqrt(u ** 2 + v ** 2)), max_w=np.max(np.abs(wp)),
               max_theta=np.max(np.abs(tp)), max_tw=np.max(np.abs(wp * tp)))
    return {k: float(v) for k, v in out.items()}


# the further scalars of compute_diagnostics (nhqg/diagnostics.py:680-699)
DIAG_EXTRA_KEYS = ("max_speed", "max_w", "max_theta", "max_tw", "heat_flux_mismatch")


# ---------------------------------------------------------------------------
# Spectra -- nhqg/diagnostics.py:48-101 (energy_spectrum and its helpers) and
# :583-594 (vertical_mode_energy, high_mode_fraction)
# ---------------------------------------------------------------------------

def horizontal_rfft_weight(ksq: np.ndarray) -> np.ndarray:
    """rfft2 Parseval weights: 2 on columns 1..Nk-2, 1 on ky = 0 and the
    Nyquist column (nhqg/diagnostics.py:48-53)."""
    Nk = ksq.shape[1]
    w = np.ones_like(ksq)
    if Nk > 2:
        w[:, 1:Nk - 1] = 2.0
    return w


def shell_bins(ksq: np.ndarray, L: float, n_bins: int | None = None):
    """(|k|, dk, bin centres): dk = 2 pi / L, n_bins = int(k_max / dk) + 1 by
    default (nhqg/diagnostics.py:56-65)."""
    k_mag = np.sqrt(ksq)
    dk = 2.0 * np.pi / L
    k_max = np.sqrt(np.max(ksq))
    if n_bins is None:
        n_bins = int(float(k_max / dk)) + 1
    return k_mag, dk, np.arange(n_bins) * dk + dk / 2


def shell_bin_index(ksq: np.ndarray, L: float, n_bins: int | None = None) -> np.ndarray:
    """Shell of every mode under the reference's test i dk <= |k| < (i+1) dk
    (nhqg/diagnostics.py:68-77), -1 where no shell holds the mode."""
    k_mag, dk, k_bins = shell_bins(ksq, L, n_bins)
    idx = np.full(ksq.shape, -1, dtype=np.int64)
    for i in range(k_bins.shape[0]):
        idx[(k_mag >= i * dk) & (k_mag < (i + 1) * dk)] = i
    return idx


def shell_bin_sum(q: np.ndarray, ksq: np.ndarray, L: float, n_bins: int | None = None):
    """Sum of a per-mode quantity over each shell (nhqg/diagnostics.py:68-77)."""
    k_mag, dk, k_bins = shell_bins(ksq, L, n_bins)
    spec = np.zeros_like(k_bins)
    for i in range(k_bins.shape[0]):
        spec[i] = np.sum(np.where((k_mag >= i * dk) & (k_mag < (i + 1) * dk), q, 0.0))
    return k_bins, spec


def energy_spectrum(psi_nodal: np.ndarray, ksq: np.ndarray, cc_weights: np.ndarray, L: float,
                    n_bins: int | None = None):
    """Barotropic, baroclinic and total kinetic energy per horizontal shell
    (k_bins, E_bt, E_bc, E_tot), unnormalised (nhqg/diagnostics.py:80-101)."""
    psi_bt = np.einsum("j,j...->...", cc_weights, psi_nodal)
    e_bt = 0.5 * ksq * np.abs(psi_bt) ** 2
    e_tot = 0.5 * ksq * np.einsum("j,j...->...", cc_weights, np.abs(psi_nodal) ** 2)
    w = horizontal_rfft_weight(ksq)
    k_bins, E_bt = shell_bin_sum(e_bt * w, ksq, L, n_bins)
    _, E_tot = shell_bin_sum(e_tot * w, ksq, L, n_bins)
    return k_bins, E_bt, E_tot - E_bt, E_tot


def shell_spectrum(field_nodal: np.ndarray, ksq: np.ndarray, cc_weights: np.ndarray, L: float,
                   n_bins: int | None = None):
    """Depth-integrated shell spectrum of a horizontally spectral field:
    (k_bins, sum over each shell of w_k sum_j cc_j |f_j(k)|^2), unnormalised
    (nhqg/diagnostics.py:104-111)."""
    f2 = np.einsum("j,j...->...", cc_weights, np.abs(field_nodal) ** 2)
    return shell_bin_sum(f2 * horizontal_rfft_weight(ksq), ksq, L, n_bins)


def field_shell_spectra(state: OracleState, grid: OracleGrid, n_bins: int | None = None) -> dict:
    """The q, w, theta horizontal shell spectra of compute_diagnostics at the
    CGL nodes (nhqg/diagnostics.py:667-669)."""
    q, w, th, _ = state
    cc, ksq, L = grid.cc_weights, grid.ksq, grid.cfg.L
    k_bins, qs = shell_spectrum(vmat(grid.V, q), ksq, cc, L, n_bins)
    _, ws = shell_spectrum(vmat(grid.V, vmat(grid.w_stencil, w)), ksq, cc, L, n_bins)
    _, ts = shell_spectrum(vmat(grid.V, vmat(grid.dirichlet_stencil, th)), ksq, cc, L, n_bins)
    return dict(k_bins=k_bins, q=qs, w=ws, th=ts)


def vertical_mode_energy(field_hat: np.ndarray) -> np.ndarray:
    """Sum over the horizontal modes of |f_n|^2 per Chebyshev index
    (nhqg/diagnostics.py:583-585)."""
    return np.sum(np.abs(field_hat) ** 2, axis=(1, 2))


def high_mode_fraction(spec: np.ndarray, frac: float = 0.25) -> float:
    """Share of the top max(1, int(n frac)) entries (nhqg/diagnostics.py:588-594)."""
    n = spec.shape[0]
    n_tail = max(1, int(n * frac))
    total = np.sum(spec)
    return float(np.sum(spec[-n_tail:]) / total) if total > 0 else 0.0


def psi_ke_vertical_spectrum(q_hat: np.ndarray, grid: OracleGrid) -> np.ndarray:
    """psi kinetic energy per Chebyshev index, sum_k w_k |k|^2 |psi_n(k)|^2 with
    the rfft weights w_k: the vertical-tail measure of the learned-closure study
    (a reported number in the reference, not one of its functions)."""
    psi = invert_psi(q_hat, grid.inv_denom)
    return np.sum(horizontal_rfft_weight(grid.ksq) * grid.ksq * np.abs(psi) ** 2, axis=(1, 2))


def spectra(state: OracleState, grid: OracleGrid, n_bins: int | None = None) -> dict:
    """energy_spectrum of the state's psi and the vertical mode energies of q,
    w, theta and of the psi kinetic energy."""
    q, w, th, _ = state
    psi_n = vmat(grid.V, invert_psi(q, grid.inv_denom))
    k_bins, E_bt, E_bc, E_tot = energy_spectrum(psi_n, grid.ksq, grid.cc_weights, grid.cfg.L, n_bins)
    return dict(k_bins=k_bins, E_bt=E_bt, E_bc=E_bc, E_tot=E_tot, q=vertical_mode_energy(q),
                w=vertical_mode_energy(w), th=vertical_mode_energy(th),
                psi_ke=psi_ke_vertical_spectrum(q, grid))
