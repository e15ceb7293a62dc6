"""Host precompute of every table the GPU time step reads.

``make_grid(cfg) -> Grid`` mirrors the reference entry point
(nhqg/grid.py:439-789) and the Grid field names (nhqg/grid.py:29-141) for
the fields the time step uses; arrays are host NumPy float64.  The Grid is
handed to the GPU engine once (``nhqg_ctx_create`` uploads it) and cached.

Operator construction follows the reference formulas term by term.  For the
per-|k|^2-shell IMEX inverses this is deliberate down to the evaluation
order: the reference forms B = w_pinv @ G_Z @ q_solve @ G_Z @ w_stencil with
large integer-valued factors, so the table carries rounding at the 1e-10
(Nz=64) .. 1e-9 (Nz=256) relative level for the lowest |k|; reproducing the
same NumPy operations on the same machine reproduces those bits, which the
parity tolerances (1e-12 per stage, 1e-9 over 100 steps) need.  Only shells
that own a 2/3-band mode are built (the time step never reads the others):
``imex_inv`` holds those rows and ``imex_shell_row`` maps each (kx, ky) to its
row, -1 outside the band; ``ksq_idx`` keeps the reference's shell numbering.
"""

from __future__ import annotations

from typing import NamedTuple

import numpy as np

from .config import NHQGConfig


class Grid(NamedTuple):
    Z: np.ndarray
    xi: np.ndarray
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
    Z_sbp: np.ndarray
    sbp_H: np.ndarray
    sbp_D1: np.ndarray
    sbp_L: np.ndarray
    cgl_to_sbp: np.ndarray
    sbp_to_cgl: np.ndarray
    kx: np.ndarray
    ky: np.ndarray
    ksq: np.ndarray
    inv_denom: np.ndarray
    mask_23: np.ndarray
    diss_q: np.ndarray
    diss_w: np.ndarray
    diss_th: np.ndarray
    diss_rate_q: np.ndarray
    diss_rate_w: np.ndarray
    diss_rate_th: np.ndarray
    inv_alpha_q: np.ndarray
    inv_alpha_th: np.ndarray
    imex_inv: np.ndarray
    q_solve: None
    ksq_idx: np.ndarray
    proj_dirichlet: np.ndarray
    proj_neumann: np.ndarray
    proj_w: np.ndarray
    beta: float
    eta_hat: np.ndarray | None
    sponge_phys: np.ndarray | None
    Ra_sigma: float
    sigma: float
    L: float
    Ld_inv_sq: float
    dt: float
    gamma_imex: float
    mean_temp_eps_sq: float
    Nx: int
    Nk: int
    Nz: int
    Nz_gal: int
    Npad: int
    thermal_closure: str
    q_boundary: str
    w_bc_top: str
    nonlinear_advection: str
    vertical_cutoff_n: int | None
    imex_scheme: str
    vertical_dealiasing: str
    horizontal_dealiasing: str
    mean_exchange_discretization: str
    sbp_transfer_mode: str
    sbp_corrector_substeps: int
    imex_matmul_chunk: int
    # GPU-engine extras
    imex_shell_row: np.ndarray       # (Nx, Nk) row of imex_inv, -1 outside the band
    eta_phys: np.ndarray | None      # irfft2(eta_hat) on the Nx grid (2/3 rule), or of the
                                     # zero-padded eta_hat on the Npad grid (3/2 rule)
    mean_solve: np.ndarray | None    # (P, P) inverse of the tau'd legacy mean operator
    imex_shell_coef: np.ndarray      # (rows of imex_inv, 2) alpha_w_eff, (gamma dt)^2 c_k / alpha_q
    cfg: NHQGConfig
    # (Npad, Npad) irfft2 of the zero-padded sigma, no rescale (nhqg/grid.py:110-113, 663-667)
    sponge_phys_pad: np.ndarray | None = None


_CLOSURES = ("fixed_conduction", "evolve_mean")
_DEALIASING = ("23_rule", "32_rule")
_EXCHANGES = ("legacy", "balanced_sbp2", "balanced_sbp2_pc")


def _cheb_coeff_diff(N: int) -> np.ndarray:
    """d/dxi on Chebyshev coefficients: (T_n)' = 2n sum_{k<n, n-k odd} T_k / c_k,
    c_0 = 2 (same integer matrix as the recurrence in nhqg/grid.py:148-169)."""
    G = np.zeros((N + 1, N + 1))
    for n in range(1, N + 1):
        for k in range(n - 1, -1, -2):
            G[k, n] = float(n) if k == 0 else 2.0 * n
    return G


def _cc_weights(N: int) -> np.ndarray:
    """Clenshaw-Curtis weights on [0, 1] (nhqg/grid.py:176-189)."""
    theta = np.pi * np.arange(N + 1, dtype=np.float64) / N
    w = np.zeros(N + 1)
    for j in range(N + 1):
        s = 0.0
        for k in range(1, N // 2 + 1):
            b = 1.0 if k == N // 2 else 2.0
            s += b * np.cos(2.0 * k * theta[j]) / (4.0 * k * k - 1.0)
        w[j] = (1.0 - s) / (N * (2.0 if j in (0, N) else 1.0))
    return w


def _interp_matrix(x_src: np.ndarray, x_dst: np.ndarray) -> np.ndarray:
    """Row-stochastic piecewise-linear interpolation (nhqg/grid.py:229-258)."""
    rev = bool(x_src[0] > x_src[-1])
    xs = x_src[::-1] if rev else x_src
    Mt = np.zeros((x_dst.size, xs.size))
    for i, x in enumerate(x_dst):
        if x <= xs[0]:
            Mt[i, 0] = 1.0
        elif x >= xs[-1]:
            Mt[i, -1] = 1.0
        else:
            j = int(np.searchsorted(xs, x, side="right") - 1)
            t = (x - xs[j]) / (xs[j + 1] - xs[j])
            Mt[i, j], Mt[i, j + 1] = 1.0 - t, t
    return Mt[:, ::-1] if rev else Mt


def _sbp2(N: int):
    """SBP2 norm, first derivative, Laplacian with zero boundary rows
    (nhqg/grid.py:261-286)."""
    dz = 1.0 / N
    h = np.ones(N + 1)
    h[0] = h[-1] = 0.5
    H = dz * np.diag(h)
    D1 = np.zeros((N + 1, N + 1))
    D1[0, :2] = [-1.0 / dz, 1.0 / dz]
    D1[N, N - 1:] = [-1.0 / dz, 1.0 / dz]
    Lp = np.zeros((N + 1, N + 1))
    for i in range(1, N):
        D1[i, i - 1], D1[i, i + 1] = -0.5 / dz, 0.5 / dz
        Lp[i, i - 1:i + 2] = [1.0 / dz ** 2, -2.0 / dz ** 2, 1.0 / dz ** 2]
    return H, D1, Lp


def _tau_projection(rows: np.ndarray, N: int) -> np.ndarray:
    """Rewrite a_{N-1}, a_N so two constraint rows hold (nhqg/grid.py:293-319)."""
    MR = np.linalg.inv(rows[:, N - 1:N + 1]) @ rows[:, :N - 1]
    P = np.eye(N + 1)
    P[N - 1, :] = 0.0
    P[N, :] = 0.0
    P[N - 1, :N - 1] = -MR[0]
    P[N, :N - 1] = -MR[1]
    return P


def _shell_inverse(kv, hyper_order, gamma, dt, nu_q, nu_w, nu_theta, drag, sigma,
                   Ra_sigma, Ld_inv_sq, WG, G_Z, w_stencil, NG, buoyancy_K):
    """A'^-1 for one shell, evaluated with the reference's operation order
    (nhqg/grid.py:398-430), q_boundary='none', and the shell's scalar
    coefficients (alpha_w_eff, (gamma dt)^2 c_k / alpha_q) of
    A' = alpha_w_eff I - (gamma dt)^2 c_k / alpha_q pinv_w G_Z^2 S_w, which the
    O(Nz) tau solve of the mixed-precision path uses (c_k = 0 when
    |k|^2 + Ld^-2 = 0)."""
    ksq_p = kv ** hyper_order
    alpha_q = 1.0 + gamma * dt * (nu_q * ksq_p + drag)
    alpha_w = 1.0 + gamma * dt * nu_w * ksq_p
    alpha_th = 1.0 + gamma * dt * (nu_theta / sigma) * ksq_p
    alpha_w_eff = alpha_w - (gamma * dt) ** 2 * Ra_sigma / alpha_th
    if buoyancy_K is None:
        couple = alpha_w_eff * np.eye(NG)
    else:
        couple = alpha_w * np.eye(NG) - (gamma * dt) ** 2 * (Ra_sigma / alpha_th) * buoyancy_K
    denom = kv + Ld_inv_sq
    if denom == 0.0:
        return np.linalg.inv(couple), (alpha_w_eff, 0.0)
    c_k = 1.0 / denom
    # (WG @ q_solve) with q_solve = (1/alpha_q) I is WG scaled entrywise
    # (each entry is one product plus exact zeros in the GEMM).
    B = ((WG * (1.0 / alpha_q)) @ G_Z) @ w_stencil
    coef = (alpha_w_eff, (gamma * dt) ** 2 * c_k / alpha_q)
    return np.linalg.inv(couple - (gamma * dt) ** 2 * c_k * B), coef


def _smooth_23(n: int) -> bool:
    while n % 2 == 0:
        n //= 2
    while n % 3 == 0:
        n //= 3
    return n == 1


def _zero_pad(f_hat: np.ndarray, Nx: int, Npad: int) -> np.ndarray:
    """(Nx, Nk) spectrum onto the (Npad, Npad//2+1) grid (nhqg/spectral.py:18-34)."""
    out = np.zeros((Npad, Npad // 2 + 1), dtype=np.complex128)
    out[:Nx // 2, :Nx // 2 + 1] = f_hat[:Nx // 2]
    out[Npad - Nx // 2:, :Nx // 2 + 1] = f_hat[Nx // 2:]
    return out


def compact_layout(grid: Grid) -> tuple[np.ndarray, int]:
    """Rows (fftfreq order) and column count of the engine's compact mode
    layout: the 2/3-rule keep-rectangle, or every rfft2 mode (3/2 rule)."""
    Nx = grid.Nx
    if grid.horizontal_dealiasing == "32_rule":
        return np.arange(Nx), Nx // 2 + 1
    K = Nx // 3
    return np.concatenate([np.arange(K + 1), np.arange(Nx - K, Nx)]), K + 1


def make_grid(cfg: NHQGConfig) -> Grid:
    """Build the Grid of ``cfg`` (nhqg/grid.py:439-789)."""
    if cfg.float_dtype != "float64":
        raise ValueError("the GPU time step computes in float64; set float_dtype='float64'")
    if cfg.horizontal_dealiasing not in _DEALIASING:
        raise ValueError(f"Unsupported horizontal_dealiasing={cfg.horizontal_dealiasing!r}")
    full = cfg.horizontal_dealiasing == "32_rule"
    if full and not _smooth_23(3 * cfg.Nx // 2):
        raise ValueError(f"the 3/2 rule needs Npad = 3Nx/2 = 2^a 3^b (Nx={cfg.Nx})")
    if cfg.q_boundary != "none":
        raise ValueError(f"Unsupported q_boundary={cfg.q_boundary!r} (GPU path: 'none')")
    if cfg.vertical_dealiasing != "none":
        raise ValueError(f"Unsupported vertical_dealiasing={cfg.vertical_dealiasing!r}")
    if cfg.vertical_cutoff_n is not None:
        raise ValueError("vertical_cutoff_n is not implemented by the GPU time step")
    if cfg.imex_scheme not in ("ars222", "rk443"):
        raise ValueError(f"Unsupported imex_scheme={cfg.imex_scheme!r} (GPU path: 'ars222', 'rk443')")
    if cfg.thermal_closure not in _CLOSURES:
        raise ValueError(f"Unsupported thermal_closure={cfg.thermal_closure!r}")
    if cfg.mean_exchange_discretization not in _EXCHANGES:
        raise ValueError(f"Unsupported mean_exchange_discretization={cfg.mean_exchange_discretization!r}")
    if cfg.nonlinear_advection not in ("flux", "jacobian"):
        raise ValueError(f"Unsupported nonlinear_advection={cfg.nonlinear_advection!r}")

    Nx, Nz, L, N = cfg.Nx, cfg.Nz, cfg.L, cfg.Nz
    Nk = cfg.Nk
    dt = cfg.dt
    j = np.arange(N + 1, dtype=np.float64)
    xi = np.cos(np.pi * j / N)
    Z = 0.5 * (1.0 + xi)
    cc_w = _cc_weights(N)
    G_Z = 2.0 * _cheb_coeff_diff(N)
    G_Z2 = G_Z @ G_Z
    V = np.cos(np.outer(j, j) * (np.pi / N))
    c = np.ones(N + 1)
    c[0] = c[N] = 2.0
    V_inv = (2.0 / N) * np.outer(1.0 / c, 1.0 / c) * V.T

    S = np.zeros((N + 1, N - 1))
    for n in range(N - 1):
        S[n, n], S[n + 2, n] = -1.0, 1.0
    S_pinv = np.zeros((N - 1, N + 1))
    S_pinv[:, :N - 1] = np.linalg.inv(S[:N - 1, :])

    e_plus = np.ones(N + 1)
    e_minus = np.array([(-1.0) ** n for n in range(N + 1)])
    tau_dir = np.stack([e_plus, e_minus])
    tau_neu = np.stack([e_plus @ G_Z, e_minus @ G_Z])
    proj_dir = _tau_projection(tau_dir, N)
    proj_neu = _tau_projection(tau_neu, N)

    if cfg.w_bc_top == "dirichlet":
        w_stencil, w_pinv, proj_w = S, S_pinv, proj_dir
        map_w_to_th = map_th_to_w = buoyancy_K = None
    elif cfg.w_bc_top == "neumann":
        w_stencil = np.zeros((N + 1, N - 1))
        for n in range(N - 1):
            b = -(n ** 2 + (n + 1) ** 2) / ((n + 1) ** 2 + (n + 2) ** 2)
            w_stencil[n, n], w_stencil[n + 1, n], w_stencil[n + 2, n] = 1.0, 1.0 + b, b
        w_pinv = np.zeros((N - 1, N + 1))
        w_pinv[:, :N - 1] = np.linalg.inv(w_stencil[:N - 1, :])
        proj_w = _tau_projection(np.stack([tau_neu[0], tau_dir[1]]), N)
        map_w_to_th = S_pinv @ w_stencil
        map_th_to_w = w_pinv @ S
        buoyancy_K = map_th_to_w @ map_w_to_th
    else:
        raise ValueError(f"Unsupported w_bc_top={cfg.w_bc_top!r}")

    Z_sbp = np.linspace(0.0, 1.0, N + 1)
    H, D1, Lsbp = _sbp2(N)
    c2s_lin = _interp_matrix(Z, Z_sbp)
    if cfg.sbp_transfer_mode == "interp":
        c2s, s2c = c2s_lin, _interp_matrix(Z_sbp, Z)
    elif cfg.sbp_transfer_mode == "mass_adjoint":
        c2s = c2s_lin
        s2c = np.linalg.solve(np.diag(cc_w), c2s.T @ H)
    elif cfg.sbp_transfer_mode == "weighted_polar":
        h = np.diag(H)
        U, _, Vt = np.linalg.svd(np.diag(np.sqrt(h)) @ c2s_lin @ np.diag(1.0 / np.sqrt(cc_w)),
                                 full_matrices=False)
        c2s = np.diag(1.0 / np.sqrt(h)) @ (U @ Vt) @ np.diag(np.sqrt(cc_w))
        s2c = np.linalg.solve(np.diag(cc_w), c2s.T @ H)
    else:
        raise ValueError(f"Unsupported sbp_transfer_mode={cfg.sbp_transfer_mode!r}")

    kx1 = 2.0 * np.pi * np.fft.fftfreq(Nx, d=L / Nx)
    ky1 = 2.0 * np.pi * np.arange(Nk) / L
    kx, ky = kx1[:, None], ky1[None, :]
    ksq = kx ** 2 + ky ** 2
    denom = ksq + cfg.Ld_inv_sq
    inv_denom = np.zeros_like(denom)
    np.divide(1.0, denom, out=inv_denom, where=denom > 0)

    K = Nx // 3
    ii = np.arange(Nx)
    kint = np.where(ii <= Nx // 2, ii, ii - Nx)
    mask = ((np.abs(kint)[:, None] <= K) & (np.arange(Nk)[None, :] <= K)).astype(np.float64)
    # modes the engine stores: the 2/3 keep-rectangle, or all of them (3/2 rule)
    in_band = np.ones((Nx, Nk), dtype=bool) if full else mask != 0
    Npad = cfg.Npad

    if cfg.gamma != 0.0 and cfg.beta != 0.0:
        raise ValueError("gamma (polar trap) and beta (flat beta-plane) are mutually exclusive")
    xy = np.arange(Nx) * (L / Nx)
    X, Y = np.meshgrid(xy, xy, indexing="ij")
    r = np.sqrt((X - L / 2.0) ** 2 + (Y - L / 2.0) ** 2)
    eta_hat = eta_phys = None
    r_star = None
    if cfg.gamma != 0.0:
        r_star = cfg.trap_r_star if cfg.trap_r_star is not None else 0.45 * (L / 2.0)
        sig_t = 0.5 * (1.0 - np.tanh(cfg.trap_sharpness * (r - r_star) / r_star))
        eta_hat = np.fft.rfft2(-0.5 * cfg.gamma * r ** 2 * sig_t)
        e_tot = np.sum(np.abs(eta_hat) ** 2)
        e_out = np.sum(np.abs(eta_hat * (1.0 - mask)) ** 2)
        if e_out > 1e-10 * e_tot:
            raise ValueError(
                f"Trap background PV is under-resolved: {e_out / e_tot:.2e} of its spectral "
                f"energy lies outside the 2/3 band (tolerance 1e-10)")
        if full:
            eta_phys = np.fft.irfft2(_zero_pad(eta_hat, Nx, Npad), s=(Npad, Npad))
        else:
            eta_hat = eta_hat * mask
            eta_phys = np.fft.irfft2(eta_hat, s=(Nx, Nx))
    sponge_phys = sponge_phys_pad = None
    if cfg.sponge_rate < 0.0:
        raise ValueError("sponge_rate must be >= 0")
    if cfg.sponge_rate > 0.0:
        if cfg.sponge_r_start is not None:
            r_s = cfg.sponge_r_start
        elif cfg.gamma != 0.0:
            r_s = 1.18 * r_star
        else:
            raise ValueError("sponge_r_start is required when gamma == 0 "
                             "(no trap radius to derive it from)")
        sig = cfg.sponge_rate * 0.5 * (1.0 + np.tanh(cfg.sponge_sharpness * (r - r_s) / r_s))
        sig_hat = np.fft.rfft2(sig)
        s_tot = np.sum(np.abs(sig_hat) ** 2)
        s_out = np.sum(np.abs(sig_hat * (1.0 - mask)) ** 2)
        if s_out > 1e-10 * s_tot:
            raise ValueError(
                f"Sponge profile is under-resolved: {s_out / s_tot:.2e} of its spectral "
                f"energy lies outside the 2/3 band (tolerance 1e-10)")
        if not full:
            sig_hat = sig_hat * mask
        sponge_phys = np.fft.irfft2(sig_hat, s=(Nx, Nx))
        sponge_phys_pad = np.fft.irfft2(_zero_pad(sig_hat, Nx, Npad), s=(Npad, Npad))

    # implicit coefficient of the scheme (nhqg/grid.py:671-676)
    gamma_imex = 1.0 - 1.0 / np.sqrt(2.0) if cfg.imex_scheme == "ars222" else 0.5
    p = cfg.hyper_order
    drq = cfg.nu_q * ksq ** p + cfg.drag
    drw = cfg.nu_w * ksq ** p
    drt = (cfg.nu_theta / cfg.sigma) * ksq ** p
    inv_aq = 1.0 / (1.0 + gamma_imex * dt * drq)
    inv_at = 1.0 / (1.0 + gamma_imex * dt * drt)

    # shells: reference numbering over all modes; tables for in-band shells
    ksq_rounded = np.round(ksq.ravel(), decimals=8)
    unique_ksq, inv_idx = np.unique(ksq_rounded, return_inverse=True)
    ksq_idx = inv_idx.astype(np.int32).reshape(Nx, Nk)
    used = np.unique(ksq_idx[in_band])
    row_of = -np.ones(len(unique_ksq), dtype=np.int32)
    row_of[used] = np.arange(len(used), dtype=np.int32)
    shell_row = np.where(in_band, row_of[ksq_idx], -1).astype(np.int32)
    WG = w_pinv @ G_Z
    Ra_sigma = cfg.Ra_tilde / cfg.sigma
    args = (p, gamma_imex, dt, cfg.nu_q, cfg.nu_w, cfg.nu_theta, cfg.drag, cfg.sigma, Ra_sigma,
            cfg.Ld_inv_sq, WG, G_Z, w_stencil, N - 1, buoyancy_K)
    imex_inv = np.empty((len(used), N - 1, N - 1))
    shell_coef = np.empty((len(used), 2))

    # one shell at a time: the BLAS inside each product is already threaded
    # (host threads around threaded BLAS calls oversubscribe the cores)
    for i in range(len(used)):
        imex_inv[i], shell_coef[i] = _shell_inverse(unique_ksq[used[i]], *args)

    mean_solve = None
    if cfg.thermal_closure == "evolve_mean" and cfg.mean_exchange_discretization == "legacy":
        alpha = gamma_imex * dt * cfg.mean_temp_eps_sq / cfg.sigma
        A = np.eye(N + 1) - alpha * G_Z2
        A[N - 1, :] = e_plus
        A[N, :] = e_minus
        mean_solve = np.linalg.inv(A)

    return Grid(
        Z=Z, xi=xi, cc_weights=cc_w, G_Z=G_Z, G_Z2=G_Z2, V=V, V_inv=V_inv,
        dirichlet_stencil=S, dirichlet_pinv=S_pinv, w_stencil=w_stencil, w_pinv=w_pinv,
        map_w_to_th=map_w_to_th, map_th_to_w=map_th_to_w, Z_sbp=Z_sbp, sbp_H=H, sbp_D1=D1,
        sbp_L=Lsbp, cgl_to_sbp=c2s, sbp_to_cgl=s2c, kx=kx, ky=ky, ksq=ksq, inv_denom=inv_denom,
        mask_23=mask, diss_q=np.exp(-drq * dt), diss_w=np.exp(-drw * dt), diss_th=np.exp(-drt * dt),
        diss_rate_q=drq, diss_rate_w=drw, diss_rate_th=drt, inv_alpha_q=inv_aq,
        inv_alpha_th=inv_at, imex_inv=imex_inv, q_solve=None, ksq_idx=ksq_idx,
        proj_dirichlet=proj_dir, proj_neumann=proj_neu, proj_w=proj_w, beta=float(cfg.beta),
        eta_hat=eta_hat, sponge_phys=sponge_phys, Ra_sigma=float(Ra_sigma), sigma=float(cfg.sigma),
        L=float(L), Ld_inv_sq=float(cfg.Ld_inv_sq), dt=float(dt), gamma_imex=float(gamma_imex),
        mean_temp_eps_sq=float(cfg.mean_temp_eps_sq), Nx=Nx, Nk=Nk, Nz=Nz, Nz_gal=Nz - 1,
        Npad=cfg.Npad, thermal_closure=cfg.thermal_closure, q_boundary=cfg.q_boundary,
        w_bc_top=cfg.w_bc_top, nonlinear_advection=cfg.nonlinear_advection,
        vertical_cutoff_n=cfg.vertical_cutoff_n, imex_scheme=cfg.imex_scheme,
        vertical_dealiasing=cfg.vertical_dealiasing,
        horizontal_dealiasing=cfg.horizontal_dealiasing,
        mean_exchange_discretization=cfg.mean_exchange_discretization,
        sbp_transfer_mode=cfg.sbp_transfer_mode,
        sbp_corrector_substeps=int(cfg.sbp_corrector_substeps),
        imex_matmul_chunk=int(cfg.imex_matmul_chunk),
        imex_shell_row=shell_row, eta_phys=eta_phys, mean_solve=mean_solve,
        imex_shell_coef=shell_coef, cfg=cfg, sponge_phys_pad=sponge_phys_pad,
    )
