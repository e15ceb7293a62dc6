"""Generate golden input/output vectors by executing the NHQG reference source.

Run in a checkout that has the reference mounted (it is NOT needed to run the
tests)::

    python tests/golden/make_golden.py /path/to/NHQG
    python tests/golden/make_golden.py /path/to/NHQG --diagnostics
    python tests/golden/make_golden.py /path/to/NHQG --diagnostics-extra
    python tests/golden/make_golden.py /path/to/NHQG --spectra
    python tests/golden/make_golden.py /path/to/NHQG --rk443
    python tests/golden/make_golden.py /path/to/NHQG --pad32

The reference (``nhqg/*.py``, unmodified, read-only) is imported under the
NumPy stand-in for ``jax`` in ``tests/golden/refshim``.  Every case records
the reference's own outputs for:

* ``s0``      the seeded theta' initial state (1e-3 x N(0,1) x sin(pi Z) on
              the CGL nodes, rfft2 -> V^-1 -> Dirichlet pinv, q'=w=0,
              Theta_bar=0, then ``sanitize_state``), PCG64 ``default_rng(seed)``
* ``sN``      ``imex_step`` applied N times to ``s0``
* ``r``       a strongly nonlinear band-limited random state, and at ``r``:
              ``E`` = explicit RHS, ``I`` = implicit tendency (reduced/base grid
              for the split SBP2 recipes), ``solve`` = ``imex_implicit_solve``
              with (R_q, R_w, R_th) = r, ``corr`` = the SBP2 thermal corrector
              with alpha = gamma*dt (split recipes only), ``r1``/``r5`` =
              ``imex_step`` applied 1/5 times.

Spectral arrays are stored packed to the 2/3 band (see ``fixtures.py``); the
script asserts the out-of-band content is exactly zero first.  The 3/2-rule
cases (``--pad32``) carry full-band states and store them unpacked.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from fixtures import out_of_band_max, pack  # noqa: E402

L_C = 2.0 * np.pi / 1.3048  # critical wavelength of rotating convection


BASE = dict(Ra_tilde=100.0, sigma=1.0, beta=0.0, Ld=float("inf"),
            nu_q=1.0, nu_w=1.0, nu_theta=1.0, hyper_order=1,
            nonlinear_advection="flux", horizontal_dealiasing="23_rule",
            float_dtype="float64", imex_scheme="ars222", dt=5e-5,
            L=10 * L_C)

CASES = {
    # production recipe (evolve_mean + balanced SBP2 predictor/corrector)
    "prod16": dict(Nx=16, Nz=12, thermal_closure="evolve_mean",
                   mean_exchange_discretization="balanced_sbp2_pc",
                   sbp_corrector_substeps=4),
    # plain ARS222 with fixed conduction (the config default closure)
    "fixed16": dict(Nx=16, Nz=10, thermal_closure="fixed_conduction"),
    # Jacobian form, beta plane, finite deformation radius, hyperviscosity, drag
    "jac16": dict(Nx=16, Nz=8, thermal_closure="fixed_conduction",
                  nonlinear_advection="jacobian", beta=0.7, Ld=3.0,
                  hyper_order=2, nu_q=1e-3, nu_w=2e-3, nu_theta=3e-3, drag=0.05),
    # open top + production recipe; trap eta and sponge sigma replaced by
    # band-limited fields (the resolution guards need Nx >= 96, see grid96)
    "polar16": dict(Nx=16, Nz=8, w_bc_top="neumann", thermal_closure="evolve_mean",
                    mean_exchange_discretization="balanced_sbp2_pc",
                    sbp_corrector_substeps=4, _override_eta_sponge=True),
    # radix-3 horizontal size, two substeps, mass-adjoint SBP transfer
    "radix24": dict(Nx=24, Nz=6, thermal_closure="evolve_mean",
                    mean_exchange_discretization="balanced_sbp2_pc",
                    sbp_corrector_substeps=2, sbp_transfer_mode="mass_adjoint"),
    # legacy explicit mean exchange (implicit 1-D mean solve), eps^2 != 1
    "legacy16": dict(Nx=16, Nz=8, thermal_closure="evolve_mean",
                     mean_exchange_discretization="legacy", mean_temp_eps_sq=0.7),
}

# ARS(4,4,3) ("rk443", nhqg/solver.py:1056-1122): the reference runs it with
# the legacy exchange only (nhqg/solver.py:1228-1242), gamma = 1/2 in the
# shell tables (nhqg/grid.py:671-676)
RK_CASES = {
    "rk443f16": dict(Nx=16, Nz=10, imex_scheme="rk443", thermal_closure="fixed_conduction"),
    "rk443l16": dict(Nx=16, Nz=8, imex_scheme="rk443", thermal_closure="evolve_mean",
                     mean_exchange_discretization="legacy", mean_temp_eps_sq=0.7),
}

# 3/2-rule padded products (horizontal_dealiasing='32_rule', the reference's
# config default; nhqg/spectral.py:147-253): states are full band, so these
# fixtures store spectral fields unpacked (Nx x Nk)
PAD_CASES = {
    # production recipe: padded <w theta> means in the SBP2 corrector
    "pad32p16": dict(Nx=16, Nz=8, horizontal_dealiasing="32_rule", thermal_closure="evolve_mean",
                     mean_exchange_discretization="balanced_sbp2_pc", sbp_corrector_substeps=4),
    # Jacobian form, beta plane, finite deformation radius, hyperviscosity, drag
    "pad32j16": dict(Nx=16, Nz=8, horizontal_dealiasing="32_rule", thermal_closure="fixed_conduction",
                     nonlinear_advection="jacobian", beta=0.7, Ld=3.0, hyper_order=2, nu_q=1e-3,
                     nu_w=2e-3, nu_theta=3e-3, drag=0.05),
    # open top, trap eta and padded sponge (band-limited stand-ins), flux form
    "pad32o16": dict(Nx=16, Nz=8, horizontal_dealiasing="32_rule", w_bc_top="neumann",
                     thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
                     sbp_corrector_substeps=4, _override_eta_sponge=True),
    # Jacobian form with eta and the padded sponge
    "pad32s16": dict(Nx=16, Nz=6, horizontal_dealiasing="32_rule", thermal_closure="fixed_conduction",
                     nonlinear_advection="jacobian", _override_eta_sponge=True),
    # radix-3 sizes (Nx = 24, Npad = 36), legacy explicit exchange
    "pad32l24": dict(Nx=24, Nz=6, horizontal_dealiasing="32_rule", thermal_closure="evolve_mean",
                     mean_exchange_discretization="legacy", mean_temp_eps_sq=0.7),
}

# grid-only fixture: the polar trap / sponge / open-top tables at a size whose
# resolution guards pass (production flavour scaled down from 256^2 x 32)
GRID_CASE = dict(Nx=96, Nz=8, L=40.0, gamma=2.2e-3, trap_r_star=8.0,
                 trap_sharpness=5.0, sponge_rate=5.0, sponge_r_start=10.4,
                 sponge_sharpness=5.0, w_bc_top="neumann",
                 thermal_closure="evolve_mean",
                 mean_exchange_discretization="balanced_sbp2_pc",
                 sbp_corrector_substeps=4)

N_STEPS = 10
jnp_asarray = None  # bound to the stand-in's jax.numpy.asarray in main()


def theta_init(grid, solver, seed, amplitude=1e-3):
    P, Nx = grid.Nz + 1, grid.Nx
    rng = np.random.default_rng(seed)
    Z = np.asarray(grid.Z)
    th = amplitude * rng.standard_normal((P, Nx, Nx)) * np.sin(np.pi * Z)[:, None, None]
    th_nodal = np.fft.rfft2(th)
    th_cheb = np.einsum("ij,j...->i...", np.asarray(grid.V_inv), th_nodal)
    th_gal = np.einsum("ij,j...->i...", np.asarray(grid.dirichlet_pinv), th_cheb)
    zeros_q = np.zeros((P, Nx, Nx // 2 + 1), dtype=np.complex128)
    zeros_w = np.zeros_like(th_gal)
    s = solver.State(*(jnp_asarray(a) for a in (zeros_q, zeros_w, th_gal, np.zeros(P))))
    return solver.sanitize_state(s, grid)


def rich_state(grid, solver, seed):
    """Band-limited random state with O(1) nonlinearity."""
    rng = np.random.default_rng(1000 + seed)
    P, G, Nx, Nk = grid.Nz + 1, grid.Nz - 1, grid.Nx, grid.Nx // 2 + 1
    ksq = np.asarray(grid.ksq)
    env = np.exp(-ksq / (2.0 * float(np.max(ksq)) / 9.0))

    def field(n):
        z = rng.standard_normal((n, Nx, Nk)) + 1j * rng.standard_normal((n, Nx, Nk))
        decay = 1.0 / (1.0 + np.arange(n))[:, None, None]
        return 0.3 * z * env[None] * decay

    q, w, th = field(P), field(G), field(G)
    th_bar = np.asarray(grid.proj_dirichlet) @ (0.05 * rng.standard_normal(P) / (1 + np.arange(P)))
    s = solver.State(*(jnp_asarray(a) for a in (q, w, th, th_bar)))
    s = solver.sanitize_state(s, grid)
    return solver.State(solver.zero_mean(s.q_hat), solver.zero_mean(s.w_hat),
                        solver.zero_mean(s.th_hat), s.th_bar)


def smooth_eta_sponge(grid):
    """Band-limited stand-ins for the trap PV eta and the sponge rate sigma."""
    Nx, L = grid.Nx, float(grid.L)
    x = np.arange(Nx) * (L / Nx)
    X, Y = np.meshgrid(x, x, indexing="ij")
    k0 = 2.0 * np.pi / L
    eta = -2.2e-3 * (3.0 + np.cos(k0 * X) + np.cos(k0 * Y) + 0.5 * np.cos(k0 * (X + 2 * Y)))
    sigma = 5.0 * (0.5 + 0.25 * np.cos(k0 * X) * np.cos(k0 * Y) + 0.2 * np.sin(2 * k0 * X))
    return np.fft.rfft2(eta), sigma


def padded_sponge(sponge_phys, Nx, Npad):
    """The pre-attenuated padded sponge of a sponge field, built as
    nhqg/grid.py:663-667 builds grid.sponge_phys_pad."""
    s_hat = np.fft.rfft2(sponge_phys)
    Nk = Nx // 2 + 1
    pad = np.zeros((Npad, Npad // 2 + 1), dtype=np.complex128)
    pad[:Nx // 2, :Nk] = s_hat[:Nx // 2, :]
    pad[Npad - Nx // 2:, :Nk] = s_hat[Nx // 2:, :]
    return np.fft.irfft2(pad, s=(Npad, Npad))


def main(ref_root: str, cases: dict | None = None, grid_fixture: bool = True) -> None:
    sys.path.insert(0, str(HERE / "refshim"))
    sys.path.insert(0, ref_root)
    from nhqg import solver  # noqa: E402
    from nhqg.config import NHQGConfig  # noqa: E402
    from nhqg.grid import make_grid  # noqa: E402
    import jax.numpy as jnp  # the stand-in  # noqa: E402

    global jnp_asarray
    jnp_asarray = jnp.asarray

    for name, over in (CASES if cases is None else cases).items():
        cfgd = dict(BASE)
        cfgd.update(over)
        override = cfgd.pop("_override_eta_sponge", False)
        cfg = NHQGConfig(**cfgd)
        grid = make_grid(cfg)
        Nx = grid.Nx
        extra = {}
        full = grid.horizontal_dealiasing == "32_rule"
        if override:
            eta_hat, sponge_phys = smooth_eta_sponge(grid)
            grid = grid._replace(eta_hat=jnp.asarray(eta_hat),
                                 sponge_phys=jnp.asarray(sponge_phys))
            extra = {"grid.eta_hat__packed": pack(eta_hat[None], Nx),
                     "grid.sponge_phys": sponge_phys}
            if full:
                pad_sponge = padded_sponge(sponge_phys, Nx, int(grid.Npad))
                grid = grid._replace(sponge_phys_pad=jnp.asarray(pad_sponge))
                extra["grid.sponge_phys_pad"] = pad_sponge
        split = solver.uses_split_thermal_exchange(grid)
        base = (grid._replace(thermal_closure="fixed_conduction",
                              mean_exchange_discretization="legacy") if split else grid)
        out: dict[str, np.ndarray] = {}

        def put_state(prefix, s):
            for fname, arr in zip(("q_hat", "w_hat", "th_hat", "th_bar"), s):
                arr = np.asarray(arr)
                if arr.ndim == 3 and full:
                    out[f"{prefix}.{fname}"] = arr
                elif arr.ndim == 3:
                    oob = out_of_band_max(arr, Nx)
                    assert oob == 0.0, (name, prefix, fname, oob)
                    out[f"{prefix}.{fname}__packed"] = pack(arr, Nx)
                else:
                    out[f"{prefix}.{fname}"] = np.asarray(arr, dtype=np.float64)

        s0 = theta_init(grid, solver, seed=0)
        put_state("s0", s0)
        s = s0
        for _ in range(N_STEPS):
            s = solver.imex_step(s, grid)
        put_state("sN", s)

        r = rich_state(grid, solver, seed=0)
        put_state("r", r)
        put_state("E", solver.explicit_rhs_dispatch(r, base))
        put_state("I", solver.implicit_tendency(r, base))
        qn, wn, thn = solver.imex_implicit_solve(r.q_hat, r.w_hat, r.th_hat, base)
        th_bar_n = solver.imex_mean_temp_solve(r.th_bar, base)
        put_state("solve", (qn, wn, thn, th_bar_n))
        if split:
            alpha = float(grid.gamma_imex) * float(grid.dt)
            put_state("corr", solver._apply_balanced_sbp2_corrector(r, grid, alpha))
        s = solver.imex_step(r, grid)
        put_state("r1", s)
        for _ in range(4):
            s = solver.imex_step(s, grid)
        put_state("r5", s)

        out.update(extra)
        meta = dict(cfg=cfgd, n_steps=N_STEPS, split=split, seed=0,
                    override_eta_sponge=bool(override),
                    rng="numpy PCG64 default_rng", generator="tests/golden/make_golden.py")
        np.savez_compressed(HERE / f"{name}.npz", meta=json.dumps(meta), **out)
        size = (HERE / f"{name}.npz").stat().st_size
        print(f"{name}: {len(out)} arrays, {size / 1024:.0f} KiB")

    if not grid_fixture:
        return
    cfgd = dict(BASE)
    cfgd.update(GRID_CASE)
    grid = make_grid(NHQGConfig(**cfgd))
    Nx = grid.Nx
    g = {}
    for key in ("eta_hat",):
        g[f"grid.{key}__packed"] = pack(np.asarray(getattr(grid, key))[None], Nx)
    for key in ("sponge_phys", "G_Z", "G_Z2", "V", "V_inv", "dirichlet_stencil",
                "dirichlet_pinv", "w_stencil", "w_pinv", "map_w_to_th", "map_th_to_w",
                "proj_dirichlet", "proj_neumann", "proj_w", "sbp_D1", "sbp_L",
                "cgl_to_sbp", "sbp_to_cgl", "Z", "cc_weights", "inv_denom",
                "inv_alpha_q", "inv_alpha_th", "diss_rate_q", "mask_23", "ksq_idx"):
        g[f"grid.{key}"] = np.asarray(getattr(grid, key))
    ksq_idx = np.asarray(grid.ksq_idx)
    picks = np.unique(pack(ksq_idx[None], Nx)[0].ravel())[::97]
    g["grid.imex_inv_pick"] = picks
    g["grid.imex_inv"] = np.asarray(grid.imex_inv)[picks]
    meta = dict(cfg=cfgd, generator="tests/golden/make_golden.py")
    np.savez_compressed(HERE / "grid96.npz", meta=json.dumps(meta), **g)
    print(f"grid96: {(HERE / 'grid96.npz').stat().st_size / 1024:.0f} KiB")


DIAG_KEYS = ("KE_bt", "KE_bc", "KE_tot", "enstrophy", "Nusselt", "Nusselt_dealiased",
             "vol_avg_tw", "vol_avg_tw_dealiased", "q_rms", "w_rms", "th_rms", "th_bar_max")


def diagnostics_main(ref_root: str) -> None:
    """Reference ``compute_diagnostics`` (nhqg/diagnostics.py:597-690) scalars
    at the ``r`` and ``s0`` states of every case -> ``diagnostics.npz``
    (``<case>.<state>`` = values in ``DIAG_KEYS`` order)."""
    sys.path.insert(0, str(HERE / "refshim"))
    sys.path.insert(0, ref_root)
    from nhqg import diagnostics, solver  # noqa: E402
    from nhqg.config import NHQGConfig  # noqa: E402
    from nhqg.grid import make_grid  # noqa: E402
    import jax.numpy as jnp  # the stand-in  # noqa: E402

    global jnp_asarray
    jnp_asarray = jnp.asarray
    out = {}
    for name, over in CASES.items():
        cfgd = dict(BASE)
        cfgd.update(over)
        override = cfgd.pop("_override_eta_sponge", False)
        grid = make_grid(NHQGConfig(**cfgd))
        if override:
            eta_hat, sponge_phys = smooth_eta_sponge(grid)
            grid = grid._replace(eta_hat=jnp.asarray(eta_hat), sponge_phys=jnp.asarray(sponge_phys))
        for label, st in (("r", rich_state(grid, solver, seed=0)),
                          ("s0", theta_init(grid, solver, seed=0))):
            d = diagnostics.compute_diagnostics(st, grid)
            out[f"{name}.{label}"] = np.array([float(np.asarray(d[k])) for k in DIAG_KEYS])
    np.savez_compressed(HERE / "diagnostics.npz", keys=np.array(DIAG_KEYS), **out)
    print(f"diagnostics: {len(out)} entries")


DIAG_EXTRA_KEYS = ("max_speed", "max_w", "max_theta", "max_tw", "heat_flux_mismatch")


def diagnostics_extra_main(ref_root: str) -> None:
    """The further compute_diagnostics outputs (nhqg/diagnostics.py:631-641,
    667-669, 680-699) at the ``r`` and ``s0`` states of the 2/3- and 3/2-rule
    cases: the physical-space maxima at the CGL nodes and the heat-flux
    mismatch -> ``diagnostics_extra.npz`` (``<case>.<state>`` = values in
    DIAG_EXTRA_KEYS order), and the q, w, theta horizontal shell spectra ->
    ``field_spectra.npz`` (``<case>.<state>.<k_bins|q|w|th>``)."""
    sys.path.insert(0, str(HERE / "refshim"))
    sys.path.insert(0, ref_root)
    from nhqg import diagnostics, solver  # noqa: E402
    from nhqg.config import NHQGConfig  # noqa: E402
    from nhqg.grid import make_grid  # noqa: E402
    import jax.numpy as jnp  # the stand-in  # noqa: E402

    global jnp_asarray
    jnp_asarray = jnp.asarray
    out, spec = {}, {}
    for name, over in {**CASES, **PAD_CASES}.items():
        cfgd = dict(BASE)
        cfgd.update(over)
        override = cfgd.pop("_override_eta_sponge", False)
        grid = make_grid(NHQGConfig(**cfgd))
        if override:
            eta_hat, sponge_phys = smooth_eta_sponge(grid)
            grid = grid._replace(eta_hat=jnp.asarray(eta_hat), sponge_phys=jnp.asarray(sponge_phys))
            if grid.horizontal_dealiasing == "32_rule":
                grid = grid._replace(sponge_phys_pad=jnp.asarray(
                    padded_sponge(sponge_phys, grid.Nx, int(grid.Npad))))
        for label, st in (("r", rich_state(grid, solver, seed=0)),
                          ("s0", theta_init(grid, solver, seed=0))):
            d = diagnostics.compute_diagnostics(st, grid)
            out[f"{name}.{label}"] = np.array([float(np.asarray(d[k])) for k in DIAG_EXTRA_KEYS])
            for key, ref_key in (("k_bins", "k_bins"), ("q", "q_horiz_spec"), ("w", "w_horiz_spec"),
                                 ("th", "th_horiz_spec")):
                spec[f"{name}.{label}.{key}"] = np.asarray(d[ref_key], dtype=np.float64)
    np.savez_compressed(HERE / "diagnostics_extra.npz", keys=np.array(DIAG_EXTRA_KEYS), **out)
    np.savez_compressed(HERE / "field_spectra.npz", **spec)
    print(f"diagnostics_extra: {len(out)} entries; field_spectra: {len(spec)} arrays")


SPEC_KEYS = ("k_bins", "E_bt", "E_bc", "E_tot", "q", "w", "th")


def spectra_main(ref_root: str) -> None:
    """Reference ``energy_spectrum`` of psi at the CGL nodes
    (nhqg/diagnostics.py:80-101, called as compute_diagnostics' budget path
    does, with grid.L) and ``vertical_mode_energy`` (:583-585) of q, w, theta
    at the ``r`` and ``s0`` states of every case -> ``spectra.npz``
    (``<case>.<state>.<key>``, keys SPEC_KEYS)."""
    sys.path.insert(0, str(HERE / "refshim"))
    sys.path.insert(0, ref_root)
    from nhqg import diagnostics, solver  # noqa: E402
    from nhqg.config import NHQGConfig  # noqa: E402
    from nhqg.grid import make_grid  # noqa: E402
    import jax.numpy as jnp  # the stand-in  # noqa: E402

    global jnp_asarray
    jnp_asarray = jnp.asarray
    out = {}
    for name, over in CASES.items():
        cfgd = dict(BASE)
        cfgd.update(over)
        override = cfgd.pop("_override_eta_sponge", False)
        grid = make_grid(NHQGConfig(**cfgd))
        if override:
            eta_hat, sponge_phys = smooth_eta_sponge(grid)
            grid = grid._replace(eta_hat=jnp.asarray(eta_hat), sponge_phys=jnp.asarray(sponge_phys))
        for label, st in (("r", rich_state(grid, solver, seed=0)),
                          ("s0", theta_init(grid, solver, seed=0))):
            psi_nodal = solver._to_nodal(solver.invert_psi(st.q_hat, grid.inv_denom), grid.V)
            k_bins, E_bt, E_bc, E_tot = diagnostics.energy_spectrum(psi_nodal, grid.ksq, grid.cc_weights,
                                                                    float(grid.L))
            vals = dict(k_bins=k_bins, E_bt=E_bt, E_bc=E_bc, E_tot=E_tot,
                        q=diagnostics.vertical_mode_energy(st.q_hat),
                        w=diagnostics.vertical_mode_energy(st.w_hat),
                        th=diagnostics.vertical_mode_energy(st.th_hat))
            for k in SPEC_KEYS:
                out[f"{name}.{label}.{k}"] = np.asarray(vals[k], dtype=np.float64)
    np.savez_compressed(HERE / "spectra.npz", **out)
    print(f"spectra: {len(out)} arrays, {(HERE / 'spectra.npz').stat().st_size / 1024:.0f} KiB")


# the reference's own bitwise regression (tests/test_mixed_bc_plumbing.py:99-117):
# make_initial_state(seed=0, amplitude=1e-3) with JAX's PRNG, then 20 steps
JAXPRNG_CFG = dict(Nx=32, Nz=16, L=20.0, Ra_tilde=100.0, sigma=1.0, beta=0.0, Ld=float("inf"),
                   dt=1e-3, float_dtype="float64", nu_q=1.0, nu_w=1.0, nu_theta=1.0, hyper_order=1,
                   nonlinear_advection="flux", horizontal_dealiasing="23_rule",
                   thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
                   sbp_corrector_substeps=2)


def jaxprng_main(ref_root: str) -> None:
    """Pack the reference's data file tests/data/m2b_dirichlet_evolvemean_ref.npz
    (generated by the reference with JAX on CPU) into jaxprng_m2b.npz."""
    z = np.load(Path(ref_root) / "tests" / "data" / "m2b_dirichlet_evolvemean_ref.npz")
    out = {}
    for f in ("q_hat", "w_hat", "th_hat"):
        a = np.asarray(z[f])
        assert out_of_band_max(a, JAXPRNG_CFG["Nx"]) == 0.0, f
        out[f"sN.{f}__packed"] = pack(a, JAXPRNG_CFG["Nx"])
    out["sN.th_bar"] = np.asarray(z["th_bar"], dtype=np.float64)
    meta = dict(cfg=JAXPRNG_CFG, n_steps=20, seed=0, amplitude=1e-3,
                source="reference tests/data/m2b_dirichlet_evolvemean_ref.npz",
                generator="tests/golden/make_golden.py --jaxprng")
    np.savez_compressed(HERE / "jaxprng_m2b.npz", meta=json.dumps(meta), **out)
    print(f"jaxprng_m2b: {(HERE / 'jaxprng_m2b.npz').stat().st_size / 1024:.0f} KiB")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        sys.exit("usage: make_golden.py <path to the NHQG reference checkout> [--diagnostics | "
                 "--diagnostics-extra | --spectra | --rk443 | --pad32 | --jaxprng]")
    root = args[0]
    if "--diagnostics" in sys.argv:
        diagnostics_main(root)
    elif "--diagnostics-extra" in sys.argv:
        diagnostics_extra_main(root)
    elif "--spectra" in sys.argv:
        spectra_main(root)
    elif "--rk443" in sys.argv:
        main(root, RK_CASES, grid_fixture=False)
    elif "--pad32" in sys.argv:
        main(root, PAD_CASES, grid_fixture=False)
    elif "--jaxprng" in sys.argv:
        jaxprng_main(root)
    else:
        main(root)
