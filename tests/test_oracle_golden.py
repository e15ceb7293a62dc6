"""Pin the CPU oracle against golden vectors produced by the reference source.

The fixtures in ``tests/golden`` hold the unmodified reference's outputs
(``tests/golden/make_golden.py``).  The oracle restates the same algorithm in
NumPy with different operation order (GEMM vs einsum, SciPy vs NumPy FFT), so
agreement is to round-off, not bitwise.
"""

import numpy as np
import pytest

import fixtures
import oracle
from oracle.nhqg_oracle import OracleConfig, OracleState
from _util import assert_state_close, rel_l2

TOL = 1e-12


def _grid(meta, arrays):
    cfg = dict(meta["cfg"])
    cfg.pop("_override_eta_sponge", None)
    grid = oracle.make_grid(OracleConfig(**cfg))
    if meta.get("override_eta_sponge"):
        grid = grid.replace(eta_hat=arrays["grid.eta_hat"][0], sponge_phys=arrays["grid.sponge_phys"],
                            sponge_phys_pad=arrays.get("grid.sponge_phys_pad"))
    return grid


def _state(arrays, prefix):
    return OracleState(*fixtures.state_from(arrays, prefix))


@pytest.fixture(scope="module", params=fixtures.CASES + fixtures.RK_CASES + fixtures.PAD_CASES)
def case(request):
    meta, arrays = fixtures.load_case(request.param)
    return request.param, meta, arrays, _grid(meta, arrays)


def _base(grid, meta):
    if meta["split"]:
        return grid.replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    return grid


def test_initial_state(case):
    name, meta, arrays, grid = case
    s0 = oracle.theta_perturbation_state(grid, seed=meta["seed"])
    assert_state_close(s0, _state(arrays, "s0"), TOL, th_bar_abs=0.0)


def test_explicit_rhs(case):
    name, meta, arrays, grid = case
    E = oracle.explicit_rhs_dispatch(_state(arrays, "r"), _base(grid, meta))
    assert_state_close(E, _state(arrays, "E"), TOL, th_bar_abs=1e-14)


def test_implicit_tendency(case):
    name, meta, arrays, grid = case
    I = oracle.implicit_tendency(_state(arrays, "r"), _base(grid, meta))
    assert_state_close(I, _state(arrays, "I"), TOL, th_bar_abs=1e-12)


def test_implicit_solve(case):
    name, meta, arrays, grid = case
    r = _state(arrays, "r")
    base = _base(grid, meta)
    q, w, th = oracle.imex_implicit_solve(r.q_hat, r.w_hat, r.th_hat, base)
    tb = oracle.imex_mean_temp_solve(r.th_bar, base)
    assert_state_close((q, w, th, tb), _state(arrays, "solve"), TOL, th_bar_abs=1e-13)


def test_corrector(case):
    name, meta, arrays, grid = case
    if not meta["split"]:
        pytest.skip("no SBP2 corrector in this recipe")
    alpha = grid.gamma_imex * grid.dt
    out = oracle.apply_balanced_sbp2_corrector(_state(arrays, "r"), grid, alpha)
    assert_state_close(out, _state(arrays, "corr"), TOL, th_bar_abs=1e-14)


def test_steps(case):
    name, meta, arrays, grid = case
    s = _state(arrays, "r")
    s = oracle.imex_step(s, grid)
    assert_state_close(s, _state(arrays, "r1"), TOL, th_bar_abs=1e-14)
    for _ in range(4):
        s = oracle.imex_step(s, grid)
    assert_state_close(s, _state(arrays, "r5"), 1e-11, th_bar_abs=1e-13)


def test_seeded_trajectory(case):
    name, meta, arrays, grid = case
    s = _state(arrays, "s0")
    for _ in range(meta["n_steps"]):
        s = oracle.imex_step(s, grid)
    assert_state_close(s, _state(arrays, "sN"), 1e-11, th_bar_abs=1e-16)


@pytest.mark.parametrize("case", fixtures.CASES)
def test_oracle_diagnostics_golden(case):
    """Scalar diagnostics against the reference's compute_diagnostics
    (tests/golden/diagnostics.npz, nhqg/diagnostics.py:597-690)."""
    meta, arrays = fixtures.load_case(case)
    grid = _grid(meta, arrays)
    gd = fixtures.load_diagnostics()
    for label in ("r", "s0"):
        got = oracle.compute_diagnostics(_state(arrays, label), grid)
        ref = gd[f"{case}.{label}"]
        for i, key in enumerate(oracle.DIAG_KEYS):
            assert abs(got[key] - ref[i]) <= 1e-12 * max(abs(ref[i]), 1e-300) + 1e-300, (case, label, key)


@pytest.mark.parametrize("case", fixtures.CASES + fixtures.PAD_CASES)
def test_oracle_diagnostics_extra_golden(case):
    """Physical-space maxima at the CGL nodes (max |u|, |w|, |theta|,
    |w theta|) and the heat-flux mismatch against the reference's
    compute_diagnostics (tests/golden/diagnostics_extra.npz,
    nhqg/diagnostics.py:631-641, 680-699), both dealiasing rules."""
    meta, arrays = fixtures.load_case(case)
    grid = _grid(meta, arrays)
    gd = fixtures.load_diagnostics_extra()
    keys = [str(k) for k in gd["keys"]]
    assert tuple(keys) == oracle.DIAG_EXTRA_KEYS
    for label in ("r", "s0"):
        got = oracle.compute_diagnostics(_state(arrays, label), grid)
        ref = gd[f"{case}.{label}"]
        for i, key in enumerate(keys):
            tol = 1e-12 * max(abs(ref[i]), 1e-300) if key != "heat_flux_mismatch" else 1e-13
            assert abs(got[key] - ref[i]) <= tol + 1e-300, (case, label, key, got[key], ref[i])


@pytest.mark.parametrize("case", fixtures.CASES + fixtures.PAD_CASES)
def test_oracle_field_spectra_golden(case):
    """Horizontal shell spectra of q, w, theta (compute_diagnostics' q/w/th
    horizontal spectra, nhqg/diagnostics.py:104-111, 667-669) against the
    reference: 1e-12 relative to each spectrum's largest entry."""
    meta, arrays = fixtures.load_case(case)
    grid = _grid(meta, arrays)
    gs = fixtures.load_field_spectra()
    for label in ("r", "s0"):
        got = oracle.field_shell_spectra(_state(arrays, label), grid)
        for key in ("k_bins", "q", "w", "th"):
            ref = gs[f"{case}.{label}.{key}"]
            assert got[key].shape == ref.shape, (case, label, key)
            scale = max(float(np.max(np.abs(ref))), 1e-300)
            assert float(np.max(np.abs(got[key] - ref))) <= 1e-12 * scale, (case, label, key)


@pytest.mark.parametrize("case", fixtures.CASES)
def test_oracle_spectra_golden(case):
    """Shell and vertical spectra against the reference's energy_spectrum and
    vertical_mode_energy (tests/golden/spectra.npz, nhqg/diagnostics.py:80-101,
    583-585): 1e-12 relative to each spectrum's largest entry."""
    meta, arrays = fixtures.load_case(case)
    grid = _grid(meta, arrays)
    gs = fixtures.load_spectra()
    for label in ("r", "s0"):
        got = oracle.spectra(oracle.OracleState(*_state(arrays, label)), grid)
        for key in fixtures.SPEC_KEYS:
            ref = gs[f"{case}.{label}.{key}"]
            assert got[key].shape == ref.shape, (case, label, key)
            scale = max(float(np.max(np.abs(ref))), 1e-300)
            assert float(np.max(np.abs(got[key] - ref))) <= 1e-12 * scale, (case, label, key)
        assert 0.0 <= oracle.high_mode_fraction(got["q"]) <= 1.0


def test_product_rounding_hook_changes_products():
    """The oracle's product-rounding test hook is off by default and, set to a
    BF16 rounding, moves the flux products by far more than 1e-6."""
    import oracle.nhqg_oracle as O
    assert O.PRODUCT_ROUNDING is None
    rng = np.random.default_rng(5)
    Nx = 16
    kx = 2 * np.pi * np.fft.fftfreq(Nx, d=1.0 / Nx) / 10.0
    ky = 2 * np.pi * np.arange(Nx // 2 + 1) / 10.0
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    mask = ((np.abs(np.round(KX * 10 / (2 * np.pi))) <= Nx // 3) &
            (np.round(KY * 10 / (2 * np.pi)) <= Nx // 3)).astype(float)
    f = [rng.standard_normal((2, Nx, Nx // 2 + 1)) * mask + 0j for _ in range(4)]
    ref = O.triple_conservative_flux_divergence_23(*f, KX, KY, mask, Nx)

    def bf16(a):
        b = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
        b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
        return b.astype(np.uint32).view(np.float32).astype(np.float64)

    try:
        O.PRODUCT_ROUNDING = bf16
        bad = O.triple_conservative_flux_divergence_23(*f, KX, KY, mask, Nx)
    finally:
        O.PRODUCT_ROUNDING = None
    for a, b in zip(bad, ref):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) > 1e-4
