"""GPU parity of the 3/2-rule path (horizontal_dealiasing='32_rule', the
reference's config default) through the C ABI: products on the zero-padded
Npad = 3Nx/2 grid (nhqg/spectral.py:18-75, 147-253), full-band states and the
padded horizontal means of the mean exchange (nhqg/solver.py:204-245, 836,
931), against the reference's golden vectors (tests/golden/pad32*.npz, made
by tests/golden/make_golden.py --pad32) and the CPU oracle.

Tolerances (relative L2 per field) as for the 2/3 rule: 1e-13 for the plane
products, 1e-12 for one operator or one step, 1e-11 for 5 and 10 steps, 1e-9
after 40 steps against the oracle; the mixed-precision step within 1e-6 of
the plain one; diagnostics 1e-12 and spectra 1e-11 relative.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fixtures
import oracle
from oracle.nhqg_oracle import OracleConfig, OracleState
from _util import assert_state_close, rel_l2

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402
from nhqg_gb300 import spectral as SP  # noqa: E402
from nhqg_gb300.diagnostics import DIAG_KEYS, compute_diagnostics, spectra  # noqa: E402

L_C = 2.0 * np.pi / 1.3048


def _host(state):
    return tuple(t.detach().cpu().numpy() for t in state)


def _box(Nx, L):
    kx = (2 * np.pi * np.fft.fftfreq(Nx, d=L / Nx))[:, None]
    ky = (2 * np.pi * np.arange(Nx // 2 + 1) / L)[None, :]
    return kx, ky


# ---------------------------------------------------------------- planes
@pytest.mark.parametrize("Nx", [16, 24, 64, 128, 256])
@pytest.mark.parametrize("form", ["flux", "jacobian"])
def test_padded_products_random(Nx, form):
    """Full-band random planes (Nyquist row and column included, and the
    imaginary parts irfft2 drops) against the oracle's padded products."""
    rng = np.random.default_rng(Nx + 7)
    kx, ky = _box(Nx, 37.0)
    shp = (3, Nx, Nx // 2 + 1)
    f = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(4)]
    Npad = 3 * Nx // 2
    ofn = oracle.triple_conservative_flux_divergence_32 if form == "flux" else oracle.triple_jacobian_32
    gfn = SP.triple_conservative_flux_divergence if form == "flux" else SP.triple_jacobian
    ref = ofn(*f, kx, ky, Nx, Npad)
    got = gfn(*f, kx, ky, Nx, Npad)
    for g, r in zip(got, ref):
        assert rel_l2(g.cpu().numpy(), r) <= 1e-13


def test_padded_jacobian_analytic():
    """J[sin x, sin y] = cos x cos y exactly under the 3/2 rule too
    (reference tests/test_spectral.py:40-62)."""
    Nx, L = 32, 2 * np.pi
    kx, ky = _box(Nx, L)
    x = np.linspace(0, L, Nx, endpoint=False)
    X, Y = np.meshgrid(x, x, indexing="ij")
    A, B = np.fft.rfft2(np.sin(X))[None], np.fft.rfft2(np.sin(Y))[None]
    for fn in (SP.triple_jacobian, SP.triple_conservative_flux_divergence):
        J = fn(A, B, B, B, kx, ky, Nx, 3 * Nx // 2)[0].cpu().numpy()[0]
        np.testing.assert_allclose(np.fft.irfft2(J, s=(Nx, Nx)), np.cos(X) * np.cos(Y), atol=1e-12)


def test_padded_sponge_product():
    Nx = 48
    Npad = 3 * Nx // 2
    rng = np.random.default_rng(5)
    x = np.arange(Npad) * (2 * np.pi / Npad)
    X, Y = np.meshgrid(x, x, indexing="ij")
    sigma_pad = 2.0 + np.cos(X) * np.sin(2 * Y)
    f = rng.standard_normal((4, Nx, Nx // 2 + 1)) + 1j * rng.standard_normal((4, Nx, Nx // 2 + 1))
    ref = oracle.sponge_product_32(f, sigma_pad, Nx, Npad)
    got = SP.sponge_product_32(f, sigma_pad, Nx, Npad).cpu().numpy()
    assert rel_l2(got, ref) <= 1e-13
    with pytest.raises(ValueError):
        SP.sponge_product_32(f, sigma_pad, Nx, Nx)


# ---------------------------------------------------------------- golden cases
def _grids(meta, arrays):
    cfg = dict(meta["cfg"])
    cfg.pop("_override_eta_sponge", None)
    g = make_grid(NHQGConfig(**cfg))
    o = oracle.make_grid(OracleConfig(**cfg))
    if meta.get("override_eta_sponge"):
        eta = arrays["grid.eta_hat"][0]
        sp, spp = arrays["grid.sponge_phys"], arrays["grid.sponge_phys_pad"]
        g = g._replace(eta_hat=eta, sponge_phys=sp, sponge_phys_pad=spp)
        o = o.replace(eta_hat=eta, sponge_phys=sp, sponge_phys_pad=spp)
    return g, o


@pytest.fixture(scope="module", params=fixtures.PAD_CASES)
def case(request):
    meta, arrays = fixtures.load_case(request.param)
    g, o = _grids(meta, arrays)
    return request.param, meta, arrays, g, o


def _base(grid, meta):
    if meta["split"]:
        return grid._replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    return grid


def test_golden_operators(case):
    name, meta, arrays, g, o = case
    assert g.horizontal_dealiasing == "32_rule" and g.Npad == 3 * g.Nx // 2
    r = fixtures.state_from(arrays, "r")
    base = _base(g, meta)
    assert_state_close(_host(S.explicit_rhs(r, base)), fixtures.state_from(arrays, "E"), 1e-12,
                       th_bar_abs=1e-14)
    assert_state_close(_host(S.implicit_tendency(r, base)), fixtures.state_from(arrays, "I"), 1e-12,
                       th_bar_abs=1e-12)
    q, w, th = S.imex_implicit_solve(r[0], r[1], r[2], base)
    tb = S.imex_mean_temp_solve(r[3], base)
    assert_state_close(_host((q, w, th, tb)), fixtures.state_from(arrays, "solve"), 1e-12,
                       th_bar_abs=1e-13)
    if meta["split"]:
        out = S.apply_balanced_sbp2_corrector(r, g, g.gamma_imex * g.dt)
        assert_state_close(_host(out), fixtures.state_from(arrays, "corr"), 1e-12, th_bar_abs=1e-14)


def test_golden_steps(case):
    name, meta, arrays, g, o = case
    s = S.imex_step(fixtures.state_from(arrays, "r"), g)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r1"), 1e-12, th_bar_abs=1e-14)
    S.step_inplace(s, g, 4, check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r5"), 1e-11, th_bar_abs=1e-13)
    s = S.to_device(fixtures.state_from(arrays, "s0"))
    S.step_inplace(s, g, meta["n_steps"], check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "sN"), 1e-11, th_bar_abs=1e-16)


def test_steps_keep_hermitian_columns(case):
    """sanitize_state under the 3/2 rule: the ky = 0 and ky = Nx/2 columns
    are Hermitian in kx, and nothing is band-limited (nhqg/solver.py:128-146)."""
    name, meta, arrays, g, o = case
    s = _host(S.imex_step(fixtures.state_from(arrays, "r"), g))
    neg = (-np.arange(g.Nx)) % g.Nx
    for f in s[:3]:
        for c in (0, -1):
            col = f[:, :, c]
            assert np.max(np.abs(col - np.conj(col[:, neg]))) <= 1e-15 * np.max(np.abs(f))
        assert np.max(np.abs(f[:, g.Nx // 2, 1:-1])) > 0.0  # the Nyquist row evolves


def test_golden_diagnostics_vs_oracle(case):
    """Scalar diagnostics (padded dealiased flux) and spectra (rfft weights
    with the ky = Nx/2 column) on full-band states against the oracle."""
    name, meta, arrays, g, o = case
    for label in ("r", "s0"):
        st = fixtures.state_from(arrays, label)
        got = compute_diagnostics(st, g)
        ref = oracle.compute_diagnostics(OracleState(*st), o)
        for key in DIAG_KEYS:
            tol = 1e-13 if key == "heat_flux_mismatch" else 1e-12 * abs(ref[key])
            assert abs(got[key] - ref[key]) <= tol + 1e-300, (name, label, key)
        gs, os_ = spectra(st, g), oracle.spectra(OracleState(*st), o)
        for key in ("E_bt", "E_tot", "q", "w", "th", "psi_ke"):
            scale = max(float(np.max(np.abs(os_[key]))), 1e-300)
            assert float(np.max(np.abs(gs[key] - os_[key]))) <= 1e-11 * scale, (name, label, key)


# ---------------------------------------------------------------- longer runs
RECIPES = {
    "production": dict(thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
                       sbp_corrector_substeps=4, nonlinear_advection="flux"),
    "jacobian": dict(thermal_closure="fixed_conduction", nonlinear_advection="jacobian"),
    "legacy": dict(thermal_closure="evolve_mean", mean_exchange_discretization="legacy",
                   nonlinear_advection="flux"),
}


@pytest.mark.parametrize("recipe", sorted(RECIPES))
def test_40_steps_vs_oracle(recipe):
    cfg = dict(Nx=32, Nz=16, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, float_dtype="float64",
               horizontal_dealiasing="32_rule", **RECIPES[recipe])
    g = make_grid(NHQGConfig(**cfg))
    o = oracle.make_grid(OracleConfig(**cfg))
    s0 = theta_perturbation_state(g, seed=4)
    os_ = OracleState(*s0)
    for _ in range(40):
        os_ = oracle.imex_step(os_, o)
    s = S.to_device(s0)
    S.step_inplace(s, g, 40, check=True)
    assert_state_close(_host(s), os_, 1e-9, th_bar_abs=1e-18)


@pytest.mark.parametrize("nx,nz", [(32, 16), (64, 32)])
def test_mixed_step_vs_plain(nx, nz):
    """The mixed-precision step on the 3/2-rule grid (FP32 padded products,
    tensor-core vertical transforms) within 1e-6 of the plain FP64 step."""
    cfg = dict(Nx=nx, Nz=nz, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, float_dtype="float64",
               horizontal_dealiasing="32_rule", **RECIPES["production"])
    g = make_grid(NHQGConfig(**cfg))
    s0 = S.sanitize_state(theta_perturbation_state(g, seed=6), g)
    plain = _host(S.imex_step(s0, g))
    mixed = _host(S.imex_step(s0, g, precision="mixed"))
    assert_state_close(mixed, plain, 1e-6, th_bar_abs=1e-14)
    e64 = _host(S.explicit_rhs(s0, g))
    e32 = _host(S.explicit_rhs(s0, g, precision="mixed"))
    assert_state_close(e32, e64, 2e-5, th_bar_abs=1e-14)


def test_rule_mismatch_is_refused():
    """A 3/2-rule context refuses the 2/3 plane call (NHQG_ERR_UNSUPPORTED)
    and runs the 3/2 one."""
    from nhqg_gb300.engine import engine_for

    g = make_grid(NHQGConfig(Nx=16, Nz=6, L=10.0, float_dtype="float64", horizontal_dealiasing="32_rule"))
    e = engine_for(g)
    z = torch.zeros((2, 16, 9), dtype=torch.complex128, device="cuda")
    ptrs = [t.data_ptr() for t in (z, z, z, z, torch.empty_like(z), torch.empty_like(z), torch.empty_like(z))]
    assert e.lib.nhqg_triple_advection_23(e.handle, 0, 2, *ptrs, None) == 2
    assert e.lib.nhqg_triple_advection_32(e.handle, 0, 2, *ptrs, None) == 0
    torch.cuda.synchronize()
