"""GPU parity: the CUDA engine against the reference's golden vectors and the
CPU oracle, through the C ABI (nhqg_gb300.engine -> libnhqg_gpu.so).

Tolerances (relative L2 per field): 1e-12 for one operator evaluation or one
stage, 1e-11 for 1..5 steps of the golden cases, 1e-9 after 100 steps of the
64^2 x 32 benchmark configuration.  th_bar is compared with an absolute
floor where the reference keeps it at exact zero.
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

L_C = 2.0 * np.pi / 1.3048


def _host(state):
    return tuple(t.detach().cpu().numpy() for t in state)


# ---------------------------------------------------------------- spectral
def _box(Nx, L=2 * np.pi):
    kx = (2 * np.pi * np.fft.fftfreq(Nx, d=L / Nx))[:, None]
    ky = (2 * np.pi * np.arange(Nx // 2 + 1) / L)[None, :]
    K = Nx // 3
    ii = np.arange(Nx)
    kint = np.where(ii <= Nx // 2, ii, ii - Nx)
    mask = ((np.abs(kint)[:, None] <= K) & (np.arange(Nx // 2 + 1)[None] <= K)).astype(float)
    x = np.linspace(0, L, Nx, endpoint=False)
    X, Y = np.meshgrid(x, x, indexing="ij")
    return kx, ky, mask, X, Y


@pytest.mark.parametrize("form", ["flux", "jacobian"])
def test_jacobian_analytic(form):
    """J[sin x, sin y] = cos x cos y; J[sin 2x, sin 3y] = 6 cos 2x cos 3y
    (reference tests/test_spectral.py:40-62)."""
    Nx = 64
    kx, ky, mask, X, Y = _box(Nx)
    fn = SP.triple_conservative_flux_divergence_23 if form == "flux" else SP.triple_jacobian_23
    for a, b, exact, tol in ((np.sin(X), np.sin(Y), np.cos(X) * np.cos(Y), 1e-12),
                             (np.sin(2 * X), np.sin(3 * Y), 6 * np.cos(2 * X) * np.cos(3 * Y), 1e-11)):
        A = np.fft.rfft2(a)[None]
        B = np.fft.rfft2(b)[None]
        J = fn(A, B, B, B, kx, ky, mask, Nx)[0].cpu().numpy()[0]
        np.testing.assert_allclose(np.fft.irfft2(J, s=(Nx, Nx)), exact, atol=tol)


@pytest.mark.parametrize("Nx", [16, 24, 32, 48, 64, 96, 128, 256])
@pytest.mark.parametrize("form", ["flux", "jacobian"])
def test_triple_products_random(Nx, form):
    """Full-band random inputs (incl. ky=0 / Nyquist imaginary parts that
    irfft2 ignores) against the oracle's NumPy restatement."""
    rng = np.random.default_rng(Nx)
    kx, ky, mask, _, _ = _box(Nx, L=37.0)
    levels = 3
    shp = (levels, Nx, Nx // 2 + 1)
    f = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(4)]
    ofn = oracle.triple_conservative_flux_divergence_23 if form == "flux" else oracle.triple_jacobian_23
    gfn = SP.triple_conservative_flux_divergence_23 if form == "flux" else SP.triple_jacobian_23
    ref = ofn(*f, kx, ky, mask, Nx)
    got = gfn(*f, kx, ky, mask, Nx)
    for g, r in zip(got, ref):
        assert rel_l2(g.cpu().numpy(), r) <= 1e-13


def test_sponge_product():
    Nx = 48
    rng = np.random.default_rng(3)
    _, _, mask, X, Y = _box(Nx)
    sigma = 2.0 + np.cos(X) * np.sin(2 * Y)
    f = rng.standard_normal((4, Nx, Nx // 2 + 1)) + 1j * rng.standard_normal((4, Nx, Nx // 2 + 1))
    ref = oracle.sponge_product_23(f, sigma, mask, Nx)
    got = SP.sponge_product_23(f, sigma, mask, Nx).cpu().numpy()
    assert rel_l2(got, ref) <= 1e-13


# ---------------------------------------------------------------- golden cases
def _grids(meta, arrays):
    cfg = dict(meta["cfg"])
    g = make_grid(NHQGConfig(**cfg))
    o = oracle.make_grid(OracleConfig(**cfg))
    if meta.get("override_eta_sponge"):
        eta = arrays["grid.eta_hat"][0]
        sp = arrays["grid.sponge_phys"]
        g = g._replace(eta_hat=eta, sponge_phys=sp, eta_phys=np.fft.irfft2(eta, s=(g.Nx, g.Nx)))
        o = o.replace(eta_hat=eta, sponge_phys=sp)
    return g, o


@pytest.fixture(scope="module", params=fixtures.CASES)
def case(request):
    meta, arrays = fixtures.load_case(request.param)
    g, o = _grids(meta, arrays)
    return request.param, meta, arrays, g, o


def _base(grid, meta):
    if meta["split"]:
        return grid._replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    return grid


def test_golden_explicit_rhs(case):
    name, meta, arrays, g, o = case
    E = S.explicit_rhs(fixtures.state_from(arrays, "r"), _base(g, meta))
    assert_state_close(_host(E), fixtures.state_from(arrays, "E"), 1e-12, th_bar_abs=1e-14)


def test_golden_implicit_tendency(case):
    name, meta, arrays, g, o = case
    I = S.implicit_tendency(fixtures.state_from(arrays, "r"), _base(g, meta))
    assert_state_close(_host(I), fixtures.state_from(arrays, "I"), 1e-12, th_bar_abs=1e-12)


def test_golden_implicit_solve(case):
    name, meta, arrays, g, o = case
    r = fixtures.state_from(arrays, "r")
    base = _base(g, meta)
    q, w, th = S.imex_implicit_solve(r[0], r[1], r[2], base)
    tb = S.imex_mean_temp_solve(r[3], base)
    assert_state_close(_host((q, w, th, tb)), fixtures.state_from(arrays, "solve"), 1e-12,
                       th_bar_abs=1e-13)


def test_golden_corrector(case):
    name, meta, arrays, g, o = case
    if not meta["split"]:
        pytest.skip("recipe without the SBP2 corrector")
    out = S.apply_balanced_sbp2_corrector(fixtures.state_from(arrays, "r"), g, g.gamma_imex * g.dt)
    assert_state_close(_host(out), fixtures.state_from(arrays, "corr"), 1e-12, th_bar_abs=1e-14)


def test_golden_steps(case):
    name, meta, arrays, g, o = case
    s = S.imex_step(fixtures.state_from(arrays, "r"), g)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r1"), 1e-12, th_bar_abs=1e-14)
    S.step_inplace(s, g, 4, check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r5"), 1e-11, th_bar_abs=1e-13)


def test_golden_seeded_trajectory(case):
    name, meta, arrays, g, o = case
    s = S.to_device(fixtures.state_from(arrays, "s0"))
    S.step_inplace(s, g, meta["n_steps"], check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "sN"), 1e-11, th_bar_abs=1e-16)


# ---------------------------------------------------------------- 64^2 x 32 production recipe
CFG_64X32 = dict(Nx=64, Nz=32, L=10 * L_C, Ra_tilde=100.0, sigma=1.0, nu_q=1.0, nu_w=1.0, nu_theta=1.0,
            hyper_order=1, dt=5e-5, nonlinear_advection="flux", horizontal_dealiasing="23_rule",
            float_dtype="float64")


@pytest.mark.parametrize("recipe", [
    dict(thermal_closure="fixed_conduction"),
    dict(thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
         sbp_corrector_substeps=4),
])
def test_64x32_production_100_steps(recipe):
    """64^2 x 32, 100 steps: per-RHS <= 1e-12, 100-step <= 1e-9 vs the oracle."""
    cfgd = dict(CFG_64X32, **recipe)
    g = make_grid(NHQGConfig(**cfgd))
    o = oracle.make_grid(OracleConfig(**cfgd))
    s0 = theta_perturbation_state(g, seed=0)
    base_o = o.replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    base_g = g._replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    E_ref = oracle.explicit_rhs(OracleState(*s0), base_o)
    E_got = _host(S.explicit_rhs(s0, base_g))
    assert_state_close(E_got, E_ref, 1e-12, th_bar_abs=1e-15)
    os_ = OracleState(*s0)
    for _ in range(100):
        os_ = oracle.imex_step(os_, o)
    s = S.to_device(s0)
    S.step_inplace(s, g, 100, check=True)
    assert_state_close(_host(s), os_, 1e-9, th_bar_abs=1e-18)


def test_make_initial_state_reference_regression():
    """make_initial_state with JAX's PRNG stream, then 20 GPU steps, against
    the reference's own bitwise regression data
    (tests/test_mixed_bc_plumbing.py:99-117)."""
    meta, arrays = fixtures.load_case("jaxprng_m2b")
    g = make_grid(NHQGConfig(**dict(meta["cfg"])))
    s = S.make_initial_state(g, seed=meta["seed"], amplitude=meta["amplitude"])
    S.step_inplace(s, g, meta["n_steps"], check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "sN"), 1e-12, th_bar_abs=1e-18)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_imex_step_many_matches_imex_step(precision):
    """The pipelined host-state stepping (copies on two streams overlapped with
    the steps, three device states in rotation) returns exactly what
    imex_step returns for each input; six inputs reuse every device state."""
    meta, arrays = fixtures.load_case("prod16")
    g = make_grid(NHQGConfig(**dict(meta["cfg"])))
    ins = []
    for label in ("r", "s0", "r1", "r5"):
        st = fixtures.state_from(arrays, label)
        ins.append(tuple(torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in st))
    ins += ins[:2]
    got = S.imex_step_many(ins, g, precision=precision)
    assert len(got) == len(ins)
    for inp, res in zip(ins, got):
        ref = _host(S.imex_step(inp, g, precision=precision))
        for a, b in zip(res, ref):
            np.testing.assert_array_equal(a.numpy(), b)
