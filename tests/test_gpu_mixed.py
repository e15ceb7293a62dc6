"""GPU tests of the mixed-precision path against the plain FP64 path, the
reference's golden vectors and the CPU oracle.

The mixed path runs the 2/3-rule products and the Chebyshev <-> nodal
transforms around them in FP32; the Galerkin stencils, stage combinations,
the implicit w solve (an O(Nz) Chebyshev-tau recurrence) and the SBP2 mean
exchange stay FP64.  Tolerances (relative L2 per field):
- implicit solve, tau recurrence vs the reference's dense shell inverse (both
  FP64): 1e-10 at Nz <= 12, 1e-8 at Nz = 256, where the dense table itself
  carries ~1e-9 of rounding;
- explicit RHS: 2e-5 (FP32 products, about 300 FP32 ulps);
- one step: 1e-6, the accuracy target of the mixed path, and the FP32 error
  of the step increment itself below 1e-4;
- 100 steps of the 64^2 x 32 benchmark configuration: 1e-6 against the
  oracle's FP64 trajectory.
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
from nhqg_gb300._native import NativeError  # noqa: E402

L_C = 2.0 * np.pi / 1.3048
MIXED_CASES = ("prod16", "jac16", "polar16", "radix24")  # 2*Nz = 2^a 3^b, no legacy evolve_mean


def _host(state):
    return tuple(t.detach().cpu().numpy() for t in state)


def _grids(meta, arrays):
    cfg = dict(meta["cfg"])
    g = make_grid(NHQGConfig(**cfg))
    if meta.get("override_eta_sponge"):
        eta = arrays["grid.eta_hat"][0]
        g = g._replace(eta_hat=eta, sponge_phys=arrays["grid.sponge_phys"],
                       eta_phys=np.fft.irfft2(eta, s=(g.Nx, g.Nx)))
    return g


def _base(grid, meta):
    if meta["split"]:
        return grid._replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    return grid


@pytest.fixture(scope="module", params=MIXED_CASES)
def case(request):
    meta, arrays = fixtures.load_case(request.param)
    return request.param, meta, arrays, _grids(meta, arrays)


def test_tau_solve_matches_reference(case):
    """The O(Nz) tau recurrence reproduces the reference's dense per-shell
    solve (golden 'solve' vectors, nhqg/solver.py:691-738)."""
    name, meta, arrays, g = case
    r = fixtures.state_from(arrays, "r")
    base = _base(g, meta)
    q, w, th = S.imex_implicit_solve(r[0], r[1], r[2], base, precision="mixed")
    ref = fixtures.state_from(arrays, "solve")
    assert_state_close(_host((q, w, th)), ref[:3], 1e-10, names=("q_hat", "w_hat", "th_hat"))
    qd, wd, thd = S.imex_implicit_solve(r[0], r[1], r[2], base)
    assert rel_l2(w.cpu().numpy(), wd.cpu().numpy()) <= 1e-10


def test_explicit_rhs_fp32_products(case):
    name, meta, arrays, g = case
    r = fixtures.state_from(arrays, "r")
    base = _base(g, meta)
    E64 = _host(S.explicit_rhs(r, base))
    E32 = _host(S.explicit_rhs(r, base, precision="mixed"))
    assert_state_close(E32, fixtures.state_from(arrays, "E"), 2e-5, th_bar_abs=1e-14)
    assert_state_close(E32, E64, 2e-5, th_bar_abs=1e-14)


def test_one_step_and_increment(case):
    name, meta, arrays, g = case
    r = fixtures.state_from(arrays, "r")
    s64 = _host(S.imex_step(r, g))
    s32 = _host(S.imex_step(r, g, precision="mixed"))
    assert_state_close(s32, fixtures.state_from(arrays, "r1"), 1e-6, th_bar_abs=1e-14)
    assert_state_close(s32, s64, 1e-6, th_bar_abs=1e-14)
    # the step increment carries the FP32 error directly
    inc64 = [a - b for a, b in zip(s64[:3], r[:3])]
    inc32 = [a - b for a, b in zip(s32[:3], r[:3])]
    for f, (a, b) in enumerate(zip(inc32, inc64)):
        assert rel_l2(a, b) <= 1e-4, (name, f, rel_l2(a, b))


def test_mixed_then_plain_is_plain(case):
    """Switching back to FP64 restores the plain path exactly."""
    name, meta, arrays, g = case
    r = fixtures.state_from(arrays, "r")
    S.imex_step(r, g, precision="mixed")
    s = S.imex_step(r, g)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r1"), 1e-12, th_bar_abs=1e-14)


@pytest.mark.parametrize("name", ["legacy16", "fixed16"])
def test_unsupported_configs_raise(name):
    """Legacy evolve_mean (nodal exchange product) and Nz with 2*Nz outside
    2^a 3^b (dense transforms) have no mixed path: the call fails loudly."""
    meta, arrays = fixtures.load_case(name)
    g = _grids(meta, arrays)
    with pytest.raises(NativeError):
        S.imex_step(fixtures.state_from(arrays, "r"), g, precision="mixed")


def test_tau_solve_nz256():
    """At Nz = 256 the tau recurrence and the dense table differ by the
    table's rounding only."""
    cfg = dict(Nx=24, Nz=256, L=10 * L_C, Ra_tilde=100.0, dt=2e-5, nonlinear_advection="flux",
               horizontal_dealiasing="23_rule", float_dtype="float64",
               thermal_closure="fixed_conduction")
    g = make_grid(NHQGConfig(**cfg))
    rng = np.random.default_rng(3)
    s = S.sanitize_state(theta_perturbation_state(g, seed=1), g)
    Rq = s.q_hat + 1e-3 * torch.from_numpy(rng.standard_normal(s.q_hat.shape)).cuda()
    Rw = s.w_hat + 1e-3 * torch.from_numpy(rng.standard_normal(s.w_hat.shape)).cuda()
    src = S.sanitize_state((Rq, Rw, s.th_hat, s.th_bar), g)
    d = S.imex_implicit_solve(src.q_hat, src.w_hat, src.th_hat, g)
    t = S.imex_implicit_solve(src.q_hat, src.w_hat, src.th_hat, g, precision="mixed")
    for a, b in zip(t, d):
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) <= 1e-8


CFG_64X32 = dict(Nx=64, Nz=32, L=10 * L_C, Ra_tilde=100.0, sigma=1.0, nu_q=1.0, nu_w=1.0, nu_theta=1.0,
            hyper_order=1, dt=5e-5, nonlinear_advection="flux", horizontal_dealiasing="23_rule",
            float_dtype="float64", thermal_closure="evolve_mean",
            mean_exchange_discretization="balanced_sbp2_pc", sbp_corrector_substeps=4)


def test_64x32_100_steps_mixed():
    """64^2 x 32 production recipe, 100 mixed steps vs the FP64 oracle."""
    g = make_grid(NHQGConfig(**CFG_64X32))
    o = oracle.make_grid(OracleConfig(**CFG_64X32))
    s0 = theta_perturbation_state(g, seed=0)
    os_ = OracleState(*s0)
    for _ in range(100):
        os_ = oracle.imex_step(os_, o)
    s = S.to_device(s0)
    S.step_inplace(s, g, 100, check=True, precision="mixed")
    assert_state_close(_host(s), os_, 1e-6, th_bar_abs=1e-18)


@pytest.mark.parametrize("nx", [64, 128, 256])
def test_explicit_rhs_fp32_row_products_sizes(nx):
    """The FP32 row products at power-of-two row lengths (radix-4 and mixed
    radix-4/2 plans): mixed explicit RHS against the plain one on a random
    state whose spectrum fills the 2/3-rule band."""
    cfg = dict(Nx=nx, Nz=16, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, nonlinear_advection="flux",
               horizontal_dealiasing="23_rule", float_dtype="float64", thermal_closure="fixed_conduction")
    g = make_grid(NHQGConfig(**cfg))
    rng = np.random.default_rng(nx)
    P, G, Nk = g.Nz + 1, g.Nz - 1, g.Nk
    env = np.exp(-np.asarray(g.ksq) / (2.0 * float(np.max(g.ksq)) / 9.0))
    fld = lambda n: 0.3 * (rng.standard_normal((n, nx, Nk)) + 1j * rng.standard_normal((n, nx, Nk))) * env[None]  # noqa: E731
    s = S.sanitize_state((fld(P), fld(G), fld(G), np.zeros(P)), g)
    E64 = _host(S.explicit_rhs(s, g))
    E32 = _host(S.explicit_rhs(s, g, precision="mixed"))
    assert_state_close(E32, E64, 2e-5, th_bar_abs=1e-14)


def _bf16(a):
    """Round float64 values to bfloat16 (round to nearest even on the top 16
    bits of the float32 pattern)."""
    f = np.asarray(a, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def test_64x32_convecting_state_100_steps_mixed(monkeypatch):
    """64^2 x 32 production recipe from a convecting state (seeded theta'
    of amplitude 1, 4000 mixed steps: t = 0.2, Nu - 1 ~ 4), where the
    advection term is O(1) of the tendency: 100 mixed steps within 1e-6 of
    the oracle's FP64 trajectory, 100 plain steps within 1e-9.  The same 100
    oracle steps with the product factors rounded to BF16 leave the 1e-6
    band, so the gate sees the precision of the products."""
    from nhqg_gb300.diagnostics import compute_diagnostics
    g = make_grid(NHQGConfig(**CFG_64X32))
    s0 = S.to_device(theta_perturbation_state(g, seed=0, amplitude=1.0))
    S.step_inplace(s0, g, 4000, check=True, precision="mixed")
    d = compute_diagnostics(s0, g)
    assert d["Nusselt"] - 1.0 >= 0.1, d["Nusselt"]
    E = S.explicit_rhs(s0, g)
    I = S.implicit_tendency(s0, g)  # noqa: E741
    share = float(torch.linalg.norm(E.th_hat) / torch.linalg.norm(I.th_hat))
    assert share > 0.05, share  # the nonlinear term is a visible part of the theta tendency
    host = S.to_host(s0)
    o = oracle.make_grid(OracleConfig(**CFG_64X32))
    ref = OracleState(*host)
    for _ in range(100):
        ref = oracle.imex_step(ref, o)
    mix = S.State(*(t.clone() for t in s0))
    S.step_inplace(mix, g, 100, check=True, precision="mixed")
    assert_state_close(_host(mix), ref, 1e-6, th_bar_abs=1e-18)
    plain = S.State(*(t.clone() for t in s0))
    S.step_inplace(plain, g, 100, check=True)
    assert_state_close(_host(plain), ref, 1e-9, th_bar_abs=1e-18)
    monkeypatch.setattr(oracle.nhqg_oracle, "PRODUCT_ROUNDING", _bf16)
    bad = OracleState(*host)
    for _ in range(100):
        bad = oracle.imex_step(bad, o)
    worst = max(rel_l2(b, r) for b, r in zip(bad[:3], ref[:3]))
    assert worst > 1e-6, worst
