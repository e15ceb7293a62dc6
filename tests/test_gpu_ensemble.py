"""GPU tests of the batched ensemble (one CUDA graph advancing independent
contexts): every member must reproduce its own single-context run bitwise
with the same tiles, match the reference goldens with autotuned tiles, and
follow a precision change of one member."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fixtures
from _util import assert_state_close

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402
from nhqg_gb300.engine import Engine  # noqa: E402
from nhqg_gb300.ensemble import Ensemble  # noqa: E402

MEMBERS = [("prod16", "fp64"), ("radix24", "fp64"), ("polar16", "fp64"), ("jac16", "fp64"),
           ("prod16", "mixed"), ("polar16", "mixed")]


def _case(name):
    meta, arrays = fixtures.load_case(name)
    g = make_grid(NHQGConfig(**dict(meta["cfg"])))
    if meta.get("override_eta_sponge"):
        eta = arrays["grid.eta_hat"][0]
        g = g._replace(eta_hat=eta, sponge_phys=arrays["grid.sponge_phys"],
                       eta_phys=np.fft.irfft2(eta, s=(g.Nx, g.Nx)))
    return g, arrays


def _host(s):
    return tuple(t.detach().cpu().numpy() for t in s)


def _single(g, state, n, precision):
    eng = Engine(g)
    s = S.to_device(state)
    s = S.State(*(t.clone() for t in s))
    eng.step(*s, n_steps=n, precision=precision)
    return _host(s)


def test_ensemble_matches_single_runs_bitwise():
    cases = [_case(n) for n, _ in MEMBERS]
    ens = Ensemble([g for g, _ in cases], precision=[p for _, p in MEMBERS],
                   steps_per_launch=3, autotune=False)
    for i, (g, arrays) in enumerate(cases):
        ens.load(i, fixtures.state_from(arrays, "r"))
    ens.step(7)  # two 3-step graph launches + one 1-step launch
    for i, ((g, arrays), (name, prec)) in enumerate(zip(cases, MEMBERS)):
        got = _host(ens.store(i))
        ref = _single(g, fixtures.state_from(arrays, "r"), 7, prec)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (name, prec)
    ens.close()


def test_ensemble_autotuned_matches_golden():
    names = ["prod16", "radix24", "polar16", "fixed16"]
    cases = [_case(n) for n in names]
    ens = Ensemble([g for g, _ in cases], steps_per_launch=5, autotune=True)
    for i, (g, arrays) in enumerate(cases):
        ens.load(i, fixtures.state_from(arrays, "r"))
    ens.step(5)
    for i, (g, arrays) in enumerate(cases):
        assert_state_close(_host(ens.store(i)), fixtures.state_from(arrays, "r5"), 1e-11,
                           th_bar_abs=1e-13)
    ens.close()


def test_ensemble_recaptures_on_precision_change():
    g, arrays = _case("prod16")
    g2, arrays2 = _case("radix24")
    ens = Ensemble([g, g2], steps_per_launch=2, autotune=False)
    ens.load(0, fixtures.state_from(arrays, "r"))
    ens.load(1, fixtures.state_from(arrays2, "r"))
    ens.step(2)
    ens.engines[0].set_precision("mixed")
    ens.step(2)
    s0 = _host(ens.store(0))
    eng = Engine(g)
    s = S.State(*(t.clone() for t in S.to_device(fixtures.state_from(arrays, "r"))))
    eng.step(*s, n_steps=2)
    eng.step(*s, n_steps=2, precision="mixed")
    for a, b in zip(s0, _host(s)):
        assert np.array_equal(a, b)
    ens.close()


def test_ensemble_48_members_size_classes():
    """One member per size class of the 48-instance benchmark ensemble
    (64^2x32, 96^2x48 with radix-3 transforms, 128^2x64; L = 10 L_c,
    dt = 5e-5, Ra ~ U(40, 120), production recipe), each in FP64 and mixed
    precision: 20 ensemble steps equal every member's own single-context
    run bitwise, and the FP64 members match the oracle to 1e-11 after 5
    steps."""
    import sys
    from pathlib import Path

    import oracle
    from oracle.nhqg_oracle import OracleConfig, OracleState
    from nhqg_gb300 import theta_perturbation_state

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench

    cfgs = bench.ensemble_configs()
    picks = [cfgs[0], cfgs[16], cfgs[32]]  # first member of each class
    grids = [make_grid(NHQGConfig(**c)) for c in picks]
    members = [(i, p) for i in range(3) for p in ("fp64", "mixed")]
    ens = Ensemble([grids[i] for i, _ in members], precision=[p for _, p in members],
                   steps_per_launch=10, autotune=False)
    starts = [theta_perturbation_state(grids[i], seed=7 + i, amplitude=0.1) for i in range(3)]
    for j, (i, _) in enumerate(members):
        ens.load(j, starts[i])
    ens.step(20)
    for j, (i, prec) in enumerate(members):
        got = _host(ens.store(j))
        ref = _single(grids[i], starts[i], 20, prec)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), (picks[i]["Nx"], prec)
    ens.close()
    for i, c in enumerate(picks):
        o = oracle.make_grid(OracleConfig(**c))
        os_ = OracleState(*starts[i])
        for _ in range(5):
            os_ = oracle.imex_step(os_, o)
        assert_state_close(_single(grids[i], starts[i], 5, "fp64"), os_, 1e-11, th_bar_abs=1e-18)
