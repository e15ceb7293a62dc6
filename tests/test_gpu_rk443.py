"""GPU parity of the ARS(4,4,3) stepper (imex_scheme='rk443',
nhqg/solver.py:1056-1122) through the C ABI against the reference's golden
vectors (tests/golden/rk443*.npz, made by tests/golden/make_golden.py --rk443)
and the CPU oracle.

The reference runs RK443 with the legacy exchange only (fixed conduction, or
the legacy explicit evolve_mean closure); gamma = 1/2 enters the shell
tables.  Tolerances (relative L2 per field) as for ARS222: 1e-12 for one
operator or one step, 1e-11 for 5 and 10 steps, 1e-9 after 40 steps against
the oracle.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fixtures
import oracle
from oracle.nhqg_oracle import OracleConfig, OracleState
from _util import assert_state_close

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402
from nhqg_gb300._native import NativeError  # noqa: E402

L_C = 2.0 * np.pi / 1.3048


def _host(state):
    return tuple(t.detach().cpu().numpy() for t in state)


@pytest.fixture(scope="module", params=fixtures.RK_CASES)
def case(request):
    meta, arrays = fixtures.load_case(request.param)
    return request.param, meta, arrays, make_grid(NHQGConfig(**dict(meta["cfg"])))


def test_grid_gamma(case):
    name, meta, arrays, g = case
    assert g.imex_scheme == "rk443" and g.gamma_imex == 0.5


def test_operators(case):
    """E, I and the gamma = 1/2 implicit solve against the reference."""
    name, meta, arrays, g = case
    r = fixtures.state_from(arrays, "r")
    assert_state_close(_host(S.explicit_rhs(r, g)), fixtures.state_from(arrays, "E"), 1e-12,
                       th_bar_abs=1e-14)
    assert_state_close(_host(S.implicit_tendency(r, g)), fixtures.state_from(arrays, "I"), 1e-12,
                       th_bar_abs=1e-12)
    q, w, th = S.imex_implicit_solve(r[0], r[1], r[2], g)
    ref = fixtures.state_from(arrays, "solve")
    assert_state_close(_host((q, w, th)), ref[:3], 1e-12, names=("q_hat", "w_hat", "th_hat"))


def test_steps(case):
    name, meta, arrays, g = case
    s = S.imex_step(fixtures.state_from(arrays, "r"), g)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r1"), 1e-12, th_bar_abs=1e-14)
    s = S.to_device(fixtures.state_from(arrays, "r"))
    S.step_inplace(s, g, 5, check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "r5"), 1e-11, th_bar_abs=1e-13)
    s = S.to_device(fixtures.state_from(arrays, "s0"))
    S.step_inplace(s, g, meta["n_steps"], check=True)
    assert_state_close(_host(s), fixtures.state_from(arrays, "sN"), 1e-11, th_bar_abs=1e-16)


@pytest.mark.parametrize("closure", ["fixed_conduction", "evolve_mean"])
def test_40_steps_vs_oracle(closure):
    cfg = dict(Nx=32, Nz=16, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, nonlinear_advection="flux",
               horizontal_dealiasing="23_rule", float_dtype="float64", imex_scheme="rk443",
               thermal_closure=closure, mean_exchange_discretization="legacy")
    g = make_grid(NHQGConfig(**cfg))
    o = oracle.make_grid(OracleConfig(**cfg))
    s0 = theta_perturbation_state(g, seed=2)
    os_ = OracleState(*s0)
    for _ in range(40):
        os_ = oracle.imex_step(os_, o)
    s = S.to_device(s0)
    S.step_inplace(s, g, 40, check=True)
    assert_state_close(_host(s), os_, 1e-9, th_bar_abs=1e-18)


def test_mixed_precision_refused(case):
    """RK443 runs in FP64: a mixed-precision step fails loudly."""
    name, meta, arrays, g = case
    s = S.to_device(fixtures.state_from(arrays, "r"))
    with pytest.raises(NativeError):
        S.step_inplace(s, g, 1, precision="mixed")
