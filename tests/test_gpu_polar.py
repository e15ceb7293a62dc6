"""Polar-trap configuration at its benchmark size against the CPU oracle.

256^2 x 32, L = 24 L_c, Ra = 100, dt = 5e-5, radial background-PV trap
gamma = 2.2e-3 (nhqg/grid.py:605-631) with the Rayleigh sponge outside the
trap (nhqg/grid.py:633-667, nhqg/solver.py:591-597), Neumann w at the top
(nhqg/grid.py:322-342), evolve_mean with the balanced SBP2 predictor /
corrector and 4 substeps.  The trap radius and sponge parameters are the
production-scaled values (trap_r_star = 0.4 L, trap_sharpness 20,
sponge_rate 50, sponge_r_start 52, sponge_sharpness 30): the default trap
radius fails the reference's own eta resolution guard at this size.

Gates (relative L2 per field): per-RHS operators <= 1e-12 on a strongly
nonlinear band-limited state; 10 plain steps from the seeded theta' start
<= 1e-9; the mixed-precision step <= 1e-6.
"""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle
from oracle.nhqg_oracle import OracleConfig, OracleState
from _util import assert_state_close

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402

L_C = 2.0 * math.pi / 1.3048
L2 = 24 * L_C
CFG2 = dict(Nx=256, Nz=32, L=L2, Ra_tilde=100.0, sigma=1.0, nu_q=1.0, nu_w=1.0, nu_theta=1.0,
            hyper_order=1, dt=5e-5, nonlinear_advection="flux", horizontal_dealiasing="23_rule",
            float_dtype="float64", gamma=2.2e-3, w_bc_top="neumann", trap_r_star=0.4 * L2,
            trap_sharpness=20.0, sponge_rate=50.0, sponge_r_start=52.0, sponge_sharpness=30.0,
            thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
            sbp_corrector_substeps=4)


def _host(state):
    return tuple(t.detach().cpu().numpy() for t in state)


@pytest.fixture(scope="module")
def grids():
    g = make_grid(NHQGConfig(**CFG2))
    o = oracle.make_grid(OracleConfig(**CFG2))
    assert g.eta_hat is not None and g.sponge_phys is not None
    return g, o


def _rich_state(o, seed):
    """Band-limited random state with O(1) nonlinearity (zero horizontal mean)."""
    rng = np.random.default_rng(seed)
    P, G, Nx, Nk = o.Nz + 1, o.Nz - 1, o.Nx, o.Nx // 2 + 1
    ksq = np.asarray(o.ksq)
    env = np.exp(-ksq / (2.0 * float(np.max(ksq)) / 9.0))

    def field(n):
        z = rng.standard_normal((n, Nx, Nk)) + 1j * rng.standard_normal((n, Nx, Nk))
        return 0.3 * z * env[None] / (1.0 + np.arange(n))[:, None, None]

    s = oracle.sanitize_state(OracleState(field(P), field(G), field(G), np.zeros(P)), o)
    q, w, th = (oracle.nhqg_oracle.zero_mean(f) for f in s[:3])
    return OracleState(q, w, th, s.th_bar)


def test_polar_operators(grids):
    g, o = grids
    r = _rich_state(o, 11)
    base_o = o.replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    base_g = g._replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    E_ref = oracle.explicit_rhs(r, base_o)
    assert_state_close(_host(S.explicit_rhs(r, base_g)), E_ref, 1e-12, th_bar_abs=1e-15)
    I_ref = oracle.implicit_tendency(r, base_o)
    assert_state_close(_host(S.implicit_tendency(r, base_g)), I_ref, 1e-12, th_bar_abs=1e-15)
    sol_ref = oracle.imex_implicit_solve(r.q_hat, r.w_hat, r.th_hat, base_o)
    sol = S.imex_implicit_solve(r.q_hat, r.w_hat, r.th_hat, base_g)
    assert_state_close(_host(sol), sol_ref, 1e-12, names=("q_hat", "w_hat", "th_hat"))


def test_polar_10_steps(grids):
    g, o = grids
    s0 = theta_perturbation_state(g, seed=0)
    ref = OracleState(*s0)
    for _ in range(10):
        ref = oracle.imex_step(ref, o)
    s = S.to_device(s0)
    S.step_inplace(s, g, 10, check=True)
    assert_state_close(_host(s), ref, 1e-9, th_bar_abs=1e-18)
    m = S.to_device(s0)
    S.step_inplace(m, g, 10, check=True, precision="mixed")
    assert_state_close(_host(m), ref, 1e-6, th_bar_abs=1e-18)
