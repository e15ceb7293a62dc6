"""GPU tests of the tensor-core vertical transforms of the mixed path
(tcgen05 kind::tf32, TF32 hi/lo split operands, FP32 accumulation).

_to_nodal / _to_coeffs (nhqg/solver.py:45-52) are dense products with the
grid's V and V^-1 (nhqg/grid.py:192-201); the forward transforms of w and
theta include the Galerkin stencil (nhqg/solver.py:65-72).  The references
here are the same products in FP64 on the host.  Tolerance 3e-6 relative L2
per column: the split keeps 22 bits per operand (an exact-FP32 emulation of
the same products gives 7e-8), but the tensor core's FP32 accumulation is
coarser than round-to-nearest: 1.06e-6 measured at Nz = 256.  The column counts 2M are not multiples of the
128-column CTA tile, so the partial last tile is covered.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402
from nhqg_gb300._native import NativeError  # noqa: E402
from nhqg_gb300.engine import engine_for  # noqa: E402
from _util import assert_state_close, rel_l2  # noqa: E402

L_C = 2.0 * np.pi / 1.3048
SIZES = [(32, 16), (64, 32), (48, 48), (64, 256)]


def _grid(nx, nz, **kw):
    cfg = dict(Nx=nx, Nz=nz, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, nonlinear_advection="flux",
               horizontal_dealiasing="23_rule", float_dtype="float64", thermal_closure="evolve_mean",
               mean_exchange_discretization="balanced_sbp2_pc", sbp_corrector_substeps=4)
    cfg.update(kw)
    return make_grid(NHQGConfig(**cfg))


def _stencils(g):
    P, G = g.Nz + 1, g.Nz - 1
    sd = np.zeros((P, G))
    sd[np.arange(G), np.arange(G)] = -1.0
    sd[np.arange(G) + 2, np.arange(G)] = 1.0
    return np.asarray(g.w_stencil), sd


@pytest.mark.parametrize("nx,nz", SIZES)
def test_to_nodal_matches_dense(nx, nz):
    g = _grid(nx, nz)
    eng = engine_for(g)
    M = int(eng.lib.nhqg_mode_count(eng.handle))
    assert (2 * M) % 128 != 0
    V = np.asarray(g.V)
    sw, sd = _stencils(g)
    rng = np.random.default_rng(nz)
    for field, A in ((0, V), (1, V @ sw), (2, V @ sd)):
        K = A.shape[1]
        c = rng.standard_normal((K, M)) + 1j * rng.standard_normal((K, M))
        c[:, :3] *= 1e3  # columns of very different size stay independent
        out = torch.full((g.Nz + 1, M), float("nan"), dtype=torch.complex64, device="cuda")
        eng.tc_to_nodal(field, torch.from_numpy(c).cuda(), out)
        torch.cuda.synchronize()
        ref = A @ c
        got = out.cpu().numpy().astype(np.complex128)
        assert np.all(np.isfinite(got))
        err = np.linalg.norm(got - ref, axis=0) / np.linalg.norm(ref, axis=0)
        assert err.max() <= 3e-6, (nx, nz, field, err.max())


@pytest.mark.parametrize("nx,nz", SIZES)
def test_to_coef_matches_dense(nx, nz):
    g = _grid(nx, nz)
    eng = engine_for(g)
    M = int(eng.lib.nhqg_mode_count(eng.handle))
    rng = np.random.default_rng(100 + nz)
    x = (rng.standard_normal((g.Nz + 1, M)) + 1j * rng.standard_normal((g.Nz + 1, M))).astype(np.complex64)
    buf = torch.from_numpy(x).cuda()
    eng.tc_to_coef(buf)
    torch.cuda.synchronize()
    ref = np.asarray(g.V_inv) @ x.astype(np.complex128)
    got = buf.cpu().numpy().astype(np.complex128)
    err = np.linalg.norm(got - ref, axis=0) / np.linalg.norm(ref, axis=0)
    assert err.max() <= 3e-6, (nx, nz, err.max())


def test_round_trip_full_size():
    """256^2 x 256 (the benchmark size): to_coef(to_nodal(c)) == c through the
    two tensor-core transforms, and the engine reports them enabled."""
    g = _grid(256, 256)
    eng = engine_for(g)
    eng.set_precision("mixed")
    assert eng.tensor_core_vertical
    M = int(eng.lib.nhqg_mode_count(eng.handle))
    rng = np.random.default_rng(7)
    c = torch.from_numpy(rng.standard_normal((g.Nz + 1, M)) + 1j * rng.standard_normal((g.Nz + 1, M))).cuda()
    x = torch.empty((g.Nz + 1, M), dtype=torch.complex64, device="cuda")
    eng.tc_to_nodal(0, c, x)
    eng.tc_to_coef(x)
    torch.cuda.synchronize()
    assert rel_l2(x.cpu().numpy().astype(np.complex128), c.cpu().numpy()) <= 5e-6


@pytest.mark.parametrize("nx,nz", [(64, 32), (48, 48)])
def test_mixed_step_tensor_cores_vs_fft(nx, nz):
    """The mixed step with either vertical engine agrees with the plain step
    to the mixed path's 1e-6, and the explicit RHS to 2e-5."""
    g = _grid(nx, nz)
    eng = engine_for(g)
    s0 = S.sanitize_state(theta_perturbation_state(g, seed=3), g)
    host = lambda st: tuple(t.detach().cpu().numpy() for t in st)  # noqa: E731
    plain = host(S.imex_step(s0, g))
    e64 = host(S.explicit_rhs(s0, g))
    res = {}
    for on in (True, False):
        eng.set_precision("mixed")
        eng.tensor_core_vertical = on
        res[on] = host(S.imex_step(s0, g, precision="mixed"))
        assert_state_close(res[on], plain, 1e-6, th_bar_abs=1e-14)
        assert_state_close(host(S.explicit_rhs(s0, g, precision="mixed")), e64, 2e-5, th_bar_abs=1e-14)
    eng.tensor_core_vertical = True
    assert eng.tensor_core_vertical


def test_open_top_basis_has_no_tensor_core_path():
    """The open-top w basis breaks the mirror parity of V S_w: the switch
    refuses, and the mixed path keeps the FP32 DCT."""
    g = _grid(32, 16, w_bc_top="neumann")
    eng = engine_for(g)
    assert not eng.tensor_core_vertical
    with pytest.raises(NativeError):
        eng.tensor_core_vertical = True
