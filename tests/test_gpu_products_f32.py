"""FP32 horizontal products of the mixed path against the FP64 products.

At Nx = 64, 128, 256 (2/3 rule) the mixed path forms its products with
register-resident FFTs (csrc/horizontal_reg.cu); other sizes use the
shared-memory FFT kernels.  Both forms (flux, Jacobian), with and without the
trap PV eta and the sponge, are checked through the explicit RHS on a random
state whose spectrum fills the 2/3 band (reference semantics:
nhqg/spectral.py:53-60, 281-358, nhqg/solver.py:510-599).  Tolerance: 2e-5
relative L2 per field, the FP32-product bound of the other mixed-path tests.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from _util import assert_state_close

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402

L_C = 2.0 * np.pi / 1.3048


def _host(state):
    return tuple(t.detach().cpu().numpy() for t in state)


def _smooth_eta_sponge(g):
    """Band-limited stand-ins for the trap PV and the sponge rate."""
    Nx, L = g.Nx, float(g.L)
    x = np.arange(Nx) * (L / Nx)
    X, Y = np.meshgrid(x, x, indexing="ij")
    k0 = 2.0 * np.pi / L
    eta = -2.2e-3 * (3.0 + np.cos(k0 * X) + np.cos(k0 * Y) + 0.5 * np.cos(k0 * (X + 2 * Y)))
    sigma = 5.0 * (0.5 + 0.25 * np.cos(k0 * X) * np.cos(k0 * Y) + 0.2 * np.sin(2 * k0 * X))
    return np.fft.rfft2(eta), sigma


def _state(g, seed):
    rng = np.random.default_rng(seed)
    P, G, Nk, Nx = g.Nz + 1, g.Nz - 1, g.Nk, g.Nx
    env = np.exp(-np.asarray(g.ksq) / (2.0 * float(np.max(g.ksq)) / 9.0))

    def fld(n):
        return 0.3 * (rng.standard_normal((n, Nx, Nk)) + 1j * rng.standard_normal((n, Nx, Nk))) * env[None]

    return S.sanitize_state((fld(P), fld(G), fld(G), np.zeros(P)), g)


@pytest.mark.parametrize("nx", [64, 128, 256])
@pytest.mark.parametrize("form", ["flux", "jacobian"])
@pytest.mark.parametrize("extras", [False, True], ids=["plain", "eta_sponge"])
def test_fp32_products_vs_fp64(nx, form, extras):
    cfg = dict(Nx=nx, Nz=16, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, nonlinear_advection=form,
               horizontal_dealiasing="23_rule", float_dtype="float64", thermal_closure="fixed_conduction")
    g = make_grid(NHQGConfig(**cfg))
    if extras:
        eta, sigma = _smooth_eta_sponge(g)
        g = g._replace(eta_hat=eta, sponge_phys=sigma, eta_phys=np.fft.irfft2(eta, s=(nx, nx)))
    s = _state(g, nx + (7 if extras else 0))
    E64 = _host(S.explicit_rhs(s, g))
    E32 = _host(S.explicit_rhs(s, g, precision="mixed"))
    assert_state_close(E32, E64, 2e-5, th_bar_abs=1e-14)


@pytest.mark.parametrize("nx", [48, 256])
@pytest.mark.parametrize("form", ["flux", "jacobian"])
def test_fp32_products_small_q_large_eta(nx, form):
    """q five orders below an O(1) trap PV with a sponge (the polar
    configuration's start): the FP32 products take q itself and add the trap
    term in gradient form, so sigma q and the advection of eta keep their
    FP32 accuracy instead of cancelling q + eta against eta (Nx = 48 runs the
    shared-memory FFT kernels, 256 the register ones)."""
    cfg = dict(Nx=nx, Nz=16, L=10 * L_C, Ra_tilde=100.0, dt=5e-5, nonlinear_advection=form,
               horizontal_dealiasing="23_rule", float_dtype="float64", thermal_closure="fixed_conduction")
    g = make_grid(NHQGConfig(**cfg))
    eta, sigma = _smooth_eta_sponge(g)
    eta = eta * 1000.0
    g = g._replace(eta_hat=eta, sponge_phys=sigma, eta_phys=np.fft.irfft2(eta, s=(nx, nx)))
    s = _state(g, nx + 3)
    s = S.State(s.q_hat * 1e-5, s.w_hat, s.th_hat, s.th_bar)
    E64 = _host(S.explicit_rhs(s, g))
    E32 = _host(S.explicit_rhs(s, g, precision="mixed"))
    assert_state_close(E32, E64, 2e-5, th_bar_abs=1e-14)
