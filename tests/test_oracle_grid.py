"""Pin the oracle's host precompute and 2/3-rule products.

* grid tables against the reference's own ``make_grid`` output for a polar
  trap / sponge / open-top configuration (``tests/golden/grid96.npz``);
* the analytic known answers of the reference's spectral tests
  (``tests/test_spectral.py:40-120`` of the reference), restated for the 2/3
  products the time step uses.
"""

import json

import numpy as np
import pytest

import fixtures
import oracle
from oracle.nhqg_oracle import OracleConfig


@pytest.fixture(scope="module")
def grid96():
    with np.load(fixtures.GOLDEN_DIR / "grid96.npz") as z:
        meta = json.loads(str(z["meta"]))
        arrays = {k: z[k] for k in z.files if k != "meta"}
    return meta, arrays, oracle.make_grid(OracleConfig(**meta["cfg"]), with_shell_inverses=False)


TABLES = ["sponge_phys", "G_Z", "G_Z2", "V", "V_inv", "dirichlet_stencil", "dirichlet_pinv",
          "w_stencil", "w_pinv", "map_w_to_th", "map_th_to_w", "proj_dirichlet",
          "proj_neumann", "proj_w", "sbp_D1", "sbp_L", "cgl_to_sbp", "sbp_to_cgl", "Z",
          "cc_weights", "inv_denom", "inv_alpha_q", "inv_alpha_th", "diss_rate_q",
          "mask_23", "ksq_idx"]


@pytest.mark.parametrize("name", TABLES)
def test_grid_tables(grid96, name):
    meta, arrays, grid = grid96
    ref = arrays[f"grid.{name}"]
    got = np.asarray(getattr(grid, name))
    assert got.shape == ref.shape
    scale = max(float(np.max(np.abs(ref))), 1e-300)
    assert float(np.max(np.abs(got - ref))) <= 1e-13 * scale


def test_eta_hat(grid96):
    meta, arrays, grid = grid96
    ref = fixtures.unpack(arrays["grid.eta_hat__packed"], grid.Nx)[0]
    assert np.max(np.abs(grid.eta_hat - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_shell_inverses(grid96):
    meta, arrays, grid = grid96
    picks = arrays["grid.imex_inv_pick"]
    from oracle.nhqg_oracle import _shell_inverse_lookup
    got = _shell_inverse_lookup(grid, picks)
    ref = arrays["grid.imex_inv"]
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.fixture
def box64():
    Nx, L = 64, 2 * np.pi
    kx = (2 * np.pi * np.fft.fftfreq(Nx, d=L / Nx))[:, None]
    ky = (2 * np.pi * np.arange(Nx // 2 + 1) / L)[None, :]
    x = np.linspace(0, L, Nx, endpoint=False)
    X, Y = np.meshgrid(x, x, indexing="ij")
    K = Nx // 3
    ii = np.arange(Nx)
    kint = np.where(ii <= Nx // 2, ii, ii - Nx)
    mask = ((np.abs(kint)[:, None] <= K) & (np.arange(Nx // 2 + 1)[None] <= K)).astype(float)
    return Nx, kx, ky, X, Y, mask


def _single(fn, a, b, box):
    Nx, kx, ky, X, Y, mask = box
    A = np.fft.rfft2(a)[None]
    B = np.fft.rfft2(b)[None]
    return fn(A, B, B, B, kx, ky, mask, Nx)[0][0]


@pytest.mark.parametrize("fn", [oracle.triple_jacobian_23, oracle.triple_conservative_flux_divergence_23])
def test_jacobian_analytic(box64, fn):
    """J[sin x, sin y] = cos x cos y ; J[sin 2x, sin 3y] = 6 cos 2x cos 3y."""
    Nx, kx, ky, X, Y, mask = box64
    J = np.fft.irfft2(_single(fn, np.sin(X), np.sin(Y), box64), s=(Nx, Nx))
    np.testing.assert_allclose(J, np.cos(X) * np.cos(Y), atol=1e-12)
    J = np.fft.irfft2(_single(fn, np.sin(2 * X), np.sin(3 * Y), box64), s=(Nx, Nx))
    np.testing.assert_allclose(J, 6 * np.cos(2 * X) * np.cos(3 * Y), atol=1e-11)


def test_antisymmetry_and_flux_equals_jacobian(box64):
    Nx, kx, ky, X, Y, mask = box64
    a = np.sin(X) + 0.5 * np.cos(3 * Y)
    b = np.cos(2 * X) * np.sin(Y)
    jab = _single(oracle.triple_jacobian_23, a, b, box64)
    jba = _single(oracle.triple_jacobian_23, b, a, box64)
    np.testing.assert_allclose(jab + jba, 0.0, atol=1e-12)
    fab = _single(oracle.triple_conservative_flux_divergence_23, a, b, box64)
    np.testing.assert_allclose(fab, jab, atol=1e-11)
