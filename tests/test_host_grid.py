"""Host-side checks (no GPU): the product's make_grid against the oracle's
restatement of the reference, the C-ABI library surface, and the theta'
initial state against the reference fixture."""

import re
from pathlib import Path

import numpy as np
import pytest

import fixtures
import oracle
from oracle.nhqg_oracle import OracleConfig
from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state
from nhqg_gb300 import _native as nat

ROOT = Path(__file__).resolve().parent.parent

CFGS = [
    dict(Nx=32, Nz=16, L=48.154, Ra_tilde=100.0, nu_q=1.0, nu_w=1.0, nu_theta=1.0, hyper_order=1,
         dt=5e-5, thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
         sbp_corrector_substeps=4, nonlinear_advection="flux"),
    dict(Nx=24, Nz=12, L=20.0, Ra_tilde=70.0, nu_q=1e-3, nu_w=2e-3, nu_theta=3e-3, hyper_order=2,
         dt=1e-4, drag=0.1, Ld=3.0, w_bc_top="neumann", sbp_transfer_mode="mass_adjoint"),
]


# 3/2 rule (full band): every shell has a table row; trap eta (unmasked) and
# the padded sponge
CFGS_32 = [
    dict(CFGS[0], horizontal_dealiasing="32_rule"),
    dict(Nx=96, Nz=8, L=40.0, gamma=2.2e-3, trap_r_star=8.0, trap_sharpness=5.0, sponge_rate=5.0,
         sponge_r_start=10.4, sponge_sharpness=5.0, dt=1e-4, horizontal_dealiasing="32_rule"),
]


def _pair(over):
    base = dict(float_dtype="float64", horizontal_dealiasing="23_rule")
    base.update(over)
    return make_grid(NHQGConfig(**base)), oracle.make_grid(OracleConfig(**base))


@pytest.mark.parametrize("over", CFGS_32)
def test_grid_32_rule_matches_oracle(over):
    g, o = _pair(over)
    assert g.Npad == o.Npad == 3 * g.Nx // 2
    assert np.all(g.imex_shell_row >= 0)
    assert np.array_equal(g.imex_inv[g.imex_shell_row], o.imex_inv[o.ksq_idx])
    for name in ("eta_hat", "sponge_phys", "sponge_phys_pad"):
        a, b = getattr(g, name), getattr(o, name)
        assert (a is None) == (b is None), name
        if a is not None:
            assert np.array_equal(np.asarray(a), np.asarray(b)), name
    if g.eta_hat is not None:
        pad = np.zeros((g.Npad, g.Npad // 2 + 1), dtype=np.complex128)
        pad[:g.Nx // 2, :g.Nk] = g.eta_hat[:g.Nx // 2]
        pad[g.Npad - g.Nx // 2:, :g.Nk] = g.eta_hat[g.Nx // 2:]
        assert np.allclose(g.eta_phys, np.fft.irfft2(pad, s=(g.Npad, g.Npad)), rtol=0, atol=1e-15)


@pytest.mark.parametrize("over", CFGS)
def test_grid_matches_oracle(over):
    g, o = _pair(over)
    for name in ("G_Z", "G_Z2", "V", "V_inv", "dirichlet_stencil", "dirichlet_pinv", "w_stencil",
                 "w_pinv", "proj_dirichlet", "proj_neumann", "proj_w", "sbp_D1", "sbp_L",
                 "cgl_to_sbp", "sbp_to_cgl", "kx", "ky", "ksq", "inv_denom", "mask_23",
                 "diss_rate_q", "diss_rate_w", "diss_rate_th", "inv_alpha_q", "inv_alpha_th",
                 "ksq_idx", "Z", "cc_weights"):
        a, b = np.asarray(getattr(g, name)), np.asarray(getattr(o, name))
        assert a.shape == b.shape, name
        assert np.array_equal(a, b), name


@pytest.mark.parametrize("over", CFGS)
def test_shell_tables_bitwise(over):
    """In-band shell inverses equal the reference-order construction bit for bit."""
    g, o = _pair(over)
    rows = g.imex_shell_row
    band = rows >= 0
    ref = o.imex_inv[o.ksq_idx[band]]
    got = g.imex_inv[rows[band]]
    assert np.array_equal(got, ref)
    assert np.all(rows[~band] == -1)


@pytest.mark.parametrize("case", ["prod16", "pad32p16", "pad32l24"])
def test_theta_init_matches_reference_fixture(case):
    """The seeded theta' start against the reference's own, under the 2/3
    rule (band-limited) and the 3/2 rule (full band)."""
    meta, arrays = fixtures.load_case(case)
    cfg = dict(meta["cfg"])
    g = make_grid(NHQGConfig(**cfg))
    s = theta_perturbation_state(g, seed=meta["seed"])
    for got, ref in zip(s, fixtures.state_from(arrays, "s0")):
        scale = max(float(np.linalg.norm(ref)), 1e-300)
        assert float(np.linalg.norm(got - ref)) <= 1e-13 * scale


def test_unsupported_configs_raise():
    with pytest.raises(ValueError):  # 3/2 rule with Npad = 30 (a factor 5)
        make_grid(NHQGConfig(Nx=20, Nz=8, float_dtype="float64"))
    with pytest.raises(ValueError):
        make_grid(NHQGConfig(Nx=32, Nz=8, float_dtype="float64", horizontal_dealiasing="45_rule"))
    with pytest.raises(ValueError):
        make_grid(NHQGConfig(Nx=32, Nz=8, float_dtype="float32", horizontal_dealiasing="23_rule"))
    with pytest.raises(ValueError):
        make_grid(NHQGConfig(Nx=32, Nz=8, float_dtype="float64", horizontal_dealiasing="23_rule",
                             q_boundary="neumann"))
    with pytest.raises(ValueError):
        make_grid(NHQGConfig(Nx=32, Nz=8, float_dtype="float64", horizontal_dealiasing="23_rule",
                             gamma=1e-3, beta=0.5))


def _header_symbols():
    text = (ROOT / "include" / "nhqg_gpu.h").read_text()
    return set(re.findall(r"^\s*(?:int|const char \*)\s*(nhqg_\w+)\s*\(", text, flags=re.M))


def test_library_exports_header_symbols():
    lib_path = nat.build()
    lib = nat.load(lib_path)
    declared = _header_symbols()
    assert declared, "no declarations parsed from include/nhqg_gpu.h"
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(nat.SIGNATURES), declared ^ set(nat.SIGNATURES)
    assert b"sm_103a" in lib.nhqg_version()


def test_ctx_create_rejects_bad_descriptor():
    lib = nat.load()
    import ctypes
    h = ctypes.c_void_p()
    d = nat.GridDesc()
    d.Nx, d.Nz = 30, 8  # 30 = 2*3*5: no radix-5 FFT
    assert lib.nhqg_ctx_create(ctypes.byref(d), ctypes.byref(h)) == 2  # NHQG_ERR_UNSUPPORTED
    d.Nx = 32
    assert lib.nhqg_ctx_create(ctypes.byref(d), ctypes.byref(h)) == 1  # null tables
    # dealiasing rule: unknown value, and a 3/2 rule whose padded grid 3*20/2 = 30
    # has a factor 5 (checked before any table or device allocation)
    d.horizontal_dealiasing = 7
    assert lib.nhqg_ctx_create(ctypes.byref(d), ctypes.byref(h)) == 1  # NHQG_ERR_BAD_ARG
    d.horizontal_dealiasing, d.Nx = 1, 20
    assert lib.nhqg_ctx_create(ctypes.byref(d), ctypes.byref(h)) == 2  # NHQG_ERR_UNSUPPORTED
    d.Nx = 32  # Npad = 48: accepted up to the missing tables
    assert lib.nhqg_ctx_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert not h.value


def test_padded_spectral_arguments_checked_on_host():
    """The 3/2-rule plane operators reject an Npad other than 3*Nx//2 (the
    reference's Npad, nhqg/config.py:76-78) before touching the device."""
    from nhqg_gb300 import spectral as SP
    z = np.zeros((1, 16, 9), dtype=complex)
    kx, ky = np.zeros((16, 1)), np.zeros((1, 9))
    for fn in (SP.triple_jacobian, SP.triple_conservative_flux_divergence):
        with pytest.raises(ValueError):
            fn(z, z, z, z, kx, ky, 16, 16)
    with pytest.raises(ValueError):
        SP.sponge_product_32(z, np.zeros((24, 24)), 16, 32)
