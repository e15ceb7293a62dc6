"""GPU diagnostics (nhqg_diagnostics through the C ABI) against the
reference's compute_diagnostics scalars (tests/golden/diagnostics.npz) and
the oracle.  Tolerance: 1e-12 relative per scalar."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fixtures

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid  # noqa: E402
from nhqg_gb300.diagnostics import DIAG_KEYS, compute_diagnostics  # noqa: E402


def _grid(meta, arrays):
    cfg = dict(meta["cfg"])
    cfg.pop("_override_eta_sponge", None)
    g = make_grid(NHQGConfig(**cfg))
    if meta.get("override_eta_sponge"):
        eta = arrays["grid.eta_hat"][0]
        if g.horizontal_dealiasing == "32_rule":
            g = g._replace(eta_hat=eta, sponge_phys=arrays["grid.sponge_phys"],
                           sponge_phys_pad=arrays["grid.sponge_phys_pad"])
        else:
            g = g._replace(eta_hat=eta, sponge_phys=arrays["grid.sponge_phys"],
                           eta_phys=np.fft.irfft2(eta, s=(g.Nx, g.Nx)))
    return g


@pytest.mark.parametrize("case", fixtures.CASES)
def test_diagnostics_golden(case):
    meta, arrays = fixtures.load_case(case)
    g = _grid(meta, arrays)
    gd = fixtures.load_diagnostics()
    for label in ("r", "s0"):
        got = compute_diagnostics(fixtures.state_from(arrays, label), g)
        ref = gd[f"{case}.{label}"]
        for i, key in enumerate(DIAG_KEYS[:len(ref)]):  # the golden's scalar keys
            assert abs(got[key] - ref[i]) <= 1e-12 * abs(ref[i]) + 1e-300, (case, label, key, got[key], ref[i])


@pytest.mark.parametrize("case", fixtures.CASES)
def test_spectra_golden(case):
    """Device shell and vertical spectra (nhqg_spectra) against the reference's
    energy_spectrum and vertical_mode_energy (tests/golden/spectra.npz), the
    psi kinetic-energy spectrum against the oracle, and the shell sum against
    the scalar KE_tot: 1e-11 relative to each spectrum's largest entry (the
    device sums in another order)."""
    import oracle
    from oracle.nhqg_oracle import OracleConfig, OracleState
    from nhqg_gb300.diagnostics import high_mode_fraction, spectra

    meta, arrays = fixtures.load_case(case)
    g = _grid(meta, arrays)
    og = oracle.make_grid(OracleConfig(**dict(meta["cfg"])))
    gs = fixtures.load_spectra()
    for label in ("r", "s0"):
        st = fixtures.state_from(arrays, label)
        got = spectra(st, g)
        for key in fixtures.SPEC_KEYS:
            ref = gs[f"{case}.{label}.{key}"]
            assert got[key].shape == ref.shape, (case, label, key)
            scale = max(float(np.max(np.abs(ref))), 1e-300)
            assert float(np.max(np.abs(got[key] - ref))) <= 1e-11 * scale, (case, label, key)
        pke = oracle.psi_ke_vertical_spectrum(st[0], og)
        assert float(np.max(np.abs(got["psi_ke"] - pke))) <= 1e-11 * max(float(np.max(pke)), 1e-300)
        ke = compute_diagnostics(st, g)["KE_tot"]
        assert abs(float(np.sum(got["E_tot"])) / g.Nx ** 4 - ke) <= 1e-11 * abs(ke) + 1e-300
        assert abs(high_mode_fraction(got["q"]) - oracle.high_mode_fraction(gs[f"{case}.{label}.q"])) <= 1e-11


@pytest.mark.parametrize("case", fixtures.CASES + fixtures.PAD_CASES)
def test_diagnostics_extra_golden(case):
    """Device physical-space maxima over the Nx grid at every CGL node
    (max_speed = max sqrt(u^2 + v^2), max_w, max_theta, max_tw) and the
    heat-flux mismatch against the reference's compute_diagnostics
    (tests/golden/diagnostics_extra.npz, nhqg/diagnostics.py:631-641),
    both dealiasing rules: 1e-12 relative (1e-13 absolute for the mismatch,
    a difference of two nearly equal averages)."""
    meta, arrays = fixtures.load_case(case)
    g = _grid(meta, arrays)
    gd = fixtures.load_diagnostics_extra()
    keys = [str(k) for k in gd["keys"]]
    for label in ("r", "s0"):
        got = compute_diagnostics(fixtures.state_from(arrays, label), g)
        ref = gd[f"{case}.{label}"]
        for i, key in enumerate(keys):
            tol = 1e-12 * abs(ref[i]) if key != "heat_flux_mismatch" else 1e-13
            assert abs(got[key] - ref[i]) <= tol + 1e-300, (case, label, key, got[key], ref[i])


@pytest.mark.parametrize("case", fixtures.CASES + fixtures.PAD_CASES)
def test_field_shell_spectra_golden(case):
    """Device horizontal shell spectra of q, w, theta at the CGL nodes
    against the reference's (tests/golden/field_spectra.npz,
    nhqg/diagnostics.py:104-111, 667-669): 1e-11 relative to each spectrum's
    largest entry (the device sums in another order)."""
    from nhqg_gb300.diagnostics import spectra

    meta, arrays = fixtures.load_case(case)
    g = _grid(meta, arrays)
    gs = fixtures.load_field_spectra()
    for label in ("r", "s0"):
        got = spectra(fixtures.state_from(arrays, label), g)
        assert np.allclose(got["k_bins"], gs[f"{case}.{label}.k_bins"], rtol=1e-14, atol=0.0)
        for key in ("q", "w", "th"):
            ref = gs[f"{case}.{label}.{key}"]
            mine = got[f"{key}_shell"]
            assert mine.shape == ref.shape, (case, label, key)
            scale = max(float(np.max(np.abs(ref))), 1e-300)
            assert float(np.max(np.abs(mine - ref))) <= 1e-11 * scale, (case, label, key)
