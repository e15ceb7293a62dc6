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
    g = make_grid(NHQGConfig(**dict(meta["cfg"])))
    if meta.get("override_eta_sponge"):
        eta = arrays["grid.eta_hat"][0]
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
        for i, key in enumerate(DIAG_KEYS):
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
