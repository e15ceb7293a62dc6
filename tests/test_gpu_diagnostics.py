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
