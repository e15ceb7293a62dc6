"""Checkpoint schema compatibility with the reference (nhqg/io.py:107-153)."""

import numpy as np

from nhqg_gb300 import NHQGConfig
from nhqg_gb300.io import load_checkpoint, save_checkpoint

REF_KEYS = {"q_hat_real", "q_hat_imag", "w_hat_real", "w_hat_imag", "th_hat_real", "th_hat_imag",
            "th_bar", "step", "t"}


def _state(rng, P=9, Nx=16):
    Nk = Nx // 2 + 1
    z = lambda n: rng.standard_normal((n, Nx, Nk)) + 1j * rng.standard_normal((n, Nx, Nk))  # noqa: E731
    return z(P), z(P - 2), z(P - 2), rng.standard_normal(P)


def test_roundtrip_and_schema(tmp_path):
    rng = np.random.default_rng(0)
    cfg = NHQGConfig(Nx=16, Nz=8, dt=2e-5)
    s = _state(rng)
    fname = save_checkpoint(s, 1234, cfg, output_dir=str(tmp_path))
    assert fname.endswith("checkpoint_00001234.npz")
    z = np.load(fname)
    assert set(z.files) == REF_KEYS
    assert int(z["step"]) == 1234 and abs(float(z["t"]) - 1234 * 2e-5) < 1e-18
    got, step, t = load_checkpoint(fname, to_device=False)
    assert step == 1234
    neg = (-np.arange(16)) % 16
    for a, b in zip(got[:3], s[:3]):
        # interior columns unchanged; ky = 0 and Nyquist columns Hermitian-projected
        assert np.array_equal(a[:, :, 1:-1], b[:, :, 1:-1])
        for c in (0, -1):
            assert np.allclose(a[:, :, c], 0.5 * (b[:, :, c] + np.conj(b[:, neg, c])), atol=0, rtol=0)
    assert np.array_equal(got[3], s[3])


def test_band_limit_option(tmp_path):
    rng = np.random.default_rng(1)
    cfg = NHQGConfig(Nx=24, Nz=6, dt=1e-3)
    fname = save_checkpoint(_state(rng, P=7, Nx=24), 5, cfg, output_dir=str(tmp_path))
    got, _, _ = load_checkpoint(fname, to_device=False, band_limit=True)
    K = 8
    for f in got[:3]:
        assert np.all(f[:, K + 1:24 - K, :] == 0) and np.all(f[:, :, K + 1:] == 0)
