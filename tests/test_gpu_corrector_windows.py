"""The corrector's windowed 1-D solve and its fallback.

Each substep of the balanced SBP2 corrector (nhqg/solver.py:873-906, the
solve of A tb_new = B tb_sbp - mu sub_dt D1 flux) runs FP64 iterative
refinement around overlapping FP32 window solves; if the windows do not
converge the kernel factors the whole band and redoes the solve.  Every
choice of the overlap therefore solves to FP64 round-off.  Here the same
state is stepped with the host's overlap (the default, 7 rows here), with one
global FP32 LU (overlap 0) and with an overlap too small for the windows to
converge (1 row: the fallback path; tests/test_corrector_windows_cpu.py shows
on the CPU that it fails the kernel's check at this size), in both precisions;
the results agree to 1e-13 relative, far below the 1e-12 parity gates of the
step.
"""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from _util import rel_l2

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state  # noqa: E402
from nhqg_gb300 import solver as S  # noqa: E402
from nhqg_gb300.engine import Engine  # noqa: E402

L_C = 2.0 * math.pi / 1.3048
# 64 levels: two windows of 32 core rows, so the windows' coupling matters
CFG = dict(Nx=32, Nz=64, L=10 * L_C, Ra_tilde=100.0, sigma=1.0, nu_q=1.0, nu_w=1.0, nu_theta=1.0,
           hyper_order=1, dt=5e-5, nonlinear_advection="flux", horizontal_dealiasing="23_rule",
           float_dtype="float64", thermal_closure="evolve_mean",
           mean_exchange_discretization="balanced_sbp2_pc", sbp_corrector_substeps=4)


def _run(monkeypatch, overlap, precision):
    if overlap is None:
        monkeypatch.delenv("NHQG_CORR_WINDOW_OVERLAP", raising=False)
    else:
        monkeypatch.setenv("NHQG_CORR_WINDOW_OVERLAP", str(overlap))
    g = make_grid(NHQGConfig(**CFG))
    eng = Engine(g)  # a context of its own: the switch is read when it is created
    s = S.to_device(theta_perturbation_state(g, seed=3, amplitude=0.3))
    eng.step(*s, n_steps=20, precision=precision)
    torch.cuda.synchronize()
    assert eng.device_status() == 0
    return S.to_host(s)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_window_overlap_and_fallback_agree(monkeypatch, precision):
    ref = _run(monkeypatch, None, precision)
    assert all(np.all(np.isfinite(a)) for a in ref)
    for ov in (0, 1):
        got = _run(monkeypatch, ov, precision)
        for a, b in zip(got, ref):
            assert rel_l2(a, b) <= 1e-13, (ov, rel_l2(a, b))
