"""Host-side accuracy check of the mixed path's double-float arithmetic
(nhqg_gb300/csrc/df64.cuh): the operator code is compiled for the host by
nvcc (plain IEEE FP32, no contraction) and checked against long-double
references by tests/df64_check.cu -- the FP64 split and its round trip,
sums (relative to |a| + |b|), products and fused multiply-adds, and the exact
float-to-double widening."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_double_float_error_bounds(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path / "df64_check"
    build = subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                            f"-I{ROOT / 'nhqg_gb300' / 'csrc'}", f"-I{ROOT / 'include'}",
                            str(ROOT / "tests" / "df64_check.cu"), "-o", str(exe)],
                           capture_output=True, text=True, timeout=600)
    assert build.returncode == 0, build.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
