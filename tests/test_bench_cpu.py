"""CPU checks of bench.py: the reference arm's JSON contract on a tiny
workload (both dealiasing rules), and the per-kernel work model that the
roofline figures are computed from."""

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from nhqg_gb300 import NHQGConfig, make_grid  # noqa: E402


@pytest.mark.parametrize("rule", ["23_rule", "32_rule"])
def test_reference_arm_json(rule):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--nx", "16",
                          "--nz", "8", "--steps", "1", "--warmup", "1", "--rule", rule],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "steps/s"
    assert line["higher_is_better"] is True and line["steps"] == 1
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert ("3/2 rule" in line["config"]["workload"]) == (rule == "32_rule")


@pytest.mark.parametrize("rule", ["23_rule", "32_rule"])
def test_kernel_work_model(rule):
    g = make_grid(NHQGConfig(**bench.workload(48, 16, rule)))
    names = ["h1_col_ifft", "h2_row_products", "h3_col_fft", "h2_row_products_f32", "vfwd",
             "vback_stage1", "vback_stage2", "shell_solve", "tau_solve", "corr_pre", "corr_sub_mid",
             "corr_sub_last", "vpost", "tc_to_nodal", "tc_to_coef"]
    for tc in (False, True):
        for n in names:
            flops, bytes_, pipe = bench.kernel_work(n, g, 1, tc)
            assert bytes_ > 0 and flops >= 0, n
            assert pipe in ("fp64", "fp32", "df64", "hbm"), (n, pipe)
        # the mixed (tensor-core) step runs its column kernels in double-float
        assert bench.kernel_work("corr_pre", g, 1, True)[2] == "df64"
        assert bench.kernel_work("corr_pre", g, 1, False)[2] == "fp64"


def test_kernel_work_padded_products():
    """The 3/2 rule transforms Npad = 3Nx/2 points over the full band: about
    2.4 times the 2/3 rule's row-product work."""
    f23 = bench.kernel_work("h2_row_products", make_grid(NHQGConfig(**bench.workload(48, 16))), 1)[0]
    f32 = bench.kernel_work("h2_row_products", make_grid(NHQGConfig(**bench.workload(48, 16, "32_rule"))), 1)[0]
    assert 2.0 * f23 < f32 < 3.0 * f23


def test_dominant_roofline_entry():
    """The JSON roofline block of the dominant kernel, from a synthetic
    profile: largest-share class, the HBM view against the measured copy
    bandwidth, the ncu traffic of the headline workload, the pipe view."""
    g = make_grid(NHQGConfig(**bench.workload(48, 16)))
    prof = {"h2_row_products_f32": (20, 13.0), "corr_pre": (20, 8.0), "corr_sub_mid": (60, 5.0)}
    peaks = {"fp64": 1.1, "fp32": 70.0, "hbm": 6500.0}
    roof = bench._roofline(prof, g, 10, peaks)
    dom = bench.dominant_roofline(prof, roof, (256, 256, "23_rule"), peaks)
    assert dom["kernel"] == "h2_row_products_f32" and dom["bound"] == "hbm" and dom["unit"] == "GB/s"
    assert dom["peak"] == 6500.0 and 0.0 < dom["frac"] == round(dom["achieved"] / 6500.0, 4)
    assert dom["traffic"] == bench.NCU_TRAFFIC_256["h2_row_products_f32"]
    assert dom["pipe_view"]["pipe"] == "fp32" and dom["pipe_view"]["frac"] > 0
    other = bench.dominant_roofline(prof, roof, (128, 256, "23_rule"), peaks)
    assert other["traffic"] is None and "traffic_view" not in other



def test_reference_arm_polar_json():
    """The reference arm of the polar-trap configuration: whole oracle steps
    at 256^2 x 32 with the trap, the sponge and the open top."""
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--config", "polar",
                          "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["metric"] == bench.POLAR_METRIC and "polar" in line["config"]["workload"]
    assert line["config"]["Nx"] == 256 and line["config"]["Nz"] == 32
    assert "whole steps" in line["cpu_baseline"]["sample"]


def test_polar_workload_passes_resolution_guards():
    """The production-scaled trap and sponge pass the eta and sponge
    resolution guards of make_grid at 256^2 x 32."""
    g = make_grid(NHQGConfig(**bench.polar_workload()))
    assert g.eta_hat is not None and g.sponge_phys is not None and g.w_bc_top == "neumann"
