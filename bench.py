#!/usr/bin/env python
"""NHQG time-step benchmark on GB300 (steps/s at 256^2 x 256).

Workload (the headline configuration): Nx=Ny=256, Nz=256, L = 10 L_c
(L_c = 2 pi / 1.3048), Ra~=100, Pr=1, nu=1 (Laplacian), dt=2e-5, flux-form
advection, 2/3-rule dealiasing, evolve_mean closure with the balanced SBP2
predictor/corrector (4 substeps), ARS(2,2,2).  Input: the seeded theta'
start (1e-3 N(0,1) sin(pi Z), PCG64 seed 0) -- synthetic -- spun up by
--spinup plain FP64 steps (1000 by default, about 40 s; the precision
study's 5000-step spin-up is --spinup 5000, about 3 minutes).  The step's work
does not depend on the state.  Every step streams several GB, far above the
129 MB L2, so no explicit L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The default arm times the mixed-precision step (value, the headline) and the
plain FP64 step (plain_fp64) on the same state, and reports the per-field
relative L2 difference of the mixed state from the plain one after 1 and
--err-steps steps.  ``--impl reference`` times the CPU port of the reference
algorithm (NumPy/SciPy on all host cores) on the same workload.  One JSON
line on stdout (rank 0).
"""

from __future__ import annotations

import argparse
import csv
import io
import json
import math
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L_C = 2.0 * math.pi / 1.3048
METRIC = "NHQG steps/s at 256^2x256: mixed-precision vs plain FP64 on GB300, rel err <=1e-6"


def workload(nx: int, nz: int, rule: str = "23_rule") -> dict:
    return dict(Nx=nx, Nz=nz, L=10 * L_C, Ra_tilde=100.0, sigma=1.0, nu_q=1.0, nu_w=1.0,
                nu_theta=1.0, hyper_order=1, dt=2e-5, nonlinear_advection="flux",
                horizontal_dealiasing=rule, float_dtype="float64",
                thermal_closure="evolve_mean", mean_exchange_discretization="balanced_sbp2_pc",
                sbp_corrector_substeps=4)


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ distributed
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        rows = [r for r in csv.reader(io.StringIO(out)) if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ roofline bookkeeping
NOMINAL_FP32_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # FFMA lanes x 2 flops x max SM clock


def kernel_work(name: str, g, launches_per_step: int, tc: bool = False) -> tuple[float, float, str]:
    """(algorithmic flops, algorithmic DRAM bytes, limiting pipe) per launch of
    one kernel class, for the algorithm the engine runs.

    FFTs: 5 n log2 n flops per complex length-n transform.  Vertical DCT-I:
    an FFT of length 2 Nz per complex column (5 (2Nz) log2(2Nz)); dense
    fallback 4 P^2.  Bytes: each field read or written once per launch
    (complex128 = 16 B, complex64 = 8 B); the FFT intermediates of the
    horizontal products make one HBM round trip between the three kernels.
    The pipe is 'fp64' or 'fp32' (arithmetic) -- the GB300 FP64 rate is 1/64
    of FP32, so every FP64 kernel is arithmetic-bound -- 'df64' for the mixed
    path's column kernels, which run the FP64 algorithm in double-float on the
    FP32 pipe (their flops are counted as the FP64 algorithm's), or 'hbm'."""
    Nx, Nz = g.Nx, g.Nz
    P, G = Nz + 1, Nz - 1
    if g.horizontal_dealiasing == "32_rule":  # full band, products on the padded grid
        Mr, Mc, N = Nx, Nx // 2 + 1, 3 * Nx // 2
    else:
        K = Nx // 3
        Mr, Mc, N = 2 * K + 1, K + 1, Nx
    M = Mr * Mc
    f32 = name.endswith("_f32")
    base = name[:-4] if f32 else name
    col = "df64" if tc else "fp64"  # column kernels of the mixed (tensor-core) step: double-float
    cplx = 8.0 if f32 else 16.0
    pipe = "fp32" if f32 else "fp64"
    fft = 5.0 * N * math.log2(N)
    L = 2 * Nz
    smooth = L
    for f in (2, 3):
        while smooth % f == 0:
            smooth //= f
    dct = 5.0 * L * math.log2(L) if smooth == 1 else 4.0 * P * P
    field = P * M * cplx
    field64 = P * M * 16.0
    if base == "h1_col_ifft":
        return 5 * Mc * P * fft, 3 * field + 5 * P * Mc * N * cplx, pipe
    if base == "h2_row_products":
        return (5 + 6) * (N / 2) * P * fft + 6 * N * N * P, (5 + 6) * P * Mc * N * cplx, pipe
    if base == "h3_col_fft":
        return 6 * Mc * P * fft, 6 * P * Mc * N * cplx + 3 * field, pipe
    if base == "vfwd":
        nf = 3 if launches_per_step <= 1 else 2  # 3 fields at stage 1, 1 at stage 2
        return nf * dct * M, nf * (field64 + field), pipe
    if name in ("vback_stage1", "vback_stage2"):
        # 3 inverse DCTs of A (FP32 in the mixed step) + FP64 stage algebra.
        # After the tensor-core inverse (tc) the kernel reads coefficients and
        # only the stage algebra is left: stencils, G_Z and pinv recurrences and
        # stage combinations, counted from the kernel's operations (FMA = 2
        # flops) per level and mode over the three fields: 42 at stage 1, 108
        # at stage 2.
        # Bytes: every distinct field once.  Stage 1 reads A_q, A_w, A_theta
        # and the state q0, w0, t0 and writes E1 (3) and the solve's R_q,
        # R_theta, rhs_w; stage 2 reads A (3), q0, w0, t0, E1 (3), q1, w1,
        # t1, t1p and writes R_q, R_theta, rhs_w.  A is FP32 in the mixed
        # step (8 B), FP64 nodal otherwise.
        a_b = 3 * (0.5 if tc else 1.0) * field64
        if name == "vback_stage1":
            b = a_b + 3 * field64 + 6 * field64
        else:
            b = a_b + 10 * field64 + 3 * field64
        if tc:
            return (42.0 if name == "vback_stage1" else 108.0) * P * M, b, col
        return 3 * dct * M, b, "fp64"
    if name == "shell_solve":
        n_in = len(np.unique(g.imex_shell_row[g.imex_shell_row >= 0]))
        return 4.0 * G * G * M, 2 * G * M * 16.0 + n_in * G * G * 8.0, "fp64"
    if name == "tau_solve":
        return 2 * 12.0 * Nz * M, 2 * G * M * 16.0, "fp64"
    # the mixed step keeps the corrector's w in FP32 (8 B per complex value)
    wbytes = P * M * (8.0 if tc else 16.0)
    if name == "corr_pre":  # w, theta in; nodal w, SBP w, SBP theta out
        return 2 * dct * M, 3 * field64 + 2 * wbytes, col
    if name == "corr_sub":
        return 2 * 8.0 * P * M, 3 * field64 + wbytes, col
    if name == "corr_sub_mid":  # x = t - dt g w, two dots, R x + rank 2: memory-bound
        return 2 * 16.0 * P * M, 2 * field64 + wbytes, "hbm"
    if name == "corr_sub_last":  # + inverse DCT of y and the Dirichlet pseudo-inverse
        return dct * M + 2 * 16.0 * P * M, 2 * field64 + 2 * wbytes, col
    if name == "vpost":  # stencil, G_Z scan, two stage updates per mode and level
        return 12.0 * P * M, 5 * field64, col
    # tensor-core vertical transforms: two parity-folded GEMMs of Nz/2 rows
    # per field, three TF32 split products each (12 (Nz/2) K M flops);
    # designed HBM-bound: FP64 coefficients in / FP32 nodal out, or FP32 in
    # and out in place
    if name == "tc_to_nodal":
        nf = 3 if launches_per_step <= 1 else 2  # 3 fields at stage 1, 1 at stage 2
        return nf * 12.0 * (Nz // 2) * P * M, nf * (P * M * 16.0 + P * M * 8.0), "hbm"
    if name == "tc_to_coef":
        return 3 * 12.0 * (Nz // 2) * P * M, 3 * 2 * P * M * 8.0, "hbm"
    return 0.0, 0.0, "fp64"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# main kernel classes of the mixed step at 256^2 x 256 (2/3 rule), each from
# a one-launch ncu --set full capture of a timed mixed step at that size
NCU_TRAFFIC_256 = {"h2_row_products_f32": 448960256, "vback_stage2": 880899840, "corr_pre": 202028800,
                   "corr_sub_last": 143561472, "corr_sub_mid": 103279104, "tau_solve": 218991360}
NCU_TRAFFIC_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch, full size"


def dgemm_peak_tflops() -> float:
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def sgemm_peak_tflops() -> float:
    """FP32 CUDA-core GEMM rate (TF32 off), the FP32 analogue of the DGEMM peak."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, dtype=torch.float32, device="cuda")
        b = torch.randn(n, n, dtype=torch.float32, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def measured_hbm_gbs() -> float | None:
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return None


# ------------------------------------------------------------------ CPU (oracle) arm
def workload_name(nx: int, nz: int, rule: str = "23_rule") -> str:
    r = "2/3 rule" if rule == "23_rule" else f"3/2 rule (padded {3 * nx // 2}^2 products)"
    return (f"{nx}^2x{nz} ARS222, evolve_mean balanced_sbp2_pc sub4, flux, {r}, "
            "L=10Lc, Ra=100, Pr=1, dt=2e-5")


def cpu_reference(cfgd: dict, steps: int = 2, warmup: int = 1, label: str | None = None) -> dict:
    """Time whole steps of the NumPy/SciPy port of the reference step
    (``oracle.imex_step``) on all host cores.

    The grid and its per-shell tables are built first and excluded (the
    reference builds them once in make_grid); then ``warmup`` untimed steps
    and ``steps`` timed ones from the seeded theta' start; the value is
    steps / elapsed.  In a same-machine comparison the unmodified reference
    source under the NumPy stand-in for jax took 3.3x (256^2 x 256) and 1.3x
    (64^2 x 32) the port's time per step (oracle/time_reference_cpu.py), so
    the port is the faster of the two CPU paths."""
    import oracle
    from oracle.nhqg_oracle import OracleConfig
    cores = os.cpu_count() or 1
    oracle.nhqg_oracle.set_threads(cores)
    t0 = time.perf_counter()
    g = oracle.make_grid(OracleConfig(**cfgd))
    t_grid = time.perf_counter() - t0
    s = oracle.theta_perturbation_state(g, seed=0)
    for _ in range(warmup):
        s = oracle.imex_step(s, g)
    t0 = time.perf_counter()
    for _ in range(max(1, steps)):
        s = oracle.imex_step(s, g)
    t = time.perf_counter() - t0
    n = max(1, steps)
    return {"value": n / t, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": (f"{n} whole steps (oracle.imex_step, after {warmup} untimed) of "
                       f"{label or workload_name(cfgd['Nx'], cfgd['Nz'], cfgd['horizontal_dealiasing'])} "
                       f"from the seeded theta' start, {t / n:.2f} s each; grid and shell tables built "
                       f"beforehand ({t_grid:.1f} s, excluded); NumPy/SciPy restatement of the reference "
                       "step on all host cores, plain FP64 (JAX is not installed; the unmodified reference "
                       "source under a NumPy stand-in for jax is slower than this port)")}


# ------------------------------------------------------------------ GPU arm
def _rel(a, b) -> float:
    import torch
    den = float(torch.linalg.norm(b))
    num = float(torch.linalg.norm(a - b))
    return num / den if den > 0 else num


def _timed_arm(S, grid, eng, state, precision, args, ws, label=None):
    """Warm up, then CUDA-event time exactly args.steps steps (one
    step_inplace call, the way run() advances a state) bracketed by barrier +
    synchronize; the NVTX range '<precision>_steps' marks them for profilers.
    Then the same number of steps again with the engine's per-kernel event
    profiler on, for the kernel shares."""
    import torch
    S.step_inplace(state, grid, max(3, args.warmup), check=True, precision=precision)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push(f"{label or precision}_steps")
    e0.record()
    S.step_inplace(state, grid, args.steps, precision=precision)  # one call, as run() drives it
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    if eng.device_status() != 0:
        raise RuntimeError(f"device status set during the timed {precision} steps")
    eng.profile(True)
    S.step_inplace(state, grid, args.steps, precision=precision)
    prof = eng.profile_report()
    eng.profile(False)
    return allmax(ms, ws), prof


def _roofline(prof, grid, steps, peaks):
    """Per kernel class: achieved rate of its limiting pipe against the
    measured peak of that pipe, plus the HBM rate at algorithmic bytes."""
    out = {}
    tc = "tc_to_coef" in prof
    for name, (n, ms) in prof.items():
        flops, bytes_, pipe = kernel_work(name, grid, n // max(1, steps), tc)
        avg = ms / n
        entry = {"launches": n, "avg_launch_ms": round(avg, 4), "pipe": pipe,
                 "hbm_gbs_at_algorithmic_bytes": round(bytes_ / (avg * 1e-3) / 1e9, 1)}
        if pipe in ("fp64", "fp32", "df64") and flops > 0:
            ach = flops / (avg * 1e-3) / 1e12
            pk = peaks["fp64" if pipe == "df64" else pipe]
            entry.update(achieved=round(ach, 4), unit="TFLOP/s", peak=round(pk, 4),
                         frac=round(ach / pk, 4), flops_per_launch=flops)
            if pipe == "df64":
                entry["note"] = ("FP64-equivalent flops against the FP64 DGEMM peak; computed in "
                                 "double-float on the FP32 pipe, so frac can exceed 1")
        elif pipe == "hbm" and peaks.get("hbm"):
            ach = bytes_ / (avg * 1e-3) / 1e9
            entry.update(achieved=round(ach, 1), unit="GB/s", peak=peaks["hbm"],
                         frac=round(ach / peaks["hbm"], 4))
        entry["bytes_per_launch"] = bytes_
        out[name] = entry
    return out


def dominant_roofline(prof, roof, workload_key, peaks) -> dict:
    """The roofline block of the kernel class with the largest time share.

    Every kernel of the step is bounded by HBM or by a CUDA-core pipe (no
    kernel with a large share is a contraction), so the block states the HBM
    view: achieved = the class's algorithmic bytes per launch (kernel_work)
    over its average launch time, against the measured copy bandwidth
    (MEASURED_PEAKS.json); traffic = the ncu DRAM bytes of one launch where
    measured for this workload.  ``pipe_view`` keeps the limiting-pipe
    figures (FP64: the DGEMM rate measured in this run; FP32: SGEMM; double-
    float kernels count FP64-equivalent flops against DGEMM, so that figure can
    exceed 1 and only says the FP64 pipe is not the limit)."""
    dname = max(prof.items(), key=lambda kv: kv[1][1])[0]
    r = roof[dname]
    ms = r["avg_launch_ms"]
    bytes_ = r["bytes_per_launch"]
    hbm = peaks.get("hbm")
    ach = bytes_ / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    dom = {"kernel": dname, "bound": "hbm", "achieved": round(ach, 1), "unit": "GB/s",
           "peak": hbm, "frac": round(ach / hbm, 4) if hbm else None, "traffic": None,
           "launches": r["launches"], "avg_launch_ms": ms, "bytes_per_launch": bytes_,
           "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)",
           "pipe_view": {k: r[k] for k in ("pipe", "achieved", "unit", "peak", "frac", "flops_per_launch", "note")
                         if k in r}}
    if workload_key == (256, 256, "23_rule") and dname in NCU_TRAFFIC_256:
        dom["traffic"] = NCU_TRAFFIC_256[dname]
        dom["traffic_source"] = NCU_TRAFFIC_SOURCE
        if hbm:
            gbs = dom["traffic"] / (ms * 1e-3) / 1e9
            dom["traffic_view"] = {"achieved_gbs": round(gbs, 1), "frac": round(gbs / hbm, 4)}
    return dom


def _tendency_shares(S, grid, state) -> dict:
    """|E_f| / |I_f| per field: the explicit (advective) tendency against the
    implicit (linear) one, a measure of how nonlinear the state is."""
    import torch
    E = S.explicit_rhs(state, grid)
    I = S.implicit_tendency(state, grid)  # noqa: E741
    return {n: float(torch.linalg.norm(e) / torch.linalg.norm(i)) if float(torch.linalg.norm(i)) > 0 else None
            for n, e, i in zip(("q_hat", "w_hat", "th_hat"), E[:3], I[:3])}


def _precision_study(S, grid, state, err_steps: int, label: str) -> dict:
    """Mixed against plain from the same state: per-field relative L2 after 1
    and ``err_steps`` steps, the 1-step increments, and the diagnostics; plus
    the state's Nusselt number, kinetic energy and tendency shares."""
    from nhqg_gb300.diagnostics import compute_diagnostics
    names = ("q_hat", "w_hat", "th_hat", "th_bar")
    d0 = compute_diagnostics(state, grid)
    ref = S.State(*(t.clone() for t in state))
    mix = S.State(*(t.clone() for t in state))
    S.step_inplace(ref, grid, 1, check=True)
    S.step_inplace(mix, grid, 1, check=True, precision="mixed")
    err1 = {n: _rel(a, b) for n, a, b in zip(names, mix, ref)}
    inc1 = {n: _rel(a - s0, b - s0) for n, a, b, s0 in zip(names, mix, ref, state)}
    S.step_inplace(ref, grid, err_steps - 1, check=True)
    S.step_inplace(mix, grid, err_steps - 1, check=True, precision="mixed")
    errN = {n: _rel(a, b) for n, a, b in zip(names, mix, ref)}
    d_ref, d_mix = compute_diagnostics(ref, grid), compute_diagnostics(mix, grid)
    diag_cmp = {k: {"plain": d_ref[k], "mixed": d_mix[k],
                    "rel_diff": abs(d_mix[k] - d_ref[k]) / abs(d_ref[k]) if d_ref[k] else abs(d_mix[k])}
                for k in ("Nusselt", "Nusselt_dealiased", "KE_tot", "KE_bt", "w_rms", "th_rms")}
    fields = names[:3]
    return {"start": label,
            "state": {"Nusselt_minus_1": d0["Nusselt"] - 1.0, "KE_tot": d0["KE_tot"],
                      "w_rms": d0["w_rms"], "explicit_over_implicit_tendency": _tendency_shares(S, grid, state)},
            "after_1_step": err1, "increment_1_step": inc1, f"after_{err_steps}_steps": errN,
            "max_field_rel_err_after_1_step": max(err1[n] for n in fields),
            f"max_field_rel_err_after_{err_steps}_steps": max(errN[n] for n in fields),
            f"diagnostics_after_{err_steps}_steps": diag_cmp}


def convecting_state(S, grid, coarse_nz: int, coarse_steps: int, settle_steps: int, amp: float = 1.0):
    """A convecting start on ``grid``: a seeded theta' of amplitude ``amp``
    stepped ``coarse_steps`` mixed steps on a coarse grid of the same box
    (Nx/2 x coarse_nz, dt = 5e-5), spectrally prolonged onto ``grid``
    (solver.prolong_state), then ``settle_steps`` plain steps on ``grid``."""
    from nhqg_gb300 import make_grid, theta_perturbation_state
    gc = make_grid(grid.cfg.with_updates(Nx=grid.Nx // 2, Nz=coarse_nz, dt=5e-5))
    sc = S.to_device(theta_perturbation_state(gc, seed=0, amplitude=amp))
    S.step_inplace(sc, gc, coarse_steps, check=True, precision="mixed")
    fine = S.prolong_state(sc, gc, grid)
    del sc
    S.step_inplace(fine, grid, settle_steps, check=True)
    desc = (f"seeded theta' (amplitude {amp}, PCG64 seed 0) stepped {coarse_steps} mixed steps "
            f"(t = {coarse_steps * 5e-5:g}) on {grid.Nx // 2}^2x{coarse_nz}, prolonged onto "
            f"{grid.Nx}^2x{grid.Nz}, then {settle_steps} plain steps")
    return fine, desc


E2E_MIN_STEPS = 50


def _e2e(S, grid, state, steps: int, ws: int) -> dict:
    """End to end through the public API with pinned host buffers (mixed
    path): every step uploads its input state and downloads its result.
    imex_step_many overlaps those copies with the steps on two copy streams;
    the serial imex_step call per step is timed beside it.  At least
    E2E_MIN_STEPS steps are timed (one pinned input reused), so that the
    pipeline's one-time fill and drain (the first upload and the last
    download, about 2 ms each at 256^2 x 256) weigh as in a long run; the
    timed region still holds every step's own upload and download."""
    import torch
    steps = max(steps, E2E_MIN_STEPS)
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in S.to_host(state)]
    outs = [tuple(torch.empty_like(p).pin_memory() for p in pinned) for _ in range(2)]
    S.imex_step_many([pinned] * 2, grid, precision="mixed", out=outs)
    torch.cuda.synchronize()
    barrier(ws)
    ee0 = torch.cuda.Event(enable_timing=True)
    ee1 = torch.cuda.Event(enable_timing=True)
    ee0.record()
    S.imex_step_many([pinned] * steps, grid, precision="mixed", out=outs)
    ee1.record()
    torch.cuda.synchronize()
    e2e_ms = allmax(ee0.elapsed_time(ee1), ws)
    barrier(ws)
    es0 = torch.cuda.Event(enable_timing=True)
    es1 = torch.cuda.Event(enable_timing=True)
    es0.record()
    for _ in range(steps):
        res = S.imex_step(pinned, grid, precision="mixed")
        for o, r in zip(outs[0], res):
            o.copy_(r, non_blocking=True)
    es1.record()
    torch.cuda.synchronize()
    e2e_serial_ms = allmax(es0.elapsed_time(es1), ws)
    bytes_state = int(sum(p.numel() * p.element_size() for p in pinned))
    return {"value": round(ws * steps / (e2e_ms * 1e-3), 4), "unit": "steps/s",
            "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state, "steps": steps,
            "api": ("nhqg_gb300.solver.imex_step_many(pinned host States, precision='mixed'): each step "
                    "uploads its input and downloads its result, on two copy streams overlapped "
                    "with the steps"),
            "serial_imex_step": {"value": round(ws * steps / (e2e_serial_ms * 1e-3), 4), "unit": "steps/s",
                                 "api": "imex_step(pinned host State) + D2H of the result, one "
                                        "call per step, no overlap"}}


def _shares(prof, steps: int) -> dict:
    tot = sum(v[1] for v in prof.values())
    return {k: {"launches": n, "ms_per_step": round(t / steps, 4), "share": round(t / tot, 4)}
            for k, (n, t) in sorted(prof.items(), key=lambda kv: -kv[1][1])}


def run_ours(args, ws, rank, local):
    import torch
    from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state
    from nhqg_gb300 import solver as S
    from nhqg_gb300.engine import engine_for

    cfgd = workload(args.nx, args.nz, args.rule)
    t0 = time.perf_counter()
    grid = make_grid(NHQGConfig(**cfgd))
    t_grid = time.perf_counter() - t0
    log(f"[rank {rank}] grid {args.nx}^2x{args.nz}: {t_grid:.1f}s, {grid.imex_inv.shape[0]} shells")
    eng = engine_for(grid)
    peaks = {"fp64": dgemm_peak_tflops(), "fp32": sgemm_peak_tflops(), "hbm": measured_hbm_gbs()}
    tiles = None
    if not args.no_autotune:  # horizontal-product tiles for both precisions, before any timing
        eng.set_precision("mixed")
        tiles = eng.autotune()
        eng.set_precision("fp64")

    # precision study 1: the benchmark's own start, spun up by plain FP64 steps
    t0 = time.perf_counter()
    lin = S.to_device(theta_perturbation_state(grid, seed=0))
    S.step_inplace(lin, grid, args.spinup, check=True)
    study_lin = _precision_study(S, grid, lin, args.err_steps,
                                 f"seeded theta' 1e-3 N(0,1) sin(pi Z) (PCG64 seed 0), {args.spinup} plain "
                                 "FP64 steps")
    del lin
    # precision study 2: a convecting state (the timed steps start from it too)
    state, conv_desc = convecting_state(S, grid, args.convect_nz, args.convect_steps, args.settle_steps)
    study_conv = _precision_study(S, grid, state, args.err_steps, conv_desc)
    torch.cuda.synchronize()
    t_studies = time.perf_counter() - t0
    log(f"[rank {rank}] precision studies: {t_studies:.1f}s")

    clocks = ClockSampler(local)
    clocks.start()
    ms_plain, prof_plain = _timed_arm(S, grid, eng, S.State(*(t.clone() for t in state)), "fp64", args, ws)
    ms_mixed, prof_mixed = _timed_arm(S, grid, eng, state, "mixed", args, ws)
    tc = eng.tensor_core_vertical
    ms_dct = None
    if tc:  # the same mixed step with the vertical transforms on the CUDA cores (FP32 DCT)
        eng.tensor_core_vertical = False
        ms_dct, _ = _timed_arm(S, grid, eng, S.State(*(t.clone() for t in state)), "mixed", args, ws,
                               label="mixed_dct")
        eng.tensor_core_vertical = True
    clk = clocks.stop()
    finite = all(bool(torch.isfinite(torch.view_as_real(t) if t.is_complex() else t).all()) for t in state)
    value = ws * args.steps / (ms_mixed * 1e-3)
    value_plain = ws * args.steps / (ms_plain * 1e-3)

    e2e = _e2e(S, grid, state, max(1, min(args.steps, 10)), ws)

    if rank != 0:
        return None
    roof_mixed = _roofline(prof_mixed, grid, args.steps, peaks)
    roof_plain = _roofline(prof_plain, grid, args.steps, peaks)
    dom = dominant_roofline(prof_mixed, roof_mixed, (args.nx, args.nz, args.rule), peaks)

    line = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": max(3, args.warmup),
        "ms_per_step": round(ms_mixed / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32 products + tf32x3 tensor-core vertical transforms + double-float (f32 pair) "
                  "column algebra and corrector + f64 solves"),
        "data": f"synthetic: {conv_desc}",
        "config": {"workload": workload_name(args.nx, args.nz, args.rule), "path": "mixed", "Nx": args.nx, "Nz": args.nz,
                   "timed": "one step_inplace call of `steps` steps on a device-resident state",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                   "l2": "state and per-step traffic >> 129 MB L2; no flush needed"},
        "plain_fp64": {"value": round(value_plain, 4), "unit": "steps/s",
                       "ms_per_step": round(ms_plain / args.steps, 4),
                       "kernels": _shares(prof_plain, args.steps), "roofline": roof_plain},
        "mixed_over_plain": round(value / value_plain, 3),
        "vertical_transforms": ("tcgen05 kind::tf32 tensor cores, TF32 hi/lo split operands (3 products), "
                                "FP32 accumulation" if tc else "FP32 fast DCT-I on the CUDA cores"),
        "mixed_cuda_core_dct": (None if ms_dct is None else
                                {"value": round(ws * args.steps / (ms_dct * 1e-3), 4), "unit": "steps/s",
                                 "ms_per_step": round(ms_dct / args.steps, 4)}),
        "rel_err_vs_plain": study_conv,
        "precision_study_linear_spinup": study_lin,
        "simulated_time_per_wall_hour": round(3600.0 * cfgd["dt"] * value / ws, 6),
        "gpu_launches": sum(n for n, _ in prof_mixed.values()),
        "roofline": dom,
        "kernels": _shares(prof_mixed, args.steps),
        "roofline_by_kernel": roof_mixed,
        "autotuned_tiles_kib": tiles,
        "peaks": {"fp64_tflops": round(peaks["fp64"], 4), "fp32_tflops": round(peaks["fp32"], 3),
                  "hbm_gbs": peaks["hbm"], "fp32_nominal_tflops": round(NOMINAL_FP32_TFLOPS, 1)},
        "clocks": clk,
        "e2e": e2e,
        "finite": finite,
    }
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference(cfgd)
    line["setup_s"] = {"grid": round(t_grid, 2), "precision_studies": round(t_studies, 1)}
    return line


POLAR_METRIC = "NHQG steps/s at 256^2x32 polar trap: mixed-precision and plain FP64 on GB300"
POLAR_NAME = ("256^2x32 polar trap ARS222, evolve_mean balanced_sbp2_pc sub4, flux, 2/3 rule, L=24Lc, Ra=100, "
              "dt=5e-5, gamma=2.2e-3, trap_r_star=0.4L, trap_sharpness=20, sponge_rate=50, sponge_r_start=52, "
              "sponge_sharpness=30, Neumann w top")


def polar_workload() -> dict:
    """The polar-trap configuration: 256^2 x 32, L = 24 L_c, Ra = 100,
    dt = 5e-5, radial background-PV trap gamma = 2.2e-3 with the Rayleigh
    sponge outside it, Neumann w at the top, evolve_mean + balanced SBP2-PC
    (4 substeps).  Trap radius and sponge are the production-scaled values
    (the default trap radius fails the eta resolution guard at this size)."""
    L = 24 * L_C
    c = workload(256, 32)
    c.update(L=L, dt=5e-5, gamma=2.2e-3, w_bc_top="neumann", trap_r_star=0.4 * L, trap_sharpness=20.0,
             sponge_rate=50.0, sponge_r_start=52.0, sponge_sharpness=30.0)
    return c


def run_polar(args, ws, rank, local):
    """Polar-trap configuration: plain and mixed steps/s on a device-resident
    state, a --polar-steps run of each from the seeded theta' start (finite,
    diagnostics, mixed against plain), end to end through imex_step_many."""
    import torch
    from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state
    from nhqg_gb300 import solver as S
    from nhqg_gb300.diagnostics import compute_diagnostics
    from nhqg_gb300.engine import engine_for

    cfgd = polar_workload()
    t0 = time.perf_counter()
    grid = make_grid(NHQGConfig(**cfgd))
    t_grid = time.perf_counter() - t0
    eng = engine_for(grid)
    peaks = {"fp64": dgemm_peak_tflops(), "fp32": sgemm_peak_tflops(), "hbm": measured_hbm_gbs()}
    s0 = S.to_device(theta_perturbation_state(grid, seed=0))
    # the configuration's run from the seeded start, both paths
    runs = {}
    for prec in ("fp64", "mixed"):
        s = S.State(*(t.clone() for t in s0))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        S.step_inplace(s, grid, args.polar_steps, check=True, precision=prec)
        e1.record()
        torch.cuda.synchronize()
        fin = all(bool(torch.isfinite(torch.view_as_real(t) if t.is_complex() else t).all()) for t in s)
        runs[prec] = (s, e0.elapsed_time(e1), fin)
    names = ("q_hat", "w_hat", "th_hat", "th_bar")
    err = {n: _rel(a, b) for n, a, b in zip(names, runs["mixed"][0], runs["fp64"][0])}
    diag = {p: compute_diagnostics(runs[p][0], grid) for p in runs}
    state = runs["fp64"][0]
    clocks = ClockSampler(local)
    clocks.start()
    ms_plain, prof_plain = _timed_arm(S, grid, eng, S.State(*(t.clone() for t in state)), "fp64", args, ws)
    ms_mixed, prof_mixed = _timed_arm(S, grid, eng, S.State(*(t.clone() for t in state)), "mixed", args, ws)
    clk = clocks.stop()
    e2e = _e2e(S, grid, state, max(1, min(args.steps, 10)), ws)
    if rank != 0:
        return None
    value = ws * args.steps / (ms_mixed * 1e-3)
    value_plain = ws * args.steps / (ms_plain * 1e-3)
    roof_mixed = _roofline(prof_mixed, grid, args.steps, peaks)
    dom = dominant_roofline(prof_mixed, roof_mixed, (256, 32, "polar"), peaks)
    keys = ("Nusselt", "Nusselt_dealiased", "KE_tot", "w_rms", "th_rms", "th_bar_max")
    line = {
        "metric": POLAR_METRIC, "value": round(value, 4), "unit": "steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": round(ms_mixed / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 products + f32 DCT vertical transforms (open-top w basis) + double-float column algebra "
                 "and corrector + f64 solves",
        "data": f"synthetic: seeded theta' 1e-3 N(0,1) sin(pi Z) (PCG64 seed 0), {args.polar_steps} plain steps",
        "config": {"workload": POLAR_NAME, "path": "mixed", "Nx": 256, "Nz": 32,
                   "timed": "one step_inplace call of `steps` steps on a device-resident state",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                   "l2": "state 60 MB < L2 at this size; per-step traffic (intermediates, tables) > L2"},
        "plain_fp64": {"value": round(value_plain, 4), "unit": "steps/s", "ms_per_step": round(ms_plain / args.steps, 4),
                       "kernels": _shares(prof_plain, args.steps)},
        "mixed_over_plain": round(value / value_plain, 3),
        f"run_{args.polar_steps}_steps": {
            p: {"finite": runs[p][2], "ms_per_step": round(runs[p][1] / args.polar_steps, 4),
                "diagnostics": {k: diag[p][k] for k in keys}} for p in runs},
        f"mixed_vs_plain_after_{args.polar_steps}_steps": err,
        "simulated_time_per_wall_hour": round(3600.0 * cfgd["dt"] * value / ws, 6),
        "gpu_launches": sum(n for n, _ in prof_mixed.values()),
        "roofline": dom, "kernels": _shares(prof_mixed, args.steps),
        "clocks": clk, "e2e": e2e,
        "setup_s": {"grid": round(t_grid, 2)},
    }
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference(cfgd, label=POLAR_NAME)
    return line


ENSEMBLE_CLASSES = ((64, 32), (96, 48), (128, 64))  # 16 members each


def ensemble_configs(seed: int = 0):
    """The batched-ensemble workload: 16 x 64^2x32, 16 x 96^2x48, 16 x 128^2x64,
    L = 10 L_c, dt = 5e-5, Ra ~ U(40, 120) per member from default_rng(seed),
    production recipe (evolve_mean + SBP2-PC, 4 substeps)."""
    rng = np.random.default_rng(seed)
    ras = rng.uniform(40.0, 120.0, 16 * len(ENSEMBLE_CLASSES))
    out = []
    for ci, (nx, nz) in enumerate(ENSEMBLE_CLASSES):
        for j in range(16):
            c = workload(nx, nz)
            c.update(Ra_tilde=float(ras[16 * ci + j]), dt=5e-5)
            out.append(c)
    return out


def run_ensemble(args, ws, rank):
    """48 independent instances advanced by one CUDA graph per
    `steps_per_launch` steps, against the same members stepped one after
    another through the single-instance API."""
    import torch
    from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state
    from nhqg_gb300 import solver as S
    from nhqg_gb300.ensemble import Ensemble

    t0 = time.perf_counter()
    cfgs = ensemble_configs()
    grids = [make_grid(NHQGConfig(**c)) for c in cfgs]
    states = [S.to_device(theta_perturbation_state(g, seed=i)) for i, g in enumerate(grids)]
    t_build = time.perf_counter() - t0
    results = {}
    for prec in ("fp64", "mixed"):
        ens = Ensemble(grids, precision=prec, steps_per_launch=10, autotune=True)
        for i, st in enumerate(states):
            ens.load(i, st)
        ens.step(max(3, args.warmup))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.step(args.steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        for i, eng in enumerate(ens.engines):
            if eng.device_status() != 0:
                raise RuntimeError(f"device status set for member {i}")
        tiles = {f"{k[0]}^2x{k[1]} {k[2]}": v for k, v in ens.tiles.items()}
        ens.close()
        # the same members one after another, each through step_inplace on one stream
        seq = [S.State(*(t.clone() for t in st)) for st in states]
        for g, st in zip(grids, seq):
            S.step_inplace(st, g, max(3, args.warmup), precision=prec)
        torch.cuda.synchronize()
        n_seq = max(1, args.steps // 10)
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record()
        for g, st in zip(grids, seq):
            S.step_inplace(st, g, n_seq, precision=prec)
        s1.record()
        torch.cuda.synchronize()
        ms_seq = s0.elapsed_time(s1)
        results[prec] = {
            "instance_steps_per_s": round(len(grids) * args.steps / (ms * 1e-3), 2),
            "ms_per_ensemble_step": round(ms / args.steps, 4),
            "sequential_instance_steps_per_s": round(len(grids) * n_seq / (ms_seq * 1e-3), 2),
            "batching_speedup": round((len(grids) * args.steps / ms) / (len(grids) * n_seq / ms_seq), 3),
            "autotuned_tiles_kib": tiles,
        }
        del seq
    if rank != 0:
        return None
    return {
        "metric": "NHQG ensemble instance-steps/s: 48 instances (16 x 64^2x32, 16 x 96^2x48, "
                  "16 x 128^2x64), one CUDA graph per 10 steps",
        "value": results["mixed"]["instance_steps_per_s"], "unit": "instance-steps/s",
        "n_gpus": ws, "steps": args.steps, "warmup": max(3, args.warmup),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "mixed (value); fp64 in fp64", "data": "synthetic: seeded theta' per member (seed = index)",
        "config": {"workload": "ensemble 16x64^2x32 + 16x96^2x48 + 16x128^2x64, L=10Lc, dt=5e-5, "
                               "Ra~U(40,120) default_rng(0), evolve_mean SBP2-PC sub4",
                   "members": len(grids)},
        "fp64": results["fp64"], "mixed": results["mixed"], "grid_build_s": round(t_build, 1),
    }


def _tail_fraction(g, q_hat, n0: int) -> float:
    """psi-KE fraction above Chebyshev mode n0: sum_{n>n0} sum_k w_k k^2 |psi_n|^2
    over sum_n (...), half-plane weights w_k (1 at ky = 0 and Nyquist, else 2)."""
    import torch
    ksq = torch.from_numpy(np.asarray(g.ksq)).to(q_hat.device)
    idn = torch.from_numpy(np.asarray(g.inv_denom)).to(q_hat.device)
    w = torch.full_like(ksq, 2.0)
    w[:, 0] = 1.0
    w[:, -1] = 1.0
    e = (w * ksq * idn ** 2)[None] * q_hat.abs() ** 2
    per_n = e.sum(dim=(1, 2))
    return float(per_n[n0 + 1:].sum() / per_n.sum())


def run_closure(args, ws, rank):
    """Learned vertical-tail closure, reduced form of its study: fine runs at
    128^2x256 (the closure's data source), coarse runs at 128^2x64 with and
    without the closure, on the first 64 Chebyshev modes of q."""
    import torch
    from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state
    from nhqg_gb300 import closure as CL
    from nhqg_gb300 import solver as S
    from nhqg_gb300.diagnostics import compute_diagnostics
    from nhqg_gb300.engine import Engine

    def cfg(nz):
        c = workload(128, nz)
        c.update(dt=5e-5)
        return c
    fine, coarse = make_grid(NHQGConfig(**cfg(256))), make_grid(NHQGConfig(**cfg(64)))
    base = None
    if args.closure_spinup > 0:
        # one spun-up fine state (mixed step: 1e-11 of the plain one) from
        # which every run branches with its own seeded theta' perturbation
        base = S.to_device(theta_perturbation_state(fine, seed=1000, amplitude=args.closure_amp))
        S.step_inplace(base, fine, args.closure_spinup, check=True, precision="mixed")
    runs = []
    for r in range(args.closure_runs):
        s = S.to_device(theta_perturbation_state(fine, seed=r, amplitude=args.closure_amp))
        if base is not None:
            s = S.sanitize_state(S.State(base.q_hat.clone(), base.w_hat.clone(),
                                         base.th_hat + 1e-2 * s.th_hat, base.th_bar.clone()), fine)
        snaps = []
        for _ in range(args.closure_steps // 40):
            S.step_inplace(s, fine, 40)
            snaps.append(S.State(*(x.clone() for x in s)))
        runs.append(snaps)
    train = [st for run in runs[:-1] for st in run]
    held = runs[-1]
    data, sc = CL.training_columns(fine, coarse, train, ncoef=64)
    hdata, _ = CL.training_columns(fine, coarse, held, scales=sc)
    model = CL.TailClosure(sc, seed=0)
    zero_h = model.evaluate(hdata["x"], hdata["q"], hdata["t"])
    t0 = time.perf_counter()
    hist = model.fit(data, epochs=args.closure_epochs, batch=2048, lr=1e-3)
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    train_ratio = hist[-1] / hist[0] if hist[0] > 0 else None
    held_ratio = model.evaluate(hdata["x"], hdata["q"], hdata["t"]) / zero_h
    # a posteriori: from the first held-out snapshot, fine vs coarse with / without the closure
    k = args.closure_post_steps
    s_f = S.State(*(x.clone() for x in held[0]))
    s_plain = S.State(*(x.clone() for x in CL.truncate(held[0], coarse)))
    s_cl = S.State(*(x.clone() for x in s_plain))
    e_plain, e_cl = Engine(coarse), Engine(coarse)
    model.attach(e_cl)
    S.step_inplace(s_f, fine, k)
    e_plain.step(*s_plain, n_steps=k)
    e_cl.step(*s_cl, n_steps=k)
    ref = s_f.q_hat[:coarse.Nz + 1]
    err = lambda s: float(torch.linalg.norm(s.q_hat - ref) / torch.linalg.norm(ref))  # noqa: E731
    diag = {lab: compute_diagnostics(st, g) for lab, st, g in
            (("fine", s_f, fine), ("coarse", s_plain, coarse), ("coarse_closure", s_cl, coarse))}
    pick = lambda key: {lab: d[key] for lab, d in diag.items()}  # noqa: E731
    if rank != 0:
        return None
    return {
        "metric": "learned q-tail closure at 128^2x64 vs 128^2x256: held-out a-priori error ratio",
        "value": round(held_ratio, 4), "unit": "ratio (closure / no closure)", "n_gpus": ws,
        "higher_is_better": False, "vs_baseline": None, "dtype": "bf16 weights, fp32 accumulation",
        "data": (f"{args.closure_runs} fine runs of {args.closure_steps} steps from seeded theta' "
                 f"(amplitude {args.closure_amp}"
                 + (f", added at 1e-2 to a state spun up for {args.closure_spinup} steps"
                    if args.closure_spinup > 0 else "")
                 + "), snapshots every 40 steps; the last run held out"),
        "config": {"workload": "closure study, fine 128^2x256, coarse 128^2x64, ncoef 64, dt=5e-5, "
                               "evolve_mean SBP2-PC sub4", "params": CL.n_params()},
        "train_loss_first_last_epoch": [round(hist[0], 5), round(hist[-1], 5)],
        "train_ratio": None if train_ratio is None else round(train_ratio, 4),
        "fit_seconds": round(t_fit, 2), "columns": int(data["x"].shape[0]),
        "a_posteriori": {"steps": k, "q_rel_err_no_closure": err(s_plain), "q_rel_err_closure": err(s_cl),
                         "tail_fraction_above_48": {"fine": _tail_fraction(fine, ref, 48),
                                                    "coarse": _tail_fraction(coarse, s_plain.q_hat, 48),
                                                    "coarse_closure": _tail_fraction(coarse, s_cl.q_hat, 48)},
                         "Nusselt": pick("Nusselt"), "KE_tot": pick("KE_tot")},
    }


def run_reference(args, ws, rank):
    """CPU arm: whole steps of the oracle port of the reference step on the
    host cores, on this arm's workload, metric and units; rank 0 only."""
    if rank != 0:
        return None
    if args.config == "polar":
        cfgd, metric, wname = polar_workload(), POLAR_METRIC, POLAR_NAME
    else:
        cfgd, metric = workload(args.nx, args.nz, args.rule), METRIC
        wname = workload_name(args.nx, args.nz, args.rule)
    cb = cpu_reference(cfgd, steps=args.steps, warmup=args.warmup, label=wname)
    cb["value"] = round(cb["value"], 6)  # the line's value
    return {
        "metric": metric, "value": cb["value"], "unit": "steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 / cb["value"], 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded theta' start)", "impl": "reference",
        "config": {"workload": wname, "path": "cpu_port", "Nx": cfgd["Nx"], "Nz": cfgd["Nz"],
                   "parallelism": "host cores"},
        "cpu_baseline": cb,
        "e2e": {"value": round(cb["value"], 6), "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--rule", default="23_rule", choices=["23_rule", "32_rule"],
                    help="horizontal dealiasing of the workload (the headline uses the 2/3 rule)")
    ap.add_argument("--config", default="headline", choices=["headline", "polar"],
                    help="headline: 256^2x256 (the metric's configuration); polar: the 256^2x32 "
                         "polar-trap configuration (its own JSON line)")
    ap.add_argument("--spinup", type=int, default=5000,
                    help="plain FP64 steps from the seeded 1e-3 theta' start before the first precision "
                         "study (the configuration's 5000)")
    ap.add_argument("--convect-nz", type=int, default=64,
                    help="Nz of the coarse grid (Nx/2) the convecting state is spun up on")
    ap.add_argument("--convect-steps", type=int, default=8000,
                    help="mixed steps (dt=5e-5) of the coarse spin-up from a seeded theta' of amplitude 1")
    ap.add_argument("--settle-steps", type=int, default=200,
                    help="plain steps on the full grid after the prolongation")
    ap.add_argument("--polar-steps", type=int, default=2000,
                    help="steps of the polar configuration's run from the seeded start")
    ap.add_argument("--err-steps", type=int, default=500,
                    help="steps of the mixed-vs-plain accuracy comparison")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in horizontal-product tiles")
    ap.add_argument("--closure", action="store_true",
                    help="run the learned-closure study instead (its own JSON line)")
    ap.add_argument("--closure-runs", type=int, default=3)
    ap.add_argument("--closure-steps", type=int, default=800)
    ap.add_argument("--closure-amp", type=float, default=0.1)
    ap.add_argument("--closure-epochs", type=int, default=30)
    ap.add_argument("--closure-post-steps", type=int, default=200)
    ap.add_argument("--closure-spinup", type=int, default=30000,
                    help="fine steps (mixed precision) to a common spun-up state the runs branch from")
    ap.add_argument("--ensemble", action="store_true",
                    help="time the 48-member batched ensemble instead (its own JSON line)")
    args = ap.parse_args()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        line = run_reference(args, ws, rank)
    elif args.config == "polar":
        line = run_polar(args, ws, rank, local)
    elif args.ensemble:
        line = run_ensemble(args, ws, rank)
    elif args.closure:
        line = run_closure(args, ws, rank)
    else:
        line = run_ours(args, ws, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
