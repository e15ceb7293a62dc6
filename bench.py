#!/usr/bin/env python
"""NHQG time-step benchmark on GB300 (steps/s at 256^2 x 256).

Workload (the headline configuration): Nx=Ny=256, Nz=256, L = 10 L_c
(L_c = 2 pi / 1.3048), Ra~=100, Pr=1, nu=1 (Laplacian), dt=2e-5, flux-form
advection, 2/3-rule dealiasing, evolve_mean closure with the balanced SBP2
predictor/corrector (4 substeps), float64, ARS(2,2,2).  Input: the seeded
theta' start (1e-3 N(0,1) sin(pi Z), PCG64 seed 0) -- synthetic; the
5000-step spin-up of the precision study is not run (the step's work does
not depend on the state).  Every step streams several GB, far above the
129 MB L2, so no explicit L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The default arm times the plain FP64 GPU step; ``--impl reference`` times the
CPU port of the reference algorithm (NumPy/SciPy on all host cores) on the
same workload.  One JSON line on stdout (rank 0).
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


def workload(nx: int, nz: int) -> dict:
    return dict(Nx=nx, Nz=nz, L=10 * L_C, Ra_tilde=100.0, sigma=1.0, nu_q=1.0, nu_w=1.0,
                nu_theta=1.0, hyper_order=1, dt=2e-5, nonlinear_advection="flux",
                horizontal_dealiasing="23_rule", float_dtype="float64",
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
def kernel_work(name: str, g, launches: int) -> tuple[float, float]:
    """(FP64 flops, algorithmic DRAM bytes) per launch for the algorithm the
    engine runs.  FFT: 5 n log2 n flops per complex length-n transform; dense
    vertical transforms: 4 P^2 flops per complex column; shell solve 4 G^2."""
    Nx, P, G = g.Nx, g.Nz + 1, g.Nz - 1
    K = Nx // 3
    Mc, Mr = K + 1, 2 * K + 1
    M = Mr * Mc
    fft = 5.0 * Nx * math.log2(Nx)
    cplx = 16.0
    field = P * M * cplx
    if name == "h1_col_ifft":
        return 5 * Mc * P * fft, 3 * field + 5 * P * Mc * Nx * cplx
    if name == "h2_row_products":
        return (5 + 6) * (Nx / 2) * P * fft + 6 * Nx * Nx * P, (5 + 6) * P * Mc * Nx * cplx
    if name == "h3_col_fft":
        return 6 * Mc * P * fft, 6 * P * Mc * Nx * cplx + 3 * field
    if name == "vfwd":
        nf = 3 if launches <= 1 else 2  # 3 fields at stage 1, 1 at stage 2 (mean)
        return nf * 4.0 * P * P * M, 2 * nf * field
    if name in ("vback_stage1", "vback_stage2"):
        return 3 * 4.0 * P * P * M, 12 * field
    if name == "shell_solve":
        n_in = len(np.unique(g.imex_shell_row[g.imex_shell_row >= 0]))
        return 4.0 * G * G * M, 2 * field + n_in * G * G * 8.0
    if name == "corr_pre":
        return 2 * 4.0 * P * P * M, 5 * field
    if name == "corr_sub":
        return 4.0 * P * G * M / 4.0, 4 * field
    return 0.0, 0.0


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


# ------------------------------------------------------------------ CPU (oracle) arm
def cpu_reference(cfgd: dict) -> dict:
    """Time the NumPy/SciPy port of the reference step on all host cores.

    A full oracle step at 256^2 x 256 is minutes of CPU time, so the sample is
    one evaluation of each operator of the step and the step time is their
    sum weighted by how often one ARS(2,2,2) + SBP2-PC step calls them:
    2 x explicit RHS, 2 x implicit solve, 1 x implicit tendency,
    2 x SBP2 corrector (4 substeps each), 3 x stage combination.  The per-shell
    table build (reference make_grid work) is excluded, as on the GPU side."""
    import oracle
    from oracle.nhqg_oracle import OracleConfig, OracleState
    cores = os.cpu_count() or 1
    oracle.nhqg_oracle.set_threads(cores)
    g = oracle.make_grid(OracleConfig(**cfgd), with_shell_inverses=False)
    base = g.replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    s = oracle.theta_perturbation_state(g, seed=0)
    t0 = time.perf_counter()
    oracle.imex_implicit_solve(s.q_hat, s.w_hat, s.th_hat, base)  # builds the shell table
    t_table = time.perf_counter() - t0
    oracle.explicit_rhs(s, base)  # warm-up (FFT plans, BLAS pools)

    def timed(fn):
        t = time.perf_counter()
        out = fn()
        return time.perf_counter() - t, out

    tE, E = timed(lambda: oracle.explicit_rhs(s, base))
    tI, _ = timed(lambda: oracle.implicit_tendency(s, base))
    tS, _ = timed(lambda: oracle.imex_implicit_solve(s.q_hat, s.w_hat, s.th_hat, base))
    alpha = g.gamma_imex * g.dt
    tC, _ = timed(lambda: oracle.apply_balanced_sbp2_corrector(s, g, alpha))
    tX, _ = timed(lambda: OracleState(*(a + alpha * e for a, e in zip(s, E))))
    t_step = 2 * tE + 2 * tS + tI + 2 * tC + 3 * tX
    return {"value": 1.0 / t_step, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": (f"one evaluation of each step operator at {cfgd['Nx']}^2x{cfgd['Nz']} "
                       f"(RHS {tE:.1f}s, implicit solve {tS:.1f}s, implicit tendency {tI:.1f}s, "
                       f"SBP2 corrector {tC:.1f}s, stage combination {tX:.2f}s) summed as "
                       "2E+2S+I+2C+3X; shell-table build excluded "
                       f"({t_table:.0f}s); NumPy/SciPy execution of the reference algorithm (not XLA)")}


# ------------------------------------------------------------------ GPU arm
def run_ours(args, ws, rank, local):
    import torch
    from nhqg_gb300 import NHQGConfig, make_grid, theta_perturbation_state
    from nhqg_gb300 import solver as S
    from nhqg_gb300.engine import engine_for

    cfgd = workload(args.nx, args.nz)
    t0 = time.perf_counter()
    grid = make_grid(NHQGConfig(**cfgd))
    t_grid = time.perf_counter() - t0
    log(f"[rank {rank}] grid {args.nx}^2x{args.nz}: {t_grid:.1f}s, {grid.imex_inv.shape[0]} shells")
    host0 = theta_perturbation_state(grid, seed=0)
    state = S.to_device(host0)
    eng = engine_for(grid)
    peak = dgemm_peak_tflops() if rank == 0 else None
    S.step_inplace(state, grid, max(3, args.warmup), check=True)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    eng.profile(True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        S.step_inplace(state, grid, 1)
    e1.record()
    torch.cuda.synchronize()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    prof = eng.profile_report()
    eng.profile(False)
    clk = clocks.stop()
    if eng.device_status() != 0:
        raise RuntimeError("device status set during the timed region")
    finite = all(bool(torch.isfinite(torch.view_as_real(t) if t.is_complex() else t).all()) for t in state)
    ms_max = allmax(ms, ws)
    value = ws * args.steps / (ms_max * 1e-3)

    # end to end through the public API with pinned host buffers
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in host0]
    outs = [torch.empty_like(p).pin_memory() for p in pinned]
    S.imex_step(pinned, grid)
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 10))
    barrier(ws)
    ee0 = torch.cuda.Event(enable_timing=True)
    ee1 = torch.cuda.Event(enable_timing=True)
    ee0.record()
    for _ in range(e2e_steps):
        res = S.imex_step(pinned, grid)
        for o, r in zip(outs, res):
            o.copy_(r, non_blocking=True)
    ee1.record()
    torch.cuda.synchronize()
    e2e_ms = allmax(ee0.elapsed_time(ee1), ws)
    bytes_state = int(sum(p.numel() * p.element_size() for p in pinned))

    if rank != 0:
        return None
    launches = sum(n for n, _ in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    dname, (dn, dms) = dom
    flops, bytes_ = kernel_work(dname, grid, dn // max(1, args.steps))
    avg_ms = dms / dn
    achieved = flops / (avg_ms * 1e-3) / 1e12
    kernels = {k: {"launches": n, "ms_per_step": round(t / args.steps, 4),
                   "share": round(t / sum(v[1] for v in prof.values()), 4)} for k, (n, t) in prof.items()}
    line = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": max(3, args.warmup),
        "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded theta' 1e-3 N(0,1) sin(pi Z), PCG64 seed 0; no spin-up)",
        "config": {"workload": f"{args.nx}^2x{args.nz} plain FP64 ARS222, balanced_sbp2_pc sub4, "
                               "flux, 2/3 rule, L=10Lc, Ra=100, dt=2e-5",
                   "path": "plain_fp64", "Nx": args.nx, "Nz": args.nz,
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                   "l2": "state and per-step traffic >> 129 MB L2; no flush needed"},
        "simulated_time_per_wall_hour": round(3600.0 * cfgd["dt"] * value / ws, 6),
        "gpu_launches": launches,
        "roofline": {"kernel": dname, "bound": "fp64", "achieved": round(achieved, 4),
                     "peak": round(peak, 4), "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
                     "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (FP64 pipe; "
                                    "MEASURED_PEAKS.json has no FP64 figure)",
                     "flops_per_launch": flops, "avg_launch_ms": round(avg_ms, 4),
                     "hbm_gbs_at_algorithmic_bytes": round(bytes_ / (avg_ms * 1e-3) / 1e9, 1),
                     "traffic": None},
        "kernels": kernels,
        "clocks": clk,
        "e2e": {"value": round(ws * e2e_steps / (e2e_ms * 1e-3), 4), "unit": "steps/s",
                "h2d_bytes_per_step": bytes_state, "d2h_bytes_per_step": bytes_state,
                "api": "nhqg_gb300.solver.imex_step(pinned host State) + D2H of the result"},
        "finite": finite,
        "grid_build_s": round(t_grid, 2),
    }
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference(cfgd)
    return line


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    cfgd = workload(args.nx, args.nz)
    cb = cpu_reference(cfgd)
    return {
        "metric": METRIC, "value": round(cb["value"], 6), "unit": "steps/s", "n_gpus": ws,
        "steps": 1, "warmup": 1, "ms_per_step": round(1e3 / cb["value"], 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded theta' start)", "impl": "reference",
        "config": {"workload": f"{args.nx}^2x{args.nz} plain FP64 ARS222, balanced_sbp2_pc sub4, "
                               "flux, 2/3 rule, L=10Lc, Ra=100, dt=2e-5", "path": "cpu_port"},
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
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        line = run_reference(args, ws, rank)
    else:
        line = run_ours(args, ws, rank, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
