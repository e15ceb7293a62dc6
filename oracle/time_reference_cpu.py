"""Same-machine step time of the reference source and of the oracle port.

Test infrastructure: run by hand in a checkout where the NHQG reference
source is available (it is not needed by the tests or the benchmark)::

    python oracle/time_reference_cpu.py /path/to/NHQG 64 32 5
    python oracle/time_reference_cpu.py /path/to/NHQG 256 256 2 --chunk 64

It times whole ``imex_step`` calls on the benchmark recipe (evolve_mean +
balanced SBP2-PC, 4 substeps, flux form, 2/3 rule, L = 10 L_c, Ra = 100,
dt = 2e-5) from the seeded theta' start, first of the unmodified reference
source (``nhqg/*.py``) executed under the NumPy stand-in for ``jax`` in
``tests/golden/refshim`` (jit = identity; ``imex_matmul_chunk`` as given),
then of this directory's NumPy/SciPy restatement, each after one untimed
step and with the grid / shell tables built beforehand.  The benchmark's
CPU baseline is the restatement (the reference source cannot travel to the
GPU host); this script shows how the two compare on one machine.
"""

from __future__ import annotations

import argparse
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def _time_steps(step, s, n):
    s = step(s)  # untimed
    t = []
    for _ in range(n):
        t0 = time.perf_counter()
        s = step(s)
        t.append(time.perf_counter() - t0)
    return float(np.median(t))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("reference")
    ap.add_argument("nx", type=int)
    ap.add_argument("nz", type=int)
    ap.add_argument("steps", type=int)
    ap.add_argument("--chunk", type=int, default=0, help="the reference's imex_matmul_chunk")
    args = ap.parse_args()
    import bench
    cfgd = bench.workload(args.nx, args.nz)

    sys.path.insert(0, str(ROOT / "tests" / "golden" / "refshim"))
    sys.path.insert(0, args.reference)
    from nhqg import solver  # noqa: E402
    from nhqg.config import NHQGConfig  # noqa: E402
    from nhqg.grid import make_grid  # noqa: E402
    import jax.numpy as jnp  # the stand-in  # noqa: E402

    rcfg = dict(cfgd)
    if args.chunk:
        rcfg["imex_matmul_chunk"] = args.chunk
    t0 = time.perf_counter()
    g = make_grid(NHQGConfig(**rcfg))
    t_grid_ref = time.perf_counter() - t0
    P, nx = args.nz + 1, args.nx
    rng = np.random.default_rng(0)
    th = 1e-3 * rng.standard_normal((P, nx, nx)) * np.sin(np.pi * np.asarray(g.Z))[:, None, None]
    th_cheb = np.einsum("ij,j...->i...", np.asarray(g.V_inv), np.fft.rfft2(th))
    th_gal = np.einsum("ij,j...->i...", np.asarray(g.dirichlet_pinv), th_cheb)
    s = solver.State(jnp.asarray(np.zeros((P, nx, nx // 2 + 1), complex)),
                     jnp.asarray(np.zeros_like(th_gal)), jnp.asarray(th_gal), jnp.asarray(np.zeros(P)))
    s = solver.sanitize_state(s, g)
    t_ref = _time_steps(lambda x: solver.imex_step(x, g), s, args.steps)
    del g, s

    import oracle
    from oracle.nhqg_oracle import OracleConfig
    oracle.nhqg_oracle.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    o = oracle.make_grid(OracleConfig(**cfgd))
    t_grid_port = time.perf_counter() - t0
    so = oracle.theta_perturbation_state(o, seed=0)
    t_port = _time_steps(lambda x: oracle.imex_step(x, o), so, args.steps)
    print(f"{nx}^2x{args.nz}, {os.cpu_count()} host threads: reference source under the NumPy stand-in "
          f"{t_ref:.3f} s/step (grid {t_grid_ref:.1f} s), oracle port {t_port:.3f} s/step "
          f"(grid {t_grid_port:.1f} s); reference / port = {t_ref / t_port:.2f}")


if __name__ == "__main__":
    main()
