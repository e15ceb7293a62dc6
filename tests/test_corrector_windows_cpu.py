"""CPU emulation of the corrector's windowed 1-D solve (numerical method).

The corrector's substep solves A tb_new = b with the pentadiagonal
A = I - h of the balanced SBP2 exchange (nhqg/solver.py:873-906;
half = mu kappa sub_dt / 2 L_sbp + mu sub_dt^2 / 4 D1 diag(<w^2>) D1, boundary
rows identity).  The GPU kernel runs FP64 iterative refinement around a
restricted additive Schwarz inverse: windows of 32 core rows widened by `ov`
rows on each side, each factored by an FP32 banded LU without pivoting.  The
host sets ov so that r^ov <= 1e-7 for the decay rate r of A^-1 (plus two rows
of margin).  This file restates that algorithm in NumPy -- FP32 factors and
substitutions in FP32 arithmetic, residuals in FP64 -- and checks that two
refinement sweeps reach FP64 round-off at the sizes and time steps in use,
that the kernel's convergence check (last correction <= 1e-10 of the
solution) passes there, and that it fails for an overlap too small to
converge (where the kernel falls back to one global factorisation).
"""

import math

import numpy as np
import pytest

from oracle.nhqg_oracle import sbp2_operators

f32 = np.float32
CORE = 32


def _overlap(N, sub_dt, mu=1.0, kappa=1.0):
    """The host's rule: r^ov <= 1e-7 plus two rows, at least 2; None past 24."""
    a = 0.5 * mu * kappa * sub_dt * N * N
    ov = 2
    if a > 0:
        r = 2 * a / ((1 + 2 * a) + math.sqrt(1 + 4 * a))
        ov = max(2, math.ceil(math.log(1e-7) / math.log(r)) + 2)
    return ov if ov <= 24 else None


def _factor(A, e0, n):
    F = np.zeros((5, n), np.float32)
    d1 = d2 = u11 = u21 = u12 = u22 = f32(0)
    for ii in range(n):
        i = e0 + ii
        a0 = f32(A[i, i - 2]) if ii >= 2 else f32(0)
        a1 = f32(A[i, i - 1]) if ii >= 1 else f32(0)
        a2 = f32(A[i, i])
        a3 = f32(A[i, i + 1]) if ii + 1 < n else f32(0)
        a4 = f32(A[i, i + 2]) if ii + 2 < n else f32(0)
        l2 = f32(a0 * d2)
        l1 = f32(f32(a1 - f32(l2 * u12)) * d1)
        piv = f32(f32(a2 - f32(l2 * u22)) - f32(l1 * u11))
        dv = f32(f32(1) / piv)
        s1 = f32(a3 - f32(l1 * u21))
        F[:, ii] = [l2, l1, dv, f32(s1 * dv), f32(a4 * dv)]
        u12, u22, u11, u21, d2, d1 = u11, u21, s1, a4, d1, dv
    return F


def _solve(F, r):
    n = len(r)
    y = np.zeros(n, np.float32)
    v1 = v2 = f32(0)
    for i in range(n):
        v = f32(f32(r[i] - f32(F[0, i] * v2)) - f32(F[1, i] * v1))
        y[i] = v
        v2, v1 = v1, v
    x = np.zeros(n, np.float32)
    x1 = x2 = f32(0)
    for j in range(n - 1, -1, -1):
        v = f32(f32(f32(y[j] * F[2, j]) - f32(F[4, j] * x2)) - f32(F[3, j] * x1))
        x[j] = v
        x2, x1 = x1, v
    return x


def _system(N, dt, w2, nsub=4):
    P = N + 1
    _, D1, L = sbp2_operators(N)
    sub = dt / nsub
    half = 0.5 * sub * L + 0.25 * sub ** 2 * (D1 @ np.diag(np.full(P, w2)) @ D1)
    A = np.eye(P) - half
    A[0, :] = 0.0
    A[-1, :] = 0.0
    A[0, 0] = A[-1, -1] = 1.0
    return A, sub


def _windowed(A, b, ov, sweeps=3):
    P = len(b)
    wins = []
    for w in range((P + CORE - 1) // CORE):
        c0, c1 = CORE * w, min(P, CORE * w + CORE)
        e0, e1 = max(0, c0 - ov), min(P, c1 + ov)
        wins.append((c0, c1, e0, e1, _factor(A, e0, e1 - e0)))
    sol = np.zeros(P)
    res = b.copy()
    last = None
    for _ in range(sweeps):
        rin = res.astype(np.float32)
        xo = np.zeros(P, np.float32)
        for c0, c1, e0, e1, F in wins:
            xo[c0:c1] = _solve(F, rin[e0:e1])[c0 - e0:c1 - e0]
        sol = sol + xo.astype(np.float64)
        last = xo
        res = b - A @ sol
    converged = float(np.abs(last).max()) <= 1e-10 * float(np.abs(sol).max())
    return sol, converged


def _rhs(A, seed):
    rng = np.random.default_rng(seed)
    P = A.shape[0]
    x = np.sin(np.linspace(0.0, 3.0, P)) + 0.01 * rng.standard_normal(P)
    x[0] = x[-1] = 0.0
    return A @ x


@pytest.mark.parametrize("N,dt,w2", [(32, 5e-5, 0.0), (64, 5e-5, 10.0), (256, 2e-5, 0.0),
                                     (256, 5e-5, 100.0), (512, 2e-5, 1.0)])
def test_windows_reach_fp64_roundoff(N, dt, w2):
    A, sub = _system(N, dt, w2)
    ov = _overlap(N, sub)
    assert ov is not None
    b = _rhs(A, N)
    sol, converged = _windowed(A, b, ov)
    exact = np.linalg.solve(A, b)
    assert np.abs(sol - exact).max() <= 2e-15 * np.abs(exact).max()
    assert converged


@pytest.mark.parametrize("N,dt,ov", [(64, 5e-5, 1), (256, 2e-5, 3)])
def test_small_overlap_fails_the_check(N, dt, ov):
    # the host's overlaps are 7 and 10 rows; these leave the windows' coupling
    # error above the check after two refinement sweeps, so the kernel falls
    # back to one global factorisation (the GPU test's 1-row case at 64 levels)
    A, sub = _system(N, dt, 0.0)
    assert _overlap(N, sub) in (7, 10)
    _, converged = _windowed(A, _rhs(A, 1), ov)
    assert not converged


def test_overlap_rule_disables_windows_for_slow_decay():
    # r close to 1 (large mu kappa sub_dt N^2): more than 24 rows would be needed
    assert _overlap(1024, 5e-4 / 4) is None
    assert _overlap(256, 2e-5 / 4) == 10
