"""Comparison helpers shared by the parity tests."""

from __future__ import annotations

import numpy as np


def rel_l2(a, b, floor: float = 0.0) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = max(float(np.linalg.norm(b)), floor)
    num = float(np.linalg.norm(a - b))
    if den == 0.0:
        return num
    return num / den


def assert_state_close(got, ref, tol, names=("q_hat", "w_hat", "th_hat", "th_bar"), floor=1e-30, th_bar_abs=None):
    for name, g, r in zip(names, got, ref):
        g = np.asarray(g)
        r = np.asarray(r)
        assert g.shape == r.shape, (name, g.shape, r.shape)
        if name == "th_bar" and th_bar_abs is not None:
            err = float(np.max(np.abs(g - r)))
            assert err <= th_bar_abs, f"{name}: abs err {err:.3e} > {th_bar_abs:.1e}"
            continue
        e = rel_l2(g, r, floor=floor)
        assert e <= tol, f"{name}: rel L2 {e:.3e} > {tol:.1e}"
