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


def assert_state_close(got, ref, tol, names=("q_hat", "w_hat", "th_hat", "th_bar"), th_bar_abs=0.0,
                       abs_floor=0.0):
    """Per field: ||got - ref|| <= tol * ||ref||, or <= an absolute floor
    (``th_bar_abs`` for th_bar, which the reference may keep at exact zero)."""
    for name, g, r in zip(names, got, ref):
        g = np.asarray(g)
        r = np.asarray(r)
        assert g.shape == r.shape, (name, g.shape, r.shape)
        err = float(np.linalg.norm(g - r))
        scale = float(np.linalg.norm(r))
        floor = th_bar_abs if name == "th_bar" else abs_floor
        assert err <= max(tol * scale, floor), (
            f"{name}: |diff| {err:.3e}, rel {err / scale if scale else float('inf'):.3e} > {tol:.1e}")
