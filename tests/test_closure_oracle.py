"""Pin the closure oracle (oracle/closure_oracle.py) by central finite
differences of its loss, and its BF16 rounding by known values."""

import numpy as np

from oracle import closure_oracle as co


def _batch(rng, B=12):
    x = rng.standard_normal((B, co.N_IN))
    q = rng.standard_normal((B, co.N_OUT)) + 1j * rng.standard_normal((B, co.N_OUT))
    t = rng.standard_normal((B, co.N_OUT)) + 1j * rng.standard_normal((B, co.N_OUT))
    return x, q, t


def test_bf16_round():
    a = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, -2.5, 3.0e-3], dtype=np.float32)
    got = co.bf16_round(a)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even -> 1; 1 + 3*2^-9 rounds up
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 and got[3] == np.float32(1.0078125)
    assert got[4] == -2.5
    assert abs(got[5] - 3.0e-3) <= 2 ** -8 * 3.0e-3


def test_gradient_by_finite_differences():
    rng = np.random.default_rng(4)
    flat = 0.2 * rng.standard_normal(co.N_PARAMS)
    p = co.unflatten(flat)
    x, q, t = _batch(rng)
    s, tnorm = 0.7, 3.0
    _, g = co.loss_and_grad(p, x, q, t, s, tnorm)
    gflat = co.flatten(g)
    h = 1e-6
    for idx in rng.choice(co.N_PARAMS, 40, replace=False):
        fp, fm = flat.copy(), flat.copy()
        fp[idx] += h
        fm[idx] -= h
        lp, _ = co.loss_and_grad(co.unflatten(fp), x, q, t, s, tnorm)
        lm, _ = co.loss_and_grad(co.unflatten(fm), x, q, t, s, tnorm)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gflat[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, gflat[idx])
