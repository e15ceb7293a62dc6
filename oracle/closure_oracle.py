"""NumPy restatement of the learned vertical-tail closure (test oracle).

TEST INFRASTRUCTURE -- see ``oracle/__init__.py``.  The closure has no
reference counterpart (an extension of the step); this file restates the model
that ``nhqg_gb300/csrc/closure.cu`` implements so that the GPU features,
forward pass and gradients can be checked, and it is itself pinned by
central finite differences in ``tests/test_closure_oracle.py``.

Per in-band mode column (Chebyshev coefficients q_n of q'):
  features f_n = log1p(|q_n|^2 / sq_n) (n < ncoef, 0 above, 64 slots),
           f_64 = |k| / kmax, f_65 = log1p(sum_n |k|^2 |psi_n|^2 / se),
           psi_n = -inv_denom q_n;
  (r, rho) = W3 tanh(W2 tanh(W1 f + b1) + b2) + b3 (66 -> 256 -> 128 -> 128);
  C_n = -s (r_n + i rho_n) q_n;  loss = sum_columns sum_n |C_n - t_n|^2 / (B tnorm).
The GPU stores the weights in BF16 and accumulates in FP32; the oracle
evaluates in FP64 with the same BF16-rounded weights.
"""

from __future__ import annotations

import numpy as np

N_IN, N_H1, N_H2, N_OUT = 66, 256, 128, 64
N_R = 2 * N_OUT
SHAPES = (("W1", (N_H1, N_IN)), ("b1", (N_H1,)), ("W2", (N_H2, N_H1)), ("b2", (N_H2,)),
          ("W3", (N_R, N_H2)), ("b3", (N_R,)))
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unflatten(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def bf16_round(a: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 with round-to-nearest-even, returned as float32."""
    b = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounded = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return (rounded.astype(np.uint32) << 16).view(np.float32)


def features(qcols: np.ndarray, ksq: np.ndarray, inv_denom: np.ndarray, sq: np.ndarray, se: float,
             kmax: float, ncoef: int) -> np.ndarray:
    """qcols: (M, 64) complex (zero beyond ncoef); returns (M, 66)."""
    a2 = np.abs(qcols[:, :N_OUT]) ** 2
    f = np.zeros((qcols.shape[0], N_IN))
    f[:, :ncoef] = np.log1p(a2[:, :ncoef] / sq[None, :ncoef])
    f[:, 64] = np.sqrt(ksq) / kmax
    ke = np.sum(ksq[:, None] * inv_denom[:, None] ** 2 * a2[:, :ncoef], axis=1)
    f[:, 65] = np.log1p(ke / se)
    return f


def forward(p: dict, x: np.ndarray):
    z1 = x @ p["W1"].T + p["b1"]
    h1 = np.tanh(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = np.tanh(z2)
    r = h2 @ p["W3"].T + p["b3"]
    return r, (h1, h2)


def closure(p: dict, x: np.ndarray, q: np.ndarray, s: float) -> np.ndarray:
    r, _ = forward(p, x)
    return -s * (r[:, :N_OUT] + 1j * r[:, N_OUT:]) * q


def loss_and_grad(p: dict, x: np.ndarray, q: np.ndarray, t: np.ndarray, s: float, tnorm: float):
    """Mean loss and its gradient (dict of arrays) for a batch (B, ...)."""
    B = x.shape[0]
    r, (h1, h2) = forward(p, x)
    e = -s * (r[:, :N_OUT] + 1j * r[:, N_OUT:]) * q - t
    inv = 1.0 / (B * tnorm)
    loss = float(np.sum(np.abs(e) ** 2) * inv)
    ecq = e * np.conj(q)
    g3 = np.concatenate([-2.0 * s * np.real(ecq), -2.0 * s * np.imag(ecq)], axis=1) * inv  # (B, 128)
    grads = {"W3": g3.T @ h2, "b3": g3.sum(0)}
    d2 = (g3 @ p["W3"]) * (1.0 - h2 ** 2)
    grads["W2"] = d2.T @ h1
    grads["b2"] = d2.sum(0)
    d1 = (d2 @ p["W2"]) * (1.0 - h1 ** 2)
    grads["W1"] = d1.T @ x
    grads["b1"] = d1.sum(0)
    return loss, grads


def flatten(d: dict) -> np.ndarray:
    return np.concatenate([np.ravel(d[name]) for name, _ in SHAPES])
