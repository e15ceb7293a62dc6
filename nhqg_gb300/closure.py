"""Learned vertical-tail closure for q (an extension of the step with no
reference counterpart).

The closure adds C_n = -s (r_n + i rho_n) q_n to the explicit q tendency on
the first ``ncoef`` (<= 64) Chebyshev coefficients of every horizontal mode,
with the complex per-coefficient rate (r, rho) = MLP(features of the column)
-- see ``include/nhqg_gpu.h`` (nhqg_closure_*) for the features and the
network (66 -> 256 -> 128 -> 128, BF16 weights, FP32 accumulation).  Everything runs
in the project's own CUDA kernels: features, forward, backward and Adam.

Training data are a-priori pairs from solver-generated fine-Nz states: for a
fine state s on ``fine`` and its Chebyshev truncation s_c on ``coarse`` (same
Nx), the target is the q tendency the coarse model misses,
  t_n = E_q[fine](s)_n - E_q[coarse](s_c)_n,  n < ncoef,
column by column over the in-band modes.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as nat
from .engine import Engine, _stream_handle
from .grid import Grid, compact_layout
from .solver import State, explicit_rhs, to_device

N_IN, N_H1, N_H2, N_OUT = 66, 256, 128, 64
N_R = 2 * N_OUT  # complex rate per coefficient
SHAPES = (("W1", (N_H1, N_IN)), ("b1", (N_H1,)), ("W2", (N_H2, N_H1)), ("b2", (N_H2,)),
          ("W3", (N_R, N_H2)), ("b3", (N_R,)))


def n_params() -> int:
    return sum(int(np.prod(s)) for _, s in SHAPES)


def init_params(seed: int = 0, out_gain: float = 0.0) -> np.ndarray:
    """Glorot-uniform hidden layers, zero biases, output layer scaled by
    ``out_gain`` (0: the closure starts as exactly zero)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SHAPES:
        if name.startswith("b"):
            parts.append(np.zeros(shape))
            continue
        fan_out, fan_in = shape
        lim = np.sqrt(6.0 / (fan_in + fan_out))
        w = rng.uniform(-lim, lim, shape)
        parts.append(w * out_gain if name == "W3" else w)
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def _ptr(t: torch.Tensor) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


@dataclass
class Scales:
    sq: np.ndarray       # (64,) mean |q_n|^2 per coefficient
    se: float            # mean column sum |k|^2 |psi_n|^2
    kmax: float          # largest in-band |k|
    out_scale: float     # s: typical rate
    target_norm: float   # mean column sum |t_n|^2
    ncoef: int


class TailClosure:
    """Parameters (FP32 master + BF16 copy), Adam state and feature scales on
    the device."""

    def __init__(self, scales: Scales, params: np.ndarray | None = None, seed: int = 0):
        self.lib = nat.load()
        if self.lib.nhqg_closure_param_count() != n_params():
            raise RuntimeError("closure parameter layout mismatch between Python and the library")
        flat = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        self.scales = scales
        dev = "cuda"
        self.w = torch.from_numpy(flat.copy()).to(dev)
        self.wb = self.w.to(torch.bfloat16)
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.grad = torch.zeros_like(self.w)
        self.loss_buf = torch.zeros(1, dtype=torch.float32, device=dev)
        sq = np.zeros(64, dtype=np.float32)
        sq[:] = 1.0
        sq[:scales.ncoef] = np.maximum(scales.sq[:scales.ncoef], 1e-300).astype(np.float32)
        self.sq = torch.from_numpy(sq).to(dev)
        self.step_count = 0

    # ------------------------------------------------------------ attach to a step
    def attach(self, engine: Engine) -> None:
        s = self.scales
        nat.check(self.lib.nhqg_closure_set(engine.handle, _ptr(self.wb), _ptr(self.sq), int(s.ncoef),
                                            float(s.se), float(s.kmax), float(s.out_scale)),
                  "nhqg_closure_set")

    @staticmethod
    def detach(engine: Engine) -> None:
        nat.check(engine.lib.nhqg_closure_set(engine.handle, None, None, 0, 1.0, 1.0, 0.0),
                  "nhqg_closure_set")

    def apply(self, engine: Engine, state) -> torch.Tensor:
        """C for ``state`` as (Nz+1, Nx, Nk) complex128 planes (the closure must
        be attached to ``engine``)."""
        s = to_device(state)
        g = engine.grid
        out = torch.empty((g.Nz + 1, g.Nx, g.Nk), dtype=torch.complex128, device="cuda")
        d = engine.state_desc(*s)
        nat.check(self.lib.nhqg_closure_apply(engine.handle, ctypes.byref(d), _ptr(out), _stream_handle()),
                  "nhqg_closure_apply")
        return out

    # ------------------------------------------------------------ training
    def train_step(self, x: torch.Tensor, q: torch.Tensor, t: torch.Tensor, lr: float) -> float:
        """One forward/backward pass (and Adam step if lr > 0); returns the loss
        (normalised so that the zero closure scores 1)."""
        if lr > 0:
            self.step_count += 1
        s = self.scales
        rc = self.lib.nhqg_closure_train_step(
            _ptr(self.wb), _ptr(self.w), _ptr(self.m), _ptr(self.v), _ptr(self.grad), _ptr(self.loss_buf),
            int(x.shape[0]), _ptr(x), _ptr(q), _ptr(t), float(s.out_scale), float(s.target_norm),
            float(lr), max(1, self.step_count), _stream_handle())
        nat.check(rc, "nhqg_closure_train_step")
        return float(self.loss_buf.item())

    def evaluate(self, x, q, t) -> float:
        return self.train_step(x, q, t, 0.0)

    def fit(self, data: dict, epochs: int = 50, batch: int = 2048, lr: float = 1e-3, seed: int = 0) -> list:
        """Mini-batch Adam over the columns of ``data`` (from training_columns)."""
        x, q, t = data["x"], data["q"], data["t"]
        n = x.shape[0]
        gen = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for _ in range(epochs):
            perm = torch.randperm(n, generator=gen).to(x.device)
            tot = 0.0
            for b0 in range(0, n, batch):
                idx = perm[b0:b0 + batch]
                tot += self.train_step(x[idx].contiguous(), q[idx].contiguous(), t[idx].contiguous(), lr) * len(idx)
            hist.append(tot / n)
        return hist

    def state_dict(self) -> dict:
        s = self.scales
        return {"params": self.w.cpu().numpy(), "sq": s.sq, "se": s.se, "kmax": s.kmax,
                "out_scale": s.out_scale, "target_norm": s.target_norm, "ncoef": s.ncoef}

    def save(self, path) -> None:
        np.savez(path, **self.state_dict())

    @classmethod
    def load(cls, path) -> "TailClosure":
        z = np.load(path)
        sc = Scales(np.array(z["sq"]), float(z["se"]), float(z["kmax"]), float(z["out_scale"]),
                    float(z["target_norm"]), int(z["ncoef"]))
        return cls(sc, params=np.array(z["params"]))


# ------------------------------------------------------------ data
def truncate(state, coarse: Grid) -> State:
    """Chebyshev / Galerkin truncation of a state to ``coarse``'s Nz (the
    Galerkin basis functions of the kept indices are the same functions)."""
    P, G = coarse.Nz + 1, coarse.Nz - 1
    s = to_device(state)
    # copies: a leading slice of a contiguous field is itself contiguous, and
    # a view would share memory with the fine state
    return State(s.q_hat[:P].clone(), s.w_hat[:G].clone(), s.th_hat[:G].clone(), s.th_bar[:P].clone())


def _base(g: Grid) -> Grid:
    if g.mean_exchange_discretization in ("balanced_sbp2", "balanced_sbp2_pc"):
        return g._replace(thermal_closure="fixed_conduction", mean_exchange_discretization="legacy")
    return g


def _compact(engine: Engine, q_planes: torch.Tensor) -> torch.Tensor:
    """(P, Nx, Nk) -> (M, P) complex128 in-band columns (engine's mode order)."""
    g = engine.grid
    P, G = g.Nz + 1, g.Nz - 1
    M = int(engine.lib.nhqg_mode_count(engine.handle))
    z = torch.zeros((G, g.Nx, g.Nk), dtype=torch.complex128, device="cuda")
    d = engine.state_desc(q_planes.contiguous(), z, z.clone(), torch.zeros(P, dtype=torch.float64, device="cuda"))
    out = torch.empty((P, M), dtype=torch.complex128, device="cuda")
    nat.check(engine.lib.nhqg_gather_q(engine.handle, ctypes.byref(d), _ptr(out), _stream_handle()),
              "nhqg_gather_q")
    return out.T.contiguous()


def mode_geometry(engine: Engine) -> tuple[np.ndarray, np.ndarray]:
    """|k|^2 and inv_denom of the in-band modes in the engine's compact order
    (r = kx row in fftfreq order of the band, c = ky column)."""
    g = engine.grid
    rows, ncol = compact_layout(g)
    kx = np.asarray(g.kx).reshape(g.Nx, -1)[:, 0][rows]
    ky = np.asarray(g.ky).reshape(-1)[:ncol]
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    inv = np.asarray(g.inv_denom)[np.ix_(rows, np.arange(ncol))]
    return (KX ** 2 + KY ** 2).ravel(), inv.ravel()


def training_columns(fine: Grid, coarse: Grid, states, ncoef: int | None = None,
                     scales: Scales | None = None) -> tuple[dict, Scales]:
    """Features, columns and targets of every in-band mode of every state.
    ``scales`` (from the training set) fixes the feature and loss scales;
    None derives them from these states."""
    if fine.Nx != coarse.Nx or fine.Nz <= coarse.Nz:
        raise ValueError("fine and coarse grids must share Nx with fine.Nz > coarse.Nz")
    ncoef = min(64, coarse.Nz + 1) if ncoef is None else int(ncoef)
    e_c = Engine(coarse)
    ksq, inv = mode_geometry(e_c)
    qs, ts = [], []
    for st in states:
        s = to_device(st)
        sc = truncate(s, coarse)
        t_planes = explicit_rhs(s, _base(fine)).q_hat[: coarse.Nz + 1] - explicit_rhs(sc, _base(coarse)).q_hat
        qs.append(_compact(e_c, sc.q_hat)[:, :ncoef])
        ts.append(_compact(e_c, t_planes)[:, :ncoef])
    q = torch.cat(qs)
    t = torch.cat(ts)
    if scales is None:
        a2 = (q.abs() ** 2).mean(0).cpu().numpy()
        sq = np.ones(64)
        sq[:ncoef] = np.maximum(a2, 1e-300)
        ksq_t = torch.from_numpy(np.tile(ksq, len(states))).to(q.device)
        inv_t = torch.from_numpy(np.tile(inv, len(states))).to(q.device)
        ke = (ksq_t[:, None] * inv_t[:, None] ** 2 * q.abs() ** 2).sum(1)
        se = float(max(ke.mean().item(), 1e-300))
        tn = float(max((t.abs() ** 2).sum(1).mean().item(), 1e-300))
        qn = float(max((q.abs() ** 2).sum(1).mean().item(), 1e-300))
        scales = Scales(sq, se, float(np.sqrt(ksq.max())), float(np.sqrt(tn / qn)), tn, ncoef)
    # features on the device from the same kernels the step uses
    xs = []
    sq32 = torch.from_numpy(scales.sq.astype(np.float32)).cuda()
    M = int(e_c.lib.nhqg_mode_count(e_c.handle))
    for st in states:
        sc = truncate(to_device(st), coarse)
        x = torch.empty((M, N_IN), dtype=torch.float32, device="cuda")
        qc = torch.empty((M, N_OUT, 2), dtype=torch.float32, device="cuda")
        d = e_c.state_desc(*sc)
        nat.check(e_c.lib.nhqg_closure_features(e_c.handle, ctypes.byref(d), _ptr(sq32), int(scales.ncoef),
                                                float(scales.se), float(scales.kmax), _ptr(x), _ptr(qc),
                                                _stream_handle()), "nhqg_closure_features")
        xs.append(x)
    x = torch.cat(xs)
    qpad = torch.zeros((q.shape[0], N_OUT), dtype=torch.complex64, device="cuda")
    tpad = torch.zeros_like(qpad)
    qpad[:, :ncoef] = q.to(torch.complex64)
    tpad[:, :ncoef] = t.to(torch.complex64)
    data = {"x": x, "q": torch.view_as_real(qpad).contiguous(), "t": torch.view_as_real(tpad).contiguous(),
            "q64": q, "t64": t, "ksq": ksq, "inv_denom": inv,
            "states": [truncate(to_device(st), coarse) for st in states]}
    return data, scales
