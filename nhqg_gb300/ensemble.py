"""Batched ensemble: many independent NHQG instances advanced together.

An addition without a reference counterpart (the reference runs sweeps one
instance at a time, ``tests/test_vmap.py:205-208``, ``scripts/run_sweep.py``).
Each member is its own Grid (size, Ra, closure ...) with its own engine
context; ``Ensemble.step(n)`` advances all members through one CUDA graph
launch per ``steps_per_launch`` steps (``nhqg_batch_*`` in the C ABI).  Tiles
of the horizontal products are autotuned once per (Nx, Nz, precision) class
and shared by the members of the class.
"""

from __future__ import annotations

import ctypes
from typing import Sequence

import torch

from . import _native as nat
from .engine import Engine, _stream_handle, require_cuda
from .grid import Grid
from .solver import State, to_device


class Ensemble:
    def __init__(self, grids: Sequence[Grid], precision: str | Sequence[str] = "fp64",
                 steps_per_launch: int = 10, autotune: bool = True):
        require_cuda()
        n = len(grids)
        if n == 0:
            raise ValueError("an ensemble needs at least one member")
        precs = [precision] * n if isinstance(precision, str) else list(precision)
        if len(precs) != n:
            raise ValueError("one precision per member")
        # one engine per member (not the per-Grid cache: members own their state)
        self.engines = [Engine(g) for g in grids]
        self.grids = list(grids)
        for e, p in zip(self.engines, precs):
            e.set_precision(p)
        self.precisions = precs
        self.tiles: dict[tuple, tuple] = {}
        if autotune:
            for e, g, p in zip(self.engines, self.grids, precs):
                key = (g.Nx, g.Nz, p)
                if key not in self.tiles:
                    self.tiles[key] = e.autotune()
                else:
                    e.set_tiles(self.tiles[key])
        lib = self.engines[0].lib
        self.lib = lib
        handles = (ctypes.c_void_p * n)(*[e.handle.value for e in self.engines])
        h = ctypes.c_void_p()
        nat.check(lib.nhqg_batch_create(handles, n, int(steps_per_launch), ctypes.byref(h)),
                  "nhqg_batch_create")
        self.handle = h
        self.steps_per_launch = int(steps_per_launch)

    def __len__(self) -> int:
        return len(self.engines)

    def close(self) -> None:
        if self.handle:
            torch.cuda.synchronize()
            self.lib.nhqg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, i: int, state) -> None:
        s = to_device(state)
        d = self.engines[i].state_desc(*s)
        nat.check(self.lib.nhqg_batch_load(self.handle, int(i), ctypes.byref(d), _stream_handle()),
                  "nhqg_batch_load")
        st = self.engines[i].device_status(reset=True)
        if st & nat.DEVICE_STATUS_OOB:
            raise ValueError("Ensemble.load: the state has content outside the 2/3 band")

    def step(self, n_steps: int = 1) -> None:
        """Advance every member by n_steps (stream-ordered, no host sync)."""
        nat.check(self.lib.nhqg_batch_step(self.handle, int(n_steps), _stream_handle()),
                  "nhqg_batch_step")

    def store(self, i: int) -> State:
        g = self.grids[i]
        P, G, Nx, Nk = g.Nz + 1, g.Nz - 1, g.Nx, g.Nx // 2 + 1
        out = State(torch.empty((P, Nx, Nk), dtype=torch.complex128, device="cuda"),
                    torch.empty((G, Nx, Nk), dtype=torch.complex128, device="cuda"),
                    torch.empty((G, Nx, Nk), dtype=torch.complex128, device="cuda"),
                    torch.empty((P,), dtype=torch.float64, device="cuda"))
        d = self.engines[i].state_desc(*out)
        nat.check(self.lib.nhqg_batch_store(self.handle, int(i), ctypes.byref(d), _stream_handle()),
                  "nhqg_batch_store")
        return out
