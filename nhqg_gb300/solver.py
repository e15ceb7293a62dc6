"""Drop-in time-step API on the GB300 engine.

Same names, argument meaning and return structure as the reference's
``nhqg.solver`` (nhqg/solver.py): ``State`` (q_hat, w_hat, th_hat, th_bar),
``imex_step(state, grid) -> State``, ``make_initial_state``, ``explicit_rhs``,
``explicit_rhs_dispatch``, ``implicit_tendency``, ``imex_implicit_solve``,
``imex_mean_temp_solve``, ``sanitize_state`` and ``run``.  Fields are CUDA
torch tensors (complex128 / float64) in the reference layout; NumPy arrays
are accepted and copied to the device.  Functions return new tensors, like
the reference's functional JAX API; ``step_inplace`` advances a state in
place for drivers that own their buffers (the analogue of donation).

``precision`` (an addition without a reference counterpart) selects the
plain FP64 path ('fp64', the default) or the mixed-precision path ('mixed':
FP32 horizontal products and the Chebyshev <-> nodal transforms around them,
double-float Galerkin stencils, stage combinations and SBP2 corrector
transforms, FP64 implicit and 1-D mean-temperature solves).

Every computation runs in the CUDA engine; there is no CPU path.
"""

from __future__ import annotations

from typing import NamedTuple

import numpy as np
import torch

from . import _native as nat
from .engine import engine_for, require_cuda
from .grid import Grid


class State(NamedTuple):
    """q' Chebyshev (Nz+1, Nx, Nk); w, theta Galerkin (Nz-1, Nx, Nk);
    th_bar Chebyshev (Nz+1,)  (nhqg/solver.py:33-38)."""
    q_hat: torch.Tensor
    w_hat: torch.Tensor
    th_hat: torch.Tensor
    th_bar: torch.Tensor


def _dev(x, dtype) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x))).to(device="cuda", dtype=dtype)


def to_device(state) -> State:
    """State of CUDA tensors (copies NumPy / host inputs)."""
    require_cuda()
    return State(_dev(state[0], torch.complex128), _dev(state[1], torch.complex128),
                 _dev(state[2], torch.complex128), _dev(state[3], torch.float64))


def to_host(state) -> tuple:
    return tuple(t.detach().cpu().numpy() for t in state)


def _fresh(state: State) -> State:
    return State(*(torch.empty_like(t) for t in state))


def _copy(state) -> State:
    s = to_device(state)
    return State(*(t.clone() for t in s))


def _check_band(eng, what: str) -> None:
    st = eng.device_status(reset=True)
    if st & nat.DEVICE_STATUS_OOB:
        raise ValueError(
            f"{what}: the state has content outside the 2/3 band; the GPU step "
            "assumes band-limited input (apply sanitize_state first)")


def sanitize_state(state, grid: Grid) -> State:
    """Hermitian projection of the ky=0 column + 2/3 band limit
    (nhqg/solver.py:128-146)."""
    eng = engine_for(grid)
    s = _copy(state)
    eng.sanitize(*s)
    eng.device_status(reset=True)
    return s


def step_inplace(state: State, grid: Grid, n_steps: int = 1, check: bool = False,
                 precision: str = "fp64") -> State:
    """Advance ``state`` (CUDA tensors, reference layout) by ``n_steps``
    imex_step applications in place; stream-ordered, no host sync unless
    ``check`` (then the band-limit status is verified)."""
    eng = engine_for(grid)
    eng.step(*state, n_steps=n_steps, precision=precision)
    if check:
        _check_band(eng, "imex_step")
    return state


def imex_step(state, grid: Grid, precision: str = "fp64") -> State:
    """One IMEX step incl. ``sanitize_state`` (nhqg/solver.py:1228-1242)."""
    s = _copy(state)
    return step_inplace(s, grid, 1, check=True, precision=precision)


def imex_step_many(states, grid: Grid, precision: str = "fp64", out=None) -> list:
    """``imex_step`` of each of a sequence of independent states held in host
    memory, with the host<->device copies overlapped with the steps: step k
    computes on the current stream while the input of step k+1 is uploaded
    and the result of step k-1 downloaded on two copy streams (three device
    states in rotation, ordered by CUDA events: the upload into a state waits
    only for the download of the result it held three steps earlier, so the
    two directions of the host link run at the same time).  Inputs in pinned
    memory let the copies run asynchronously.  Results go to ``out`` (a list
    of host State tuples of pinned tensors, reused cyclically if shorter than
    ``states``) or to new pinned tensors; returns the list of results,
    complete on return.  The band-limit status is checked once, after the
    last step."""
    states = list(states)
    if not states:
        return []
    eng = engine_for(grid)
    eng.set_precision(precision)
    compute = torch.cuda.current_stream()
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    dtypes = (torch.complex128, torch.complex128, torch.complex128, torch.float64)
    first = [torch.as_tensor(np.asarray(x)) if not isinstance(x, torch.Tensor) else x for x in states[0]]
    nbuf = 3
    bufs = [State(*(torch.empty(t.shape, dtype=d, device="cuda") for t, d in zip(first, dtypes)))
            for _ in range(nbuf)]
    if out is None:
        out = [tuple(torch.empty(t.shape, dtype=d, pin_memory=True) for t, d in zip(first, dtypes))
               for _ in range(len(states))]
    ev_in = [torch.cuda.Event() for _ in range(nbuf)]
    ev_done = [torch.cuda.Event() for _ in range(nbuf)]
    ev_out = [torch.cuda.Event() for _ in range(nbuf)]
    results = []
    for k, st in enumerate(states):
        b = k % nbuf
        if k >= nbuf:
            up.wait_event(ev_out[b])  # buffer b's previous result has left the device
        with torch.cuda.stream(up):
            for dst, src, d in zip(bufs[b], st, dtypes):
                src = src if isinstance(src, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(src))
                dst.copy_(src.to(dtype=d), non_blocking=True)
            ev_in[b].record(up)
        compute.wait_event(ev_in[b])
        eng.step(*bufs[b], n_steps=1, precision=precision)
        ev_done[b].record(compute)
        res = out[k % len(out)]
        down.wait_event(ev_done[b])
        with torch.cuda.stream(down):
            for dst, src in zip(res, bufs[b]):
                dst.copy_(src, non_blocking=True)
            ev_out[b].record(down)
        results.append(res)
    compute.wait_stream(down)
    compute.wait_stream(up)
    torch.cuda.synchronize()
    _check_band(eng, "imex_step_many")
    return results


def _split(grid: Grid) -> bool:
    return grid.mean_exchange_discretization in ("balanced_sbp2", "balanced_sbp2_pc")


def explicit_rhs(state, grid: Grid, precision: str = "fp64") -> State:
    """Explicit tendency E (nhqg/solver.py:510-599) for ``grid``'s closure."""
    eng = engine_for(grid)
    src = to_device(state)
    out = _fresh(src)
    eng.explicit_rhs(src, out, grid.thermal_closure, grid.mean_exchange_discretization,
                     precision=precision)
    _check_band(eng, "explicit_rhs")
    return out


def explicit_rhs_dispatch(state, grid: Grid, precision: str = "fp64") -> State:
    """nhqg/solver.py:602-608 (vertical_dealiasing='none')."""
    return explicit_rhs(state, grid, precision=precision)


def implicit_tendency(state, grid: Grid) -> State:
    """Implicit tendency I (nhqg/solver.py:615-641)."""
    eng = engine_for(grid)
    src = to_device(state)
    out = _fresh(src)
    eng.implicit_tendency(src, out, grid.thermal_closure)
    _check_band(eng, "implicit_tendency")
    return out


def imex_implicit_solve(R_q, R_w, R_th, grid: Grid, precision: str = "fp64"):
    """Block-eliminated implicit stage solve (nhqg/solver.py:691-738); with
    precision='mixed' the w system is solved by the O(Nz) Chebyshev-tau
    recurrence instead of the dense shell inverse (both FP64)."""
    eng = engine_for(grid)
    zero = torch.zeros(grid.Nz + 1, dtype=torch.float64, device="cuda")
    src = to_device((R_q, R_w, R_th, zero))
    out = _fresh(src)
    eng.implicit_solve(src, out, grid.thermal_closure, precision=precision)
    _check_band(eng, "imex_implicit_solve")
    return out.q_hat, out.w_hat, out.th_hat


def imex_mean_temp_solve(R_th_bar, grid: Grid) -> torch.Tensor:
    """1-D mean-temperature implicit solve (nhqg/solver.py:741-758)."""
    eng = engine_for(grid)
    R = _dev(R_th_bar, torch.float64)
    out = torch.empty_like(R)
    eng.mean_temp_solve(R, out, grid.thermal_closure)
    return out


def apply_balanced_sbp2_corrector(state, grid: Grid, total_dt) -> State:
    """SBP2 thermal corrector (nhqg/solver.py:909-950)."""
    eng = engine_for(grid)
    src = to_device(state)
    out = _fresh(src)
    eng.corrector(src, out, float(total_dt))
    _check_band(eng, "apply_balanced_sbp2_corrector")
    return out


def make_initial_state(grid: Grid, seed: int = 0, amplitude: float = 1e-3) -> State:
    """The reference's random q' start with JAX's PRNG stream
    (nhqg/solver.py:1343-1376; see ``initial.make_initial_state``), on the
    device."""
    from .initial import make_initial_state as _mis
    return to_device(_mis(grid, seed=seed, amplitude=amplitude))


def run(grid: Grid, state, n_steps: int, save_interval: int, use_imex: bool = True,
        callback=None, precision: str = "fp64"):
    """Time loop (nhqg/solver.py:1385-1416): sanitize the incoming state, then
    advance in chunks of ``save_interval`` steps; returns (state, snapshots)
    with snapshots = [(t, State copy), ...]."""
    if not use_imex:
        raise NotImplementedError("the GPU engine implements the IMEX stepper (use_imex=True)")
    s = sanitize_state(state, grid)
    snaps = []
    n_outer = n_steps // save_interval
    for i in range(n_outer):
        step_inplace(s, grid, save_interval, check=(i == 0), precision=precision)
        step = (i + 1) * save_interval
        t = step * float(grid.dt)
        if callback is not None:
            callback(s, step, t)
        snaps.append((t, State(*(x.clone() for x in s))))
    rem = n_steps % save_interval
    if rem:
        step_inplace(s, grid, rem, check=(n_outer == 0), precision=precision)
    return s, snaps


def prolong_state(state, grid_from: Grid, grid_to: Grid) -> State:
    """Spectral prolongation of a state onto a finer grid of the same box
    (no reference counterpart; used to start a fine run from a state spun up
    on a coarse grid).  Horizontal modes keep their wavenumbers (fftfreq rows,
    rfft columns) and are scaled by (Nx_to/Nx_from)^2, the ratio of the
    unnormalised rfft2 sums; Chebyshev (q', Theta_bar) and Dirichlet-Galerkin
    (w, theta) coefficients are zero-padded, an exact embedding of the
    coarse polynomials.  Both grids must have the Dirichlet w basis, the same
    L, Nx_to >= Nx_from and Nz_to >= Nz_from; the result is sanitized on
    ``grid_to``."""
    if grid_to.Nx < grid_from.Nx or grid_to.Nz < grid_from.Nz:
        raise ValueError("prolong_state: the target grid must be at least as fine")
    if abs(float(grid_to.L) - float(grid_from.L)) > 1e-12 * float(grid_from.L):
        raise ValueError("prolong_state: both grids must have the same box size L")
    if grid_from.w_bc_top != "dirichlet" or grid_to.w_bc_top != "dirichlet":
        raise ValueError("prolong_state: needs the Dirichlet w basis on both grids")
    s = to_device(state)
    n0, n1 = grid_from.Nx, grid_to.Nx
    h0 = n0 // 2  # coarse rows 0..h0-1 are kx >= 0, rows h0.. negative (Nyquist row kept in place)
    scale = (n1 / n0) ** 2

    def horiz(f: torch.Tensor, levels: int) -> torch.Tensor:
        out = torch.zeros((levels, n1, n1 // 2 + 1), dtype=torch.complex128, device="cuda")
        lv, nk0 = f.shape[0], f.shape[2]
        out[:lv, :h0, :nk0] = f[:, :h0] * scale
        out[:lv, n1 - (n0 - h0):, :nk0] = f[:, h0:] * scale
        return out

    P1, G1 = grid_to.Nz + 1, grid_to.Nz - 1
    tb = torch.zeros(P1, dtype=torch.float64, device="cuda")
    tb[:s.th_bar.shape[0]] = s.th_bar
    fine = State(horiz(s.q_hat, P1), horiz(s.w_hat, G1), horiz(s.th_hat, G1), tb)
    return sanitize_state(fine, grid_to)
