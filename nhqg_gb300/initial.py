"""Seeded initial states (host NumPy; transferred with ``solver.to_device``).

``theta_perturbation_state`` is the start of the benchmark configurations:
theta' = amplitude * N(0,1) * sin(pi Z) at the CGL nodes, drawn from NumPy's
PCG64 ``default_rng(seed)`` with shape (Nz+1, Nx, Nx); rfft2 per level, then
V^-1 and the Dirichlet pinv to Galerkin coefficients; q' = w = 0 and
Theta_bar = 0; finally the Hermitian projection of the ky=0 column and the
2/3 band limit (``sanitize_state`` semantics, nhqg/solver.py:128-146).
"""

from __future__ import annotations

import numpy as np

from .grid import Grid


def _sanitize_host(f: np.ndarray, Nx: int, grid: Grid) -> np.ndarray:
    """sanitize_state on one field (nhqg/solver.py:107-146): Hermitian ky = 0
    and Nyquist columns, then the 2/3 band limit under the 2/3 rule only."""
    neg = (-np.arange(Nx)) % Nx
    f = f.copy()
    col = f[:, :, 0]
    f[:, :, 0] = 0.5 * (col + np.conj(col[:, neg]))
    col = f[:, :, -1]
    f[:, :, -1] = 0.5 * (col + np.conj(col[:, neg]))
    if grid.horizontal_dealiasing == "23_rule":
        f = f * grid.mask_23[None]
    return f


def theta_perturbation_state(grid: Grid, seed: int = 0, amplitude: float = 1e-3):
    P, Nx = grid.Nz + 1, grid.Nx
    rng = np.random.default_rng(seed)
    th = amplitude * rng.standard_normal((P, Nx, Nx)) * np.sin(np.pi * grid.Z)[:, None, None]
    th_nodal = np.fft.rfft2(th)
    cols = th_nodal.reshape(P, -1)
    th_cheb = (grid.V_inv @ cols.view(np.float64)).view(np.complex128)
    th_gal = (grid.dirichlet_pinv @ th_cheb.view(np.float64)).view(np.complex128)
    th_gal = th_gal.reshape(P - 2, Nx, Nx // 2 + 1)
    q = np.zeros((P, Nx, Nx // 2 + 1), dtype=np.complex128)
    w = np.zeros_like(th_gal)
    return (q, w, _sanitize_host(th_gal, Nx, grid), np.zeros(P))


# ---------------------------------------------------------------------------
# make_initial_state (nhqg/solver.py:1343-1376) with JAX's PRNG stream
# ---------------------------------------------------------------------------
#
# The reference draws its random q' start with jax.random (PRNGKey, split,
# normal) under the default threefry2x32 implementation with partitionable
# key derivation.  Restated here from the published algorithms:
# * Threefry-2x32 with 20 rounds (Salmon, Moraes, Dror, Shaw, "Parallel random
#   numbers: as easy as 1, 2, 3", SC'11): rotation constants
#   (13, 15, 26, 6) and (17, 29, 16, 24), key-schedule parity 0x1BD11BDA, a
#   key injection after every 4 rounds with the injection counter added to
#   the second word;
# * JAX's documented key handling: a 64-bit seed becomes the key (hi, lo);
#   split(key, n) and the random bits of an array both hash the (hi, lo)
#   words of the flat element index with the key; 64-bit bits are
#   (word0 << 32) | word1;
# * normal(key, shape, float64) = sqrt(2) erfinv(u), u uniform on
#   [nextafter(-1, 0), 1) from the top 52 bits of the 64-bit random bits.
# XLA's erfinv and SciPy's agree to a few ulp, so the state matches the
# reference's to round-off rather than bitwise.

_ROT = ((13, 15, 26, 6), (17, 29, 16, 24))
_PARITY = np.uint32(0x1BD11BDA)


def _rotl(x: np.ndarray, r: int) -> np.ndarray:
    return ((x << np.uint32(r)) | (x >> np.uint32(32 - r))).astype(np.uint32)


def threefry2x32(key: tuple[int, int], x0: np.ndarray, x1: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Threefry-2x32-20 of the counter pairs (x0, x1) under ``key``."""
    k0, k1 = np.uint32(key[0]), np.uint32(key[1])
    ks = (k0, k1, np.uint32(k0 ^ k1 ^ _PARITY))
    with np.errstate(over="ignore"):
        a = (np.asarray(x0, dtype=np.uint32) + ks[0]).astype(np.uint32)
        b = (np.asarray(x1, dtype=np.uint32) + ks[1]).astype(np.uint32)
        for inj in range(5):
            for r in _ROT[inj % 2]:
                a = (a + b).astype(np.uint32)
                b = _rotl(b, r) ^ a
            a = (a + ks[(inj + 1) % 3]).astype(np.uint32)
            b = (b + ks[(inj + 2) % 3] + np.uint32(inj + 1)).astype(np.uint32)
    return a, b


def jax_prng_key(seed: int) -> tuple[int, int]:
    s = int(seed) & 0xFFFFFFFFFFFFFFFF
    return (s >> 32) & 0xFFFFFFFF, s & 0xFFFFFFFF


def jax_split(key: tuple[int, int], n: int = 2) -> list[tuple[int, int]]:
    idx = np.arange(n, dtype=np.uint64)
    a, b = threefry2x32(key, (idx >> np.uint64(32)).astype(np.uint32), (idx & np.uint64(0xFFFFFFFF)).astype(np.uint32))
    return [(int(a[i]), int(b[i])) for i in range(n)]


def jax_normal(key: tuple[int, int], shape: tuple[int, ...]) -> np.ndarray:
    from scipy.special import erfinv

    n = int(np.prod(shape))
    idx = np.arange(n, dtype=np.uint64)
    a, b = threefry2x32(key, (idx >> np.uint64(32)).astype(np.uint32), (idx & np.uint64(0xFFFFFFFF)).astype(np.uint32))
    bits = (a.astype(np.uint64) << np.uint64(32)) | b.astype(np.uint64)
    one = np.array(1.0, dtype=np.float64).view(np.uint64)
    floats = ((bits >> np.uint64(12)) | one).view(np.float64) - 1.0
    lo = np.nextafter(np.float64(-1.0), np.float64(0.0))
    u = np.maximum(lo, floats * (np.float64(1.0) - lo) + lo)
    return (np.sqrt(np.float64(2.0)) * erfinv(u)).reshape(shape)


def make_initial_state(grid: Grid, seed: int = 0, amplitude: float = 1e-3):
    """The reference's random q' start (nhqg/solver.py:1343-1376): amplitude x
    complex N(0,1) at every CGL node and (kx, ky) from jax.random with
    PRNGKey(seed) split in two (real, imaginary parts), times sin(pi Z); V^-1
    to Chebyshev coefficients; the (0,0) mode zeroed; w = theta = 0,
    Theta_bar = 0; then ``sanitize_state``.  Host NumPy arrays."""
    P, Nx, Nk = grid.Nz + 1, grid.Nx, grid.Nx // 2 + 1
    k1, k2 = jax_split(jax_prng_key(seed), 2)
    q_nodal = amplitude * (jax_normal(k1, (P, Nx, Nk)) + 1j * jax_normal(k2, (P, Nx, Nk)))
    q_nodal = q_nodal * np.sin(np.pi * np.asarray(grid.Z))[:, None, None]
    q_hat = np.einsum("ij,j...->i...", np.asarray(grid.V_inv), q_nodal)
    q_hat[:, 0, 0] = 0.0
    if grid.q_boundary != "none":
        raise ValueError(f"q_boundary={grid.q_boundary!r} is not supported")
    G = grid.Nz - 1
    z = np.zeros((G, Nx, Nk), dtype=np.complex128)
    return (_sanitize_host(q_hat, Nx, grid), z, z.copy(), np.zeros(P))
