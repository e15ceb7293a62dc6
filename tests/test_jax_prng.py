"""JAX-PRNG restatement (nhqg_gb300.initial): Threefry-2x32 known answers
(Salmon et al. 2011), and the reference's bitwise regression
(tests/test_mixed_bc_plumbing.py:99-117: make_initial_state(seed=0) then 20
steps, packed in tests/golden/jaxprng_m2b.npz) reproduced through the oracle
to round-off (XLA's and SciPy's erfinv differ in the last bits)."""

import numpy as np

import fixtures
import oracle
from oracle.nhqg_oracle import OracleConfig, OracleState
from _util import assert_state_close

from nhqg_gb300 import NHQGConfig, make_grid
from nhqg_gb300.initial import jax_prng_key, jax_split, make_initial_state, threefry2x32


def test_threefry2x32_known_answers():
    cases = [((0x00000000, 0x00000000), (0x00000000, 0x00000000), (0x6B200159, 0x99BA4EFE)),
             ((0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF), (0x1CB996FC, 0xBB002BE7)),
             ((0x13198A2E, 0x03707344), (0x243F6A88, 0x85A308D3), (0xC4923A9C, 0x483DF7A0))]
    for key, ctr, want in cases:
        a, b = threefry2x32(key, np.array([ctr[0]], np.uint32), np.array([ctr[1]], np.uint32))
        assert (int(a[0]), int(b[0])) == want


def test_key_handling():
    assert jax_prng_key(0) == (0, 0)
    assert jax_prng_key(2**32 + 5) == (1, 5)
    k1, k2 = jax_split((0, 0), 2)
    a, b = threefry2x32((0, 0), np.array([0, 0], np.uint32), np.array([0, 1], np.uint32))
    assert (k1, k2) == ((int(a[0]), int(b[0])), (int(a[1]), int(b[1])))


def test_make_initial_state_reference_regression():
    meta, arrays = fixtures.load_case("jaxprng_m2b")
    cfg = dict(meta["cfg"])
    g = make_grid(NHQGConfig(**cfg))
    s = OracleState(*make_initial_state(g, seed=meta["seed"], amplitude=meta["amplitude"]))
    o = oracle.make_grid(OracleConfig(**cfg))
    for _ in range(meta["n_steps"]):
        s = oracle.imex_step(s, o)
    assert_state_close(s, fixtures.state_from(arrays, "sN"), 1e-12)
