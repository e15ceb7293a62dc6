"""Allocation-free triple advection against the context-based entry point.

Callers that must not allocate device memory themselves -- XLA FFI handlers
(every buffer comes from XLA's allocator), hosts with a fixed device-memory
pool -- use
``nhqg_triple_advection_23_noalloc``, which keeps its working storage in one
static device array instead of a context.  The test calls it through the C ABI
twice in a row (the second call starts from the first call's leftover scratch)
and compares each result with ``nhqg_triple_advection_23`` on the same inputs,
at the tolerance of the other product parity tests (1e-13 relative L2).
"""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():  # pragma: no cover - CPU container
    pytest.skip("needs a CUDA device", allow_module_level=True)

from nhqg_gb300 import _native as nat  # noqa: E402
from nhqg_gb300.spectral import _engine  # noqa: E402


def _rel(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _wavenumbers(Nx, L=31.0):
    kx = 2 * np.pi * np.fft.fftfreq(Nx, d=L / Nx)
    ky = 2 * np.pi * np.arange(Nx // 2 + 1) / L
    return kx, ky


# Nx=256 with 9 levels runs in two chunks in both forms (6 + 3 levels)
@pytest.mark.parametrize("form,Nx,levels", [("flux", 64, 5), ("jacobian", 48, 3), ("flux", 256, 9),
                                            ("jacobian", 256, 9)])
def test_noalloc_matches_context_entry_point(form, Nx, levels):
    lib = nat.load()
    rng = np.random.default_rng(Nx + levels)
    kx, ky = _wavenumbers(Nx)
    shp = (levels, Nx, Nx // 2 + 1)
    planes = [torch.from_numpy(rng.standard_normal(shp) + 1j * rng.standard_normal(shp)).cuda()
              for _ in range(4)]
    ref = [torch.empty_like(planes[0]) for _ in range(3)]
    _engine(Nx, kx[:, None], ky[None, :]).triple_advection(form, *planes, *ref)
    kx_d = torch.tensor(kx, dtype=torch.float64, device="cuda")
    ky_d = torch.tensor(ky, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        out = [torch.full_like(planes[0], complex(1e300, -1e300)) for _ in range(3)]
        rc = lib.nhqg_triple_advection_23_noalloc(
            nat.ADV[form], Nx, levels, kx_d.data_ptr(), ky_d.data_ptr(),
            *(p.data_ptr() for p in planes), *(o.data_ptr() for o in out), stream)
        assert rc == nat.NHQG_OK, nat.STATUS_NAMES.get(rc, rc)
        torch.cuda.synchronize()
        for o, r in zip(out, ref):
            assert _rel(o, r) <= 1e-13


def test_noalloc_rejects_sizes_beyond_scratch():
    lib = nat.load()
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = dummy.data_ptr()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # one Jacobian level at Nx=2048 needs ~336 MB of intermediates
    rc = lib.nhqg_triple_advection_23_noalloc(nat.ADV["jacobian"], 2048, 1, p, p, p, p, p, p, p, p, p,
                                              stream)
    assert rc == 6  # NHQG_ERR_SCRATCH_TOO_SMALL
    rc = lib.nhqg_triple_advection_23_noalloc(nat.ADV["flux"], 4096, 1, p, p, p, p, p, p, p, p, p,
                                              stream)
    assert rc == 2  # NHQG_ERR_UNSUPPORTED
    # one flux level at Nx=768 needs ~43 MB (the largest flux size that fits is 648)
    rc = lib.nhqg_triple_advection_23_noalloc(nat.ADV["flux"], 768, 1, p, p, p, p, p, p, p, p, p,
                                              stream)
    assert rc == 6


def test_noalloc_rejects_outputs_overlapping_inputs():
    lib = nat.load()
    Nx, levels = 16, 2
    shp = (levels, Nx, Nx // 2 + 1)
    buf = [torch.zeros(shp, dtype=torch.complex128, device="cuda") for _ in range(4)]
    kx, ky = _wavenumbers(Nx)
    kx_d = torch.tensor(kx, dtype=torch.float64, device="cuda")
    ky_d = torch.tensor(ky, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = [torch.zeros_like(buf[0]) for _ in range(2)]
    # Aq == q (in-place use) is rejected before anything runs
    rc = lib.nhqg_triple_advection_23_noalloc(
        nat.ADV["flux"], Nx, levels, kx_d.data_ptr(), ky_d.data_ptr(),
        *(b.data_ptr() for b in buf), buf[1].data_ptr(), out[0].data_ptr(), out[1].data_ptr(), stream)
    assert rc == 1  # NHQG_ERR_BAD_ARG
