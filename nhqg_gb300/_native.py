"""Build and bind the C-ABI engine library ``libnhqg_gpu.so``.

The library is compiled in-tree with nvcc for sm_103a (``build()``) and bound
with ctypes; the C declarations live in ``include/nhqg_gpu.h``.  There is no
fallback: if the library is missing or fails to load, every GPU entry point
raises.
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libnhqg_gpu.so"
SOURCES = ("horizontal.cu", "horizontal_reg.cu", "vertical.cu", "corrector.cu", "capi.cu", "noalloc.cu", "tau_solve.cu",
           "diag.cu", "closure.cu", "tc_vertical.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"]

# status codes (include/nhqg_gpu.h)
NHQG_OK = 0
STATUS_NAMES = {0: "NHQG_OK", 1: "NHQG_ERR_BAD_ARG", 2: "NHQG_ERR_UNSUPPORTED", 3: "NHQG_ERR_CUDA",
                4: "NHQG_ERR_DEVICE_TIMEOUT", 5: "NHQG_ERR_NOT_BAND_LIMITED",
                6: "NHQG_ERR_SCRATCH_TOO_SMALL"}
DEVICE_STATUS_OOB = 1 << 0
DEVICE_STATUS_TIMEOUT = 1 << 1

ADV = {"flux": 0, "jacobian": 1}
CLOSURE = {"fixed_conduction": 0, "evolve_mean": 1}
EXCHANGE = {"legacy": 0, "balanced_sbp2": 1, "balanced_sbp2_pc": 2}
WBC = {"dirichlet": 0, "neumann": 1}
PRECISION = {"fp64": 0, "mixed": 1}
SCHEME = {"ars222": 0, "rk443": 1}
DEALIAS = {"23_rule": 0, "32_rule": 1}
DIAG_KEYS = ("KE_bt", "KE_bc", "KE_tot", "enstrophy", "Nusselt", "Nusselt_dealiased",
             "vol_avg_tw", "vol_avg_tw_dealiased", "q_rms", "w_rms", "th_rms", "th_bar_max",
             "max_speed", "max_w", "max_theta", "max_tw", "heat_flux_mismatch")


class NativeError(RuntimeError):
    pass


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise NativeError("nvcc not found: the NHQG GPU engine must be compiled for sm_103a")


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
    deps.append(INCLUDE / "nhqg_gpu.h")
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the engine (parallel per translation unit) into LIB."""
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise NativeError(f"nvcc failed on {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise NativeError(f"nvcc link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)


class GridDesc(ctypes.Structure):
    """Mirror of nhqg_grid_desc (include/nhqg_gpu.h)."""
    _fields_ = [
        ("Nx", ctypes.c_int), ("Nz", ctypes.c_int),
        ("advection", ctypes.c_int), ("thermal_closure", ctypes.c_int),
        ("exchange", ctypes.c_int), ("w_bc_top", ctypes.c_int),
        ("substeps", ctypes.c_int), ("n_shells", ctypes.c_int),
        ("dt", ctypes.c_double), ("gamma_imex", ctypes.c_double), ("Ra_sigma", ctypes.c_double),
        ("sigma", ctypes.c_double), ("beta", ctypes.c_double), ("eps_sq", ctypes.c_double),
        ("kx", c_double_p), ("ky", c_double_p), ("inv_denom", c_double_p),
        ("diss_rate_q", c_double_p), ("diss_rate_w", c_double_p), ("diss_rate_th", c_double_p),
        ("inv_alpha_q", c_double_p), ("inv_alpha_th", c_double_p),
        ("shell_of_mode", c_int_p), ("shell_inv", c_double_p),
        ("eta_hat", c_double_p), ("eta_phys", c_double_p), ("sponge_phys", c_double_p),
        ("V", c_double_p), ("V_inv", c_double_p), ("w_stencil", c_double_p), ("G_Z", c_double_p),
        ("proj_dirichlet", c_double_p), ("sbp_D1", c_double_p), ("sbp_L", c_double_p),
        ("cgl_to_sbp", c_double_p), ("sbp_to_cgl", c_double_p), ("mean_solve", c_double_p),
        ("shell_coef", c_double_p), ("cc_weights", c_double_p),
        ("imex_scheme", ctypes.c_int),
        ("horizontal_dealiasing", ctypes.c_int),
        ("eta_x_phys", c_double_p), ("eta_y_phys", c_double_p),
    ]


class StateDesc(ctypes.Structure):
    """Mirror of nhqg_state."""
    _fields_ = [("q_hat", ctypes.c_void_p), ("w_hat", ctypes.c_void_p),
                ("th_hat", ctypes.c_void_p), ("th_bar", ctypes.c_void_p)]


# exported symbols and their signatures (checked by the CPU test suite)
SIGNATURES = {
    "nhqg_ctx_create": (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "nhqg_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "nhqg_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.c_int, ctypes.c_void_p]),
    "nhqg_explicit_rhs": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.POINTER(StateDesc),
                                         ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "nhqg_implicit_tendency": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc),
                                              ctypes.POINTER(StateDesc), ctypes.c_int, ctypes.c_void_p]),
    "nhqg_implicit_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc),
                                           ctypes.POINTER(StateDesc), ctypes.c_int, ctypes.c_void_p]),
    "nhqg_sbp2_corrector": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc),
                                           ctypes.POINTER(StateDesc), ctypes.c_double, ctypes.c_void_p]),
    "nhqg_triple_advection_23": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] +
                                 [ctypes.c_void_p] * 7 + [ctypes.c_void_p]),
    "nhqg_triple_advection_23_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int] +
                                         [ctypes.c_void_p] * 9 + [ctypes.c_void_p]),
    "nhqg_sponge_product_23": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "nhqg_triple_advection_32": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] +
                                 [ctypes.c_void_p] * 7 + [ctypes.c_void_p]),
    "nhqg_sponge_product_32": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "nhqg_sanitize": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.c_void_p]),
    "nhqg_mean_temp_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p]),
    "nhqg_get_device_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nhqg_last_launch_count": (ctypes.c_int, [ctypes.c_void_p]),
    "nhqg_profile_enable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nhqg_set_precision": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nhqg_set_mixed_vertical": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "nhqg_spectra": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p]),
    "nhqg_get_mixed_vertical": (ctypes.c_int, [ctypes.c_void_p]),
    "nhqg_tc_to_nodal": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "nhqg_tc_to_coef": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "nhqg_diagnostics": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "nhqg_get_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "nhqg_set_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "nhqg_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "nhqg_batch_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "nhqg_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "nhqg_batch_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(StateDesc),
                                       ctypes.c_void_p]),
    "nhqg_batch_store": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(StateDesc),
                                        ctypes.c_void_p]),
    "nhqg_batch_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "nhqg_batch_size": (ctypes.c_int, [ctypes.c_void_p]),
    "nhqg_mode_count": (ctypes.c_int, [ctypes.c_void_p]),
    "nhqg_closure_param_count": (ctypes.c_int, []),
    "nhqg_closure_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "nhqg_closure_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "nhqg_closure_features": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.c_void_p,
                                             ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]),
    "nhqg_closure_train_step": (ctypes.c_int, [ctypes.c_void_p] * 6 + [ctypes.c_int] + [ctypes.c_void_p] * 3 +
                                [ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_void_p]),
    "nhqg_gather_q": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(StateDesc), ctypes.c_void_p,
                                     ctypes.c_void_p]),
    "nhqg_profile_report": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "nhqg_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path: Path | None = None) -> ctypes.CDLL:
    """Load (and bind) the engine library; raises NativeError if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB
    if not p.exists():
        raise NativeError(f"{p} is missing: run nhqg_gb300.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != NHQG_OK:
        raise NativeError(f"{what} failed: {STATUS_NAMES.get(rc, rc)}")
