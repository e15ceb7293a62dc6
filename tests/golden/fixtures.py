"""Packing helpers for the golden fixtures.

Spectral fields in NHQG's rfft2 layout ``(levels, Nx, Nx//2+1)`` are stored
packed to the 2/3-rule band: rows ``kx in [0..K] + [Nx-K..Nx-1]`` (fftfreq
order) and columns ``ky in [0..K]`` with ``K = Nx//3``.  Every state the
reference produces from a band-limited input is exactly zero outside that
rectangle, and ``make_golden.py`` asserts it before packing.  The 3/2-rule
cases (``PAD_CASES``) are full band and stored unpacked.
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN_DIR = Path(__file__).parent


def band_rows(Nx: int) -> np.ndarray:
    K = Nx // 3
    return np.concatenate([np.arange(K + 1), np.arange(Nx - K, Nx)])


def pack(field: np.ndarray, Nx: int) -> np.ndarray:
    K = Nx // 3
    rows = band_rows(Nx)
    return np.ascontiguousarray(field[:, rows, : K + 1])


def out_of_band_max(field: np.ndarray, Nx: int) -> float:
    K = Nx // 3
    rows = band_rows(Nx)
    keep = np.zeros(field.shape[1:], dtype=bool)
    keep[np.ix_(rows, np.arange(K + 1))] = True
    rest = field[:, ~keep]
    return float(np.max(np.abs(rest))) if rest.size else 0.0


def unpack(packed: np.ndarray, Nx: int) -> np.ndarray:
    K = Nx // 3
    Nk = Nx // 2 + 1
    out = np.zeros((packed.shape[0], Nx, Nk), dtype=packed.dtype)
    out[:, band_rows(Nx), : K + 1] = packed
    return out


def load_case(name: str) -> tuple[dict, dict]:
    """Return (config dict, arrays dict with spectral fields unpacked)."""
    with np.load(GOLDEN_DIR / f"{name}.npz") as z:
        meta = json.loads(str(z["meta"]))
        Nx = meta["cfg"]["Nx"]
        arrays = {}
        for key in z.files:
            if key == "meta":
                continue
            a = z[key]
            if key.endswith("__packed"):
                arrays[key[: -len("__packed")]] = unpack(a, Nx)
            else:
                arrays[key] = a
    return meta, arrays


def state_from(arrays: dict, prefix: str):
    return tuple(arrays[f"{prefix}.{f}"] for f in ("q_hat", "w_hat", "th_hat", "th_bar"))


CASES = ("prod16", "fixed16", "jac16", "polar16", "radix24", "legacy16")
# ARS(4,4,3) with the legacy exchange (fixed conduction; legacy evolve_mean)
RK_CASES = ("rk443f16", "rk443l16")
# 3/2-rule padded products: full-band states, stored unpacked
PAD_CASES = ("pad32p16", "pad32j16", "pad32o16", "pad32s16", "pad32l24")


def load_diagnostics() -> dict:
    """Reference compute_diagnostics scalars: ``<case>.<state>`` -> values in
    the order of ``keys`` (tests/golden/diagnostics.npz)."""
    with np.load(GOLDEN_DIR / "diagnostics.npz") as z:
        return {k: np.array(z[k]) for k in z.files}


def load_diagnostics_extra() -> dict:
    """Reference compute_diagnostics physical-space maxima and heat-flux
    mismatch: ``<case>.<state>`` -> values in the order of ``keys``
    (tests/golden/diagnostics_extra.npz; 2/3- and 3/2-rule cases)."""
    with np.load(GOLDEN_DIR / "diagnostics_extra.npz") as z:
        return {k: np.array(z[k]) for k in z.files}


def load_field_spectra() -> dict:
    """Reference horizontal shell spectra of q, w, theta at the CGL nodes:
    ``<case>.<state>.<k_bins|q|w|th>`` (tests/golden/field_spectra.npz)."""
    with np.load(GOLDEN_DIR / "field_spectra.npz") as z:
        return {k: np.array(z[k]) for k in z.files}


SPEC_KEYS = ("k_bins", "E_bt", "E_bc", "E_tot", "q", "w", "th")


def load_spectra() -> dict:
    """Reference energy_spectrum and vertical_mode_energy outputs:
    ``<case>.<state>.<key>`` (tests/golden/spectra.npz)."""
    with np.load(GOLDEN_DIR / "spectra.npz") as z:
        return {k: np.array(z[k]) for k in z.files}
