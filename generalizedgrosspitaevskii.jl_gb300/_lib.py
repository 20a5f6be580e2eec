"""ctypes binding of libgpe.so (include/gpe.h).

This is the Python stand-in for the ``ccall`` layer a Julia shim would use.  Loading
fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_uint64, c_void_p
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libgpe.so"

GPE_ABI_VERSION = 1
GPE_OK = 0
GPE_ERR_INVALID = -1
GPE_ERR_UNSUPPORTED = -2
GPE_ERR_CUDA = -3
GPE_ERR_NONFINITE = -4
GPE_ERR_TIMEOUT = -5
GPE_ERR_NOMEM = -6
GPE_C128 = 0
GPE_C64 = 1
GPE_FLAG_FP64_NATIVE = 1
GPE_FLAG_FP64_DW = 16
GPE_FLAG_FFT_BFP = 32
GPE_FLAG_NO_RESIDENT = 2
GPE_FLAG_NO_TMA = 4
GPE_FLAG_TMA = 8
GPE_TABLE_NONE, GPE_TABLE_SCALAR, GPE_TABLE_DIAG, GPE_TABLE_MATRIX = 0, 1, 2, 3
GPE_NOISE_OFF, GPE_NOISE_PHILOX, GPE_NOISE_REPLAY = 0, 1, 2

ERR_NAMES = {
    GPE_ERR_INVALID: "invalid argument",
    GPE_ERR_UNSUPPORTED: "unsupported",
    GPE_ERR_CUDA: "CUDA error",
    GPE_ERR_NONFINITE: "non-finite value",
    GPE_ERR_TIMEOUT: "device wait timed out",
    GPE_ERR_NOMEM: "out of device memory",
}


class GpeDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", c_int32),
        ("ndim", c_int32),
        ("n", c_int64 * 3),
        ("lengths", c_double * 3),
        ("batch", c_int64),
        ("ncomp", c_int32),
        ("dtype", c_int32),
        ("dt", c_double),
        ("t0", c_double),
        ("device", c_int32),
        ("flags", c_int32),
    ]


class GpeState(ctypes.Structure):
    _fields_ = [
        ("t", c_double),
        ("steps", c_int64),
        ("seed", c_uint64),
        ("noise_mode", c_int32),
        ("reserved", c_int32),
    ]


class GPEError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, 'error')} ({code}): {msg}")
        self.code = code


H = c_void_p
DP = POINTER(c_double)

# name -> (restype, argtypes); the full list of exported entry points
SIGNATURES = {
    "gpe_create": (c_int, [POINTER(GpeDesc), POINTER(c_void_p)]),
    "gpe_destroy": (c_int, [H]),
    "gpe_last_error": (c_char_p, [H]),
    "gpe_version": (c_char_p, []),
    "gpe_set_field": (c_int, [H, c_int, c_void_p]),
    "gpe_get_field": (c_int, [H, c_int, c_void_p]),
    "gpe_set_field_dev": (c_int, [H, c_int, c_void_p]),
    "gpe_get_field_dev": (c_int, [H, c_int, c_void_p]),
    "gpe_set_dispersion": (c_int, [H, c_void_p, c_int]),
    "gpe_set_ktable": (c_int, [H, c_void_p, c_int]),
    "gpe_set_potential": (c_int, [H, c_void_p, c_int]),
    "gpe_set_vtable": (c_int, [H, c_void_p, c_int]),
    "gpe_set_nonlinearity": (c_int, [H, c_void_p, c_void_p]),
    "gpe_set_matrix_nonlinearity": (c_int, [H, c_void_p, c_void_p]),
    "gpe_set_variant": (c_int, [H, c_int]),
    "gpe_run_ex": (c_int, [H, c_int64, c_int64, c_void_p, c_void_p, c_int64, c_void_p]),
    "gpe_set_pump": (c_int, [H, c_int, c_void_p, c_int, c_void_p, c_int64]),
    "gpe_set_noise": (c_int, [H, c_int, c_uint64, c_void_p, c_void_p]),
    "gpe_run": (c_int, [H, c_int64, c_int64, c_void_p, c_void_p]),
    "gpe_run_dev": (c_int, [H, c_int64, c_int64, c_void_p, c_void_p]),
    "gpe_run_replay": (c_int, [H, c_int64, c_int64, c_void_p, c_void_p, c_void_p]),
    "gpe_get_state": (c_int, [H, POINTER(GpeState)]),
    "gpe_set_state": (c_int, [H, POINTER(GpeState)]),
    "gpe_norm": (c_int, [H, c_void_p]),
    "gpe_energy": (c_int, [H, c_void_p]),
    "gpe_spectral_moments": (c_int, [H, c_int, c_void_p, c_void_p]),
    "gpe_set_graph": (c_int, [H, c_int64]),
    "gpe_run_async": (c_int, [H, c_int64]),
    "gpe_wait": (c_int, [H]),
    "gpe_selftest_wait": (c_int, [c_int, c_int, c_int64]),
    "gpe_set_noise_offset": (c_int, [c_void_p, c_int64]),
    "gpe_ensemble_create": (c_int, [c_void_p, c_int, POINTER(c_void_p)]),
    "gpe_ensemble_run": (c_int, [c_void_p, c_int64, c_int64]),
    "gpe_ensemble_destroy": (c_int, [c_void_p]),
    "gpe_ensemble_last_error": (c_char_p, [c_void_p]),
    "gpe_ensemble_last_run_ms": (c_double, [c_void_p]),
    "gpe_ensemble_last_run_launches": (c_int64, [c_void_p]),
    "gpe_set_timing": (c_int, [H, c_int]),
    "gpe_kernel_times": (c_int, [H, c_void_p, c_void_p]),
    "gpe_last_run_ms": (c_double, [H]),
    "gpe_last_run_launches": (c_int64, [H]),
    "gpe_norms_noalloc": (c_int, [c_void_p, c_int, c_int64, c_int64, c_int, c_double, c_void_p]),
    "gpe_noalloc_last_error": (c_char_p, []),
}

_lib = None


def load(path: Path | str | None = None):
    """Load libgpe.so and declare every entry point; raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else Path(os.environ.get("GPE_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()'); "
            "this package has no CPU fallback")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(lib, h, rc: int):
    if rc != GPE_OK:
        msg = lib.gpe_last_error(h)
        raise GPEError(rc, msg.decode() if msg else "")
    return rc


def ptr(a) -> int | None:
    """Address of a numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data
