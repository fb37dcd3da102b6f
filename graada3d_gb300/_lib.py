"""ctypes binding of ``libgrada_gpu.so`` (the C ABI declared in
``include/grada_gpu.h``).

Loading fails loudly when the library has not been built: there is no CPU
fallback for any entry point.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_uint32, c_void_p, c_char_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgrada_gpu.so"

GRADA_OK = 0
STATUS_NAMES = {
    -1: "GRADA_ERR_INVALID_ARGUMENT",
    -2: "GRADA_ERR_CUDA",
    -3: "GRADA_ERR_OUT_OF_MEMORY",
    -4: "GRADA_ERR_STATE",
    -5: "GRADA_ERR_NONFINITE",
    -6: "GRADA_ERR_BREAKDOWN",
}

_dp = POINTER(c_double)
_ip64 = POINTER(c_int64)
_ip32 = POINTER(c_int32)

# name -> (restype, argtypes)
SIGNATURES = {
    "grada_version": (c_int, []),
    "grada_ctx_create": (c_int, [c_int, POINTER(c_void_p)]),
    "grada_ctx_destroy": (c_int, [c_void_p]),
    "grada_last_error": (c_char_p, [c_void_p]),
    "grada_ctx_stream": (c_void_p, [c_void_p]),
    "grada_sync": (c_int, [c_void_p]),
    "grada_ctx_device_bytes": (c_int64, [c_void_p]),
    "grada_set_geometry": (c_int, [c_void_p, _dp, c_int64, _dp, c_int64, c_uint32]),
    "grada_get_dims": (c_int, [c_void_p, _ip64, _ip64, POINTER(c_int), _ip64, _ip64]),
    "grada_compute_G": (c_int, [c_void_p, c_int]),
    "grada_G_storage": (c_int, [c_void_p]),
    "grada_get_G": (c_int, [c_void_p, _dp, c_int64]),
    "grada_G_vec_mul": (c_int, [c_void_p, _dp, _dp]),
    "grada_GT_vec_mul": (c_int, [c_void_p, _dp, _dp]),
    "grada_G_vec_mul_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_GT_vec_mul_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_forward_field": (c_int, [c_void_p, _dp, _dp]),
    "grada_forward_field_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_measure_fp64_peak": (c_int, [c_void_p, _dp]),
}

_lib = None


class GradaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: Path | None = None):
    """Load the CUDA library once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')"
        )
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(SIGNATURES)
