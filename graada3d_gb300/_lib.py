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
    -7: "GRADA_ERR_SCRATCH_LIMIT",
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
    "grada_get_G_rows": (c_int, [c_void_p, POINTER(c_int64), c_int64, _dp]),
    "grada_G_vec_mul": (c_int, [c_void_p, _dp, _dp]),
    "grada_GT_vec_mul": (c_int, [c_void_p, _dp, _dp]),
    "grada_G_vec_mul_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_GT_vec_mul_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_forward_field": (c_int, [c_void_p, _dp, _dp]),
    "grada_expand_G": (c_int, [c_void_p, c_int64, _ip64, _dp]),
    "grada_forward_field_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_measure_fp64_peak": (c_int, [c_void_p, _dp]),
    "grada_set_operator": (c_int, [c_void_p, c_int, c_int64, c_int64, _ip32, _ip32, _dp]),
    "grada_set_cross_gradient": (c_int, [c_void_p, c_int, c_double, _dp]),
    "grada_set_data": (c_int, [c_void_p, _dp, _dp]),
    "grada_solve_cg": (c_int, [c_void_p, c_double, c_int, c_double, _dp, _dp, _dp, POINTER(_dp), _dp,
                               _dp, POINTER(c_int)]),
    "grada_invert": (c_int, [c_void_p, c_void_p, _dp, _dp, _dp, _dp, _dp, c_void_p]),
    "grada_invert_adaptive": (c_int, [c_void_p, c_void_p, c_void_p, _dp, _dp, _dp, _dp, c_void_p]),
    "grada_set_inversion_model": (c_int, [c_void_p, _dp, _dp, _dp, _dp]),
    "grada_get_model": (c_int, [c_void_p, _dp]),
    "grada_cg_phase_times": (c_int, [c_void_p, _dp, _ip64]),
    "grada_cg_loop_time": (c_int, [c_void_p, _dp, _ip64]),
    "grada_get_trials": (c_int, [c_void_p, _dp, c_int64, _ip64]),
    "grada_get_iterations": (c_int, [c_void_p, _dp, c_int64, _ip64]),
    "grada_G_vec_mul_noalloc": (c_int, [c_void_p, c_int64, c_int64, c_int64, c_void_p, c_void_p,
                                        c_void_p]),
    "grada_compute_G_batch": (c_int, [c_int, POINTER(c_void_p), c_int, c_int, POINTER(c_int)]),
    "grada_invert_batch": (c_int, [c_int, POINTER(c_void_p), c_void_p, POINTER(_dp), POINTER(_dp),
                                   POINTER(_dp), POINTER(_dp), POINTER(_dp), c_void_p, c_int,
                                   POINTER(c_int)]),
    "grada_invert_batch_persistent": (c_int, [c_int, POINTER(c_void_p), c_void_p, POINTER(_dp),
                                              POINTER(_dp), POINTER(_dp), POINTER(_dp),
                                              POINTER(_dp), c_void_p, c_int, POINTER(c_int)]),
    "grada_load_batch_tuning": (c_int, [c_char_p]),
    "grada_batch_shape": (c_int, [c_void_p, POINTER(c_int), POINTER(c_int)]),
    "grada_G_mat_mul": (c_int, [c_void_p, c_int, _dp, _dp]),
    "grada_GT_mat_mul": (c_int, [c_void_p, c_int, _dp, _dp]),
    "grada_G_block_mul_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_GT_block_mul_dev": (c_int, [c_void_p, c_void_p, c_void_p]),
    "grada_solve_cg_block": (c_int, [c_void_p, c_double, c_int, c_int, _dp, _dp, _dp, _dp,
                                     POINTER(_dp), _dp, _dp, POINTER(c_int)]),
    "grada_lambda_sweep": (c_int, [c_void_p, c_void_p, c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                   c_void_p]),
    "grada_get_sweep_trials": (c_int, [c_void_p, c_int, _dp, c_int64, _ip64]),
    "grada_inject_fault": (c_int, [c_void_p, c_int]),
    "grada_refinement_indicator": (c_int, [c_void_p, _dp, _ip64, _ip64, _dp, _dp]),
    "grada_keep_fp64_G": (c_int, [c_void_p, c_int]),
    "grada_G_column_norms": (c_int, [c_void_p, _dp]),
    "grada_build_operators": (c_int, [c_void_p, POINTER(c_int), c_double, c_int, _dp]),
    "grada_compute_G_wavelet": (c_int, [c_void_p, _ip64, c_double]),
    "grada_compute_G_wavelet_ex": (c_int, [c_void_p, _ip64, c_double, c_int]),
    "grada_get_wavelet_G": (c_int, [c_void_p, _ip64, _ip64, _ip64, POINTER(c_int), _dp]),
    "grada_get_operator": (c_int, [c_void_p, c_int, _ip64, POINTER(c_int), POINTER(c_int), _dp]),
}


class InvertParams(ctypes.Structure):
    """grada_invert_params (include/grada_gpu.h)."""

    _fields_ = [
        ("max_lambda", c_double), ("n_lambda", c_int), ("lambda_decreasing_rate", c_double),
        ("target_misfit", c_double), ("stag_tol", c_double), ("cg_tol", c_double),
        ("cg_iteration_factor", c_double), ("gn_iterations", c_int), ("lp_s", c_int),
        ("lp_x", c_int), ("lp_y", c_int), ("lp_z", c_int), ("lp_t", c_int), ("epsilon2", c_double),
        ("start_from_reference", c_int), ("fp64_refinement", c_int),
    ]


class InvertReport(ctypes.Structure):
    """grada_invert_report (include/grada_gpu.h)."""

    _fields_ = [
        ("final_misfit", c_double), ("final_lambda", c_double), ("gn_iterations", c_int),
        ("n_trials", c_int), ("cg_iterations", c_int64), ("fp64_refinements", c_int64),
        ("mesh_refinements", c_int64),
    ]


class AdaptiveParams(ctypes.Structure):
    """grada_adaptive_params (include/grada_gpu.h)."""

    _fields_ = [("max_refinement_number", c_int), ("interval_between_refinements", c_int),
                ("refine", c_void_p), ("user", c_void_p)]


# grada_refine_fn: int (*)(void *user, grada_ctx *ctx, const double *m, int64_t nm)
REFINE_FN = ctypes.CFUNCTYPE(c_int, c_void_p, c_void_p, POINTER(c_double), c_int64)

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
