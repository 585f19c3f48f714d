"""ctypes declarations of libantipodal_gb300.so (the C ABI in include/antipodal_gb300.h)."""

from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libantipodal_gb300.so")

_P = C.c_void_p
_I64 = C.c_int64
_I = C.c_int
_D = C.c_double
_PP = C.POINTER(C.c_void_p)

AGWN_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "out of device memory",
          4: "BVH traversal stack exhausted", 5: "device wait timed out", 6: "unsupported", 7: "no CUDA device"}

OPT_FRAC_MODE, OPT_MIXED_TAU, OPT_QUERIES_PER_THREAD, OPT_FRAC_BLOCK, OPT_TIMING, OPT_SEG_TILE, \
    OPT_MIXED_TERM_ERR, OPT_ROBUST_MODE, OPT_ROBUST_TERM_ERR, OPT_PARAM_MODE, OPT_INTEGER_CELLS, \
    OPT_MIXED_MIN_PAIRS, OPT_MIXED_CERTIFY = range(13)
ROBUST_EXACT, ROBUST_MIXED = 0, 1
PARAM_EXACT, PARAM_MIXED = 0, 1
FRAC_EXACT, FRAC_MIXED = 0, 1
K_FRACTIONAL, K_INTEGER, K_ROBUST, K_PARAMETRIC, K_OTHER, K_COUNT = range(6)


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double * K_COUNT), ("launches", C.c_int64 * K_COUNT),
                ("fp64_pairs", C.c_int64), ("pairs", C.c_int64), ("int_queries", C.c_int64),
                ("int_cell_entries", C.c_int64), ("int_leaves", C.c_int64), ("int_exact_tests", C.c_int64),
                ("patch_pairs", C.c_int64), ("patch_cells", C.c_int64), ("patch_pieces", C.c_int64),
                ("patch_fp64_pairs", C.c_int64), ("certified_pairs", C.c_int64)]


# name -> (restype, argtypes)
SIGNATURES = {
    "agwn_status_string": (C.c_char_p, [_I]),
    "agwn_last_error_message": (C.c_char_p, []),
    "agwn_abi_version": (_I, []),
    "agwn_context_create": (_I, [_I, _P, _PP]),
    "agwn_context_destroy": (_I, [_P]),
    "agwn_context_synchronize": (_I, [_P]),
    "agwn_context_set_option": (_I, [_P, _I, _D]),
    "agwn_context_get_option": (_I, [_P, _I, C.POINTER(_D)]),
    "agwn_context_get_stats": (_I, [_P, C.POINTER(Stats), _I]),
    "agwn_mesh_batch_fractional_f64": (_I, [_P, _P, _I64, _P, _P, _P, _I64]),
    "agwn_mesh_batch_fractional_f32": (_I, [_P, _P, _I64, _P, _P, _P, _I64]),
    "agwn_bvh_create_f64": (_I, [_P, _P, _I64, _P, _I64, _PP]),
    "agwn_bvh_create_f32": (_I, [_P, _P, _I64, _P, _I64, _PP]),
    "agwn_bvh_destroy": (_I, [_P]),
    "agwn_bvh_info": (_I, [_P, C.POINTER(_I64), C.POINTER(C.c_int32)]),
    "agwn_mesh_batch_integer_f64": (_I, [_P, _P, _P, _I64, _P, _P]),
    "agwn_mesh_batch_integer_f32": (_I, [_P, _P, _P, _I64, _P, _P]),
    "agwn_mesh_batch_f64": (_I, [_P, _P, _P, _I64, _P, _P, _P, _I64]),
    "agwn_mesh_batch_f32": (_I, [_P, _P, _P, _I64, _P, _P, _P, _I64]),
    "agwn_mesh_batch_integer_bruteforce_f64": (_I, [_P, _P, _I64, _P, _I64, _P, _I64, _P, _P]),
    "agwn_mesh_batch_integer_ties_f64": (_I, [_P, _P, _I64, _P, _I64, _P, _I64, _P, _P, _P]),
    "agwn_robust_create_f64": (_I, [_P, _I, _P, _I64, _P, _I64, _P, _I64, _PP]),
    "agwn_robust_create_f32": (_I, [_P, _I, _P, _I64, _P, _I64, _P, _I64, _PP]),
    "agwn_robust_destroy": (_I, [_P]),
    "agwn_robust_info": (_I, [_P, _P, C.POINTER(_D), C.POINTER(C.c_int32)]),
    "agwn_robust_eval_f64": (_I, [_P, _P, _P, _I64, _P, _P, _P]),
    "agwn_robust_eval_f32": (_I, [_P, _P, _P, _I64, _P, _P, _P]),
    "agwn_probe_fp32_peak": (_I, [_P, C.POINTER(_D)]),
    "agwn_probe_atan2": (_I, [_P, _P, _P, _I64, _P, _P]),
    "agwn_probe_fp64_peak": (_I, [_P, _P]),
    "agwn_robust_predicates": (_I, [_P, _I, _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    "agwn_probe_i128_mul_sub": (_I, [_P, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "agwn_param_batch_fractional_bezier3_f64": (_I, [_P, _P, _I64, _P, _P, _P, _I64, _I, _I, _D, _P, _P, _P]),
    "agwn_robust_eval_grid_f64": (_I, [_P, _P, _P, _P, _I64, _I64, _I64, _P, _P, _P]),
    "agwn_robust_eval_grid_f32": (_I, [_P, _P, _P, _P, _I64, _I64, _I64, _P, _P, _P]),
    "agwn_build_boundary_segments_f64": (_I, [_P, _P, _I64, _P, _I64, _P, _I64, _P]),
    "agwn_build_boundary_segments_f32": (_I, [_P, _P, _I64, _P, _I64, _P, _I64, _P]),
    "agwn_batch_create": (_I, [_P, _P, C.c_int32, _P, _P, _P, _P, _PP]),
    "agwn_batch_destroy": (_I, [_P]),
    "agwn_batch_tune": (_I, [_P, _P, C.c_int32]),
    "agwn_batch_set_config": (_I, [_P, _P]),
    "agwn_batch_info": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "agwn_batch_run": (_I, [_P, _P, C.c_int32]),
    "agwn_param_batch_fractional_learned_bezier3_f64": (_I, [_P, _P, _P, _I64, _P, _P, _P, _I64, _I, _I, _I, _D,
                                                             C.c_float, _P, _P]),
    "agwn_param_set_panel_network": (_I, [_P, _P, C.c_float]),
    "agwn_patches_create_f64": (_I, [_P, _P, _I64, _PP]),
    "agwn_patches_destroy": (_I, [_P]),
    "agwn_param_batch_integer_bezier3x3_f64": (_I, [_P, _P, _P, _I64, _P, _P]),
    "agwn_param_batch_integer_degenerate_bezier3x3_f64": (_I, [_P, _P, _P, _I64, _P, _P, _P]),
    "agwn_param_add_integer_bezier3x3_f64": (_I, [_P, _P, _P, _I64, _P, _P]),
    "agwn_param_panel_log_bezier3_f64": (_I, [_P, _P, _I64, _P, _P, _I64, _I, _I, _D, _P, _I64, _P]),
    "agwn_param_panel_features_bezier3_f64": (_I, [_P, _P, _I64, _P, _P, _I64, _D, _P, _I64, _P, _P]),
    "agwn_mlp_param_count": (_I, []),
    "agwn_mlp_create": (_I, [_P, C.c_uint64, _PP]),
    "agwn_mlp_destroy": (_I, [_P]),
    "agwn_mlp_set_params": (_I, [_P, _P, _P]),
    "agwn_mlp_get_params": (_I, [_P, _P, _P]),
    "agwn_param_features_bezier3_f64": (_I, [_P, _P, _I64, _P, _P, _I64, _D, _P]),
    "agwn_mlp_loss_grad": (_I, [_P, _P, _P, _P, _I64, _I, _P, _P]),
    "agwn_mlp_train": (_I, [_P, _P, _P, _P, _I64, _I, _I, _I, C.c_float, C.c_uint64, _P]),
    "agwn_param_propose_depth_bezier3_f64": (_I, [_P, _P, _P, _I64, _P, _P, _I64, _I, _I, _I, _D, C.c_float, _P,
                                                  _P]),
}

_lock = threading.Lock()
_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Loads the library once; raises if it has not been built (there is no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                f"{p} is missing: build the CUDA extension first (python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def declared_symbols() -> list[str]:
    return list(SIGNATURES)
