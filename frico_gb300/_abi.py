"""ctypes binding of include/frico_gpu.h (libfrico_gpu.so, built in-tree).

Loading fails loudly: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfrico_gpu.so"

OK, EINVAL, ESINGULAR, ETIMEOUT, ENOMEM, ECUDA, ESTATE, ENOCONV, EMESH = 0, -1, -2, -3, -4, -5, -6, -7, -8
STATUS_NAMES = {0: "OK", -1: "EINVAL", -2: "ESINGULAR", -3: "ETIMEOUT", -4: "ENOMEM", -5: "ECUDA",
                -6: "ESTATE", -7: "ENOCONV", -8: "EMESH"}
PREC_FP64, PREC_MIXED = 0, 1
EDGE_LENGTH_XY, EDGE_LENGTH_TRUE = 0, 1
HPHASE_COMPAT, HPHASE_PHYSICAL = 0, 1
GAIN_XY, GAIN_YZ, GAIN_XZ = 0, 1, 2
GEMM_AUTO, GEMM_SIMT, GEMM_TC, GEMM_TC_F16 = 0, 1, 2, 3
PIVOT_AUTO, PIVOT_PARTIAL, PIVOT_NONE = 0, 1, 2
REFINE_AUTO, REFINE_CLASSIC = 0, 1
RESIDUAL_AUTO, RESIDUAL_FP64 = 0, 1
FIELDS_AUTO, FIELDS_DIRECT, FIELDS_GEMM = 0, 1, 2

# numpy mirror of frico_rwg (112 bytes)
RWG_DTYPE = np.dtype([
    ("Aminus", "<f8"), ("Aplus", "<f8"), ("itminus", "<i8"), ("itplus", "<i8"),
    ("pminus", "<f8", (3,)), ("pplus", "<f8", (3,)), ("length", "<f8"),
    ("edge_index", "<i8"), ("matrix_index", "<i8"), ("has_interface", "<i4"), ("interface_tag", "<i4"),
])
assert RWG_DTYPE.itemsize == 112


class C128(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class Options(C.Structure):
    _fields_ = [("degree", C.c_int32), ("approx", C.c_int32), ("force_symmetry", C.c_int32),
                ("precision", C.c_int32), ("h_phase_mode", C.c_int32), ("max_refine_iters", C.c_int32),
                ("refine_tol", C.c_double), ("Z0", C.c_double), ("profile_kernels", C.c_int32),
                ("gemm_engine", C.c_int32), ("pivoting", C.c_int32), ("refine_mode", C.c_int32),
                ("residual_mode", C.c_int32), ("wait_limit_cycles", C.c_int64), ("fields_engine", C.c_int32)]


class PortValues(C.Structure):
    _fields_ = [("voltage", C128), ("current", C128), ("power", C128), ("impedance", C128),
                ("gamma", C128), ("swr", C.c_double)]


class AdjointResult(C.Structure):
    _fields_ = [("zin", C128), ("e", C128 * 3), ("e2", C.c_double), ("dzin_re_df", C.c_double),
                ("dzin_im_df", C.c_double), ("de2_df", C.c_double)]


class SweepReport(C.Structure):
    _fields_ = [("wall_ms", C.c_double), ("fill_ms", C.c_double), ("rhs_ms", C.c_double),
                ("factor_ms", C.c_double), ("solve_ms", C.c_double), ("refine_ms", C.c_double),
                ("lump_ms", C.c_double), ("fields_ms", C.c_double), ("lanes", C.c_int32),
                ("autotuned", C.c_int32), ("nrhs", C.c_int32), ("max_refine_iters", C.c_int32),
                ("max_refine_residual", C.c_double), ("partial_pivot_fallbacks", C.c_int32),
                ("not_converged", C.c_int32), ("fp64_fallbacks", C.c_int32), ("fp64_direct", C.c_int32),
                ("kernel_launches", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("fill_ms", C.c_double), ("rhs_ms", C.c_double), ("factor_ms", C.c_double),
                ("solve_ms", C.c_double), ("refine_ms", C.c_double), ("lump_ms", C.c_double),
                ("fields_ms", C.c_double), ("refine_iters", C.c_int32), ("refine_residual", C.c_double),
                ("n", C.c_int64), ("ntri", C.c_int64), ("nrhs", C.c_int64), ("green_evals", C.c_int64),
                ("kernel_launches", C.c_int64), ("gemm_launches", C.c_int64), ("gemm_ms", C.c_double),
                ("gemm_flops", C.c_double), ("gemm_bytes", C.c_double), ("pivoting_used", C.c_int32),
                ("precision_used", C.c_int32)]


P = C.c_void_p
I32, I64, D = C.c_int32, C.c_int64, C.c_double
PD = C.POINTER(C.c_double)

PROTOTYPES = {
    "frico_gpu_make_function_space": [I64, P, I64, P, I64, P, P, I32, P, I64, P, P, P, P, P],
    "frico_gpu_reorient_deltagap": [I64, P, P, P, I64, P, P, I32, P, I32, P, P],
    "frico_gpu_ctx_create": [P, C.c_int, P],
    "frico_gpu_ctx_destroy": [P],
    "frico_gpu_set_options": [P, P],
    "frico_gpu_last_error": [P],
    "frico_gpu_get_stream": [P, P],
    "frico_gpu_set_mesh": [P, I64, P, I64, P, I64, P],
    "frico_gpu_fill": [P, D, P, I64],
    "frico_gpu_set_nrhs": [P, I32],
    "frico_gpu_rhs_delta_gap": [P, D, I32, I32, P, C128, P],
    "frico_gpu_rhs_plane_wave": [P, D, I32, D, D, C128, C128],
    "frico_gpu_set_rhs": [P, I32, P, I64],
    "frico_gpu_get_rhs": [P, P, I64],
    "frico_gpu_solve": [P, P, I64, P],
    "frico_gpu_get_factors": [P, P, I64, P],
    "frico_gpu_lump_currents": [P, I32, P, P, P],
    "frico_gpu_eval_fields": [P, I32, I64, P, P, P],
    "frico_gpu_eval_fields_noalloc": [P, I32, I64, P, P, P],
    "frico_gpu_set_matrix": [P, D, P, I64],
    "frico_gpu_sweep": [P, I32, P, I32, P, C128, P, I32, P, I64, P, I32, P, P, P, P],
    "frico_gpu_adjoint": [P, D, I32, P, C128, P, P, I32, P, P, P, P],
    "frico_gpu_eval_fields_multi": [P, I32, I32, I64, P, P, P],
    "frico_gpu_rcs_points_multi": [P, I32, I32, D, I64, P, P, P],
    "frico_gpu_port_values": [P, I32, I32, P, C128, P, P],
    "frico_gpu_gain": [P, I32, D, D, I32, P],
    "frico_gpu_bistatic_rcs": [P, I32, D, P],
    "frico_gpu_rcs_points": [P, I32, D, I64, P, P, P],
    "frico_gpu_last_stats": [P, P],
    "frico_gpu_debug_cgemm": [P, I32, I32, I32, P, P, P, I32],
    "frico_gpu_debug_z64": [P, P, P],
    "frico_gpu_debug_fields_gemm_config": [I32, I32],
}

_lib = None


def load() -> C.CDLL:
    """Load libfrico_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m frico_gb300.build` (no CPU fallback exists)")
        lib = C.CDLL(str(LIB_PATH))
        for name, args in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_char_p if name == "frico_gpu_last_error" else C.c_int
        _lib = lib
    return _lib


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class FricoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code
