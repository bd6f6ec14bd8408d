"""ctypes binding of ``libopencloth_gb.so`` (the C ABI in include/opencloth_gb.h).

There is no fallback: if the native library is missing this module raises, so no
Python or CPU path can stand in for the CUDA step.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libopencloth_gb.so"

SPRING_DTYPE = np.dtype(
    [("p1", "<i4"), ("p2", "<i4"), ("rest_length", "<f4"), ("ks", "<f4"), ("kd", "<f4"), ("type", "<i4")]
)

OC_OK = 0
STATUS_NAMES = {
    0: "OC_OK",
    1: "OC_ERR_INVALID_ARGUMENT",
    2: "OC_ERR_BAD_INDEX",
    3: "OC_ERR_NON_FINITE",
    4: "OC_ERR_DEGENERATE",
    5: "OC_ERR_CUDA",
    6: "OC_ERR_OUT_OF_MEMORY",
    7: "OC_ERR_UNSUPPORTED",
    8: "OC_ERR_DEVICE_TIMEOUT",
}
FLAG_NOT_CONVERGED = 1
FLAG_BREAKDOWN = 2
FLAG_NON_FINITE = 4

EXEC_AUTO, EXEC_STREAMED, EXEC_RESIDENT, EXEC_PLAIN = 0, 1, 2, 3
JAC_REFERENCE, JAC_COUPLED = 0, 1
PASS_ELLIPSOID, PASS_PROVOT = 1, 2


class Spring(C.Structure):
    _fields_ = [("p1", C.c_int32), ("p2", C.c_int32), ("rest_length", C.c_float), ("ks", C.c_float),
                ("kd", C.c_float), ("type", C.c_int32)]


class ClothDescC(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32),
        ("n_springs", C.c_int32),
        ("springs", C.c_void_p),
        ("mass", C.c_void_p),
        ("pinned", C.c_void_p),
        ("n_pinned", C.c_int32),
        ("ext_force", C.c_void_p),
        ("gravity", C.c_float * 3),
        ("velocity_damping", C.c_float),
        ("cg_max_iter", C.c_int32),
        ("cg_tol", C.c_float),
        ("jacobian_mode", C.c_int32),
        ("passes", C.c_int32),
        ("ellipsoid", C.c_float * 16),
        ("ellipsoid_inv", C.c_float * 16),
        ("provot_ratio", C.c_float),
    ]


class BsrDescC(C.Structure):
    _fields_ = [
        ("n_rows", C.c_int32),
        ("nnzb", C.c_int32),
        ("row_ptr", C.c_void_p),
        ("col", C.c_void_p),
        ("fixed", C.c_void_p),
        ("cg_max_iter", C.c_int32),
        ("tolerance", C.c_float),
        ("tiny", C.c_float),
    ]


class OptionsC(C.Structure):
    _fields_ = [
        ("executor", C.c_int32),
        ("device", C.c_int32),
        ("stream", C.c_void_p),
        ("use_graph", C.c_int32),
        ("block_threads", C.c_int32),
        ("vertices_per_thread", C.c_int32),
        ("resident_max_vertices", C.c_int32),
    ]


class LaunchConfigC(C.Structure):
    _fields_ = [(name, C.c_int32) for name in (
        "resident_max_vertices", "resident_vcta", "resident_threads", "resident_fused", "persist", "gather_variant",
        "strip", "strip_rows", "strip_variant")]


TUNE_USE_CACHE, TUNE_STORE = 1, 2

# name -> (restype, argtypes); every symbol include/opencloth_gb.h declares.
_P = C.c_void_p
SIGNATURES = {
    "oc_default_options": (None, [C.POINTER(OptionsC)]),
    "oc_create": (C.c_int32, [C.POINTER(ClothDescC), C.c_int32, C.POINTER(OptionsC), C.POINTER(_P)]),
    "oc_destroy": (None, [_P]),
    "oc_last_error": (C.c_char_p, [_P]),
    "oc_status_string": (C.c_char_p, [C.c_int32]),
    "oc_get_counts": (C.c_int32, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "oc_get_vertex_offsets": (C.c_int32, [_P, _P]),
    "oc_set_state": (C.c_int32, [_P, _P, _P, _P]),
    "oc_get_state": (C.c_int32, [_P, _P, _P, _P]),
    "oc_set_state_device": (C.c_int32, [_P, _P, _P, _P]),
    "oc_get_state_device": (C.c_int32, [_P, _P, _P, _P]),
    "oc_step": (C.c_int32, [_P, C.c_float, C.c_int32]),
    "oc_step_host": (C.c_int32, [_P, C.c_float, C.c_int32, _P, _P]),
    "oc_synchronize": (C.c_int32, [_P]),
    "oc_set_passes": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "oc_apply_passes": (C.c_int32, [_P, C.c_int32]),
    "oc_pick_vertex": (C.c_int32, [_P, C.c_int32, _P, C.c_double, C.POINTER(C.c_int32)]),
    "oc_drag_vertex": (C.c_int32, [_P, C.c_int32, C.c_int32, _P]),
    "oc_set_vertices": (C.c_int32, [_P, C.c_int32, _P, _P, _P]),
    "oc_set_pins": (C.c_int32, [_P, C.c_int32, _P, C.c_int32]),
    "oc_get_stats": (C.c_int32, [_P, _P, _P, _P]),
    "oc_get_launch_count": (C.c_int32, [_P, C.POINTER(C.c_int64)]),
    "oc_compute_forces": (C.c_int32, [_P, _P]),
    "oc_assemble": (C.c_int32, [_P, C.c_float, _P, _P]),
    "oc_profile_steps": (C.c_int32, [_P, C.c_float, C.c_int32, C.c_int32, _P, _P, _P, _P, _P]),
    "oc_set_spring_params": (C.c_int32, [_P, _P, _P]),
    "oc_set_ext_force": (C.c_int32, [_P, _P]),
    "oc_tape_forward": (C.c_int32, [_P, C.c_float, C.c_int32, C.c_int32, C.c_int64]),
    "oc_tape_backward": (C.c_int32, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "oc_tape_info": (C.c_int32, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "oc_tape_forward_intervals": (C.c_int32, [_P, C.c_float, C.c_int32, C.c_void_p]),
    "oc_tape_layout": (C.c_int32, [_P, C.POINTER(C.c_int32), C.c_void_p]),
    "oc_test_barrier_timeout": (C.c_int32, [_P, C.c_int32, C.c_uint32]),
    "oc_test_cr_arith": (C.c_int32, [C.c_int32, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]),
    "oc_set_tape_mode": (C.c_int32, [_P, C.c_int32]),
    "oc_tape_displacement": (C.c_int32, [_P, _P]),
    "oc_get_launch_config": (C.c_int32, [_P, C.POINTER(LaunchConfigC)]),
    "oc_set_launch_config": (C.c_int32, [_P, C.POINTER(LaunchConfigC)]),
    "oc_autotune": (C.c_int32, [_P, C.c_float, C.c_char_p, C.c_int32, C.POINTER(LaunchConfigC),
                                C.POINTER(C.c_double)]),
    "oc_tune_key": (C.c_int32, [C.POINTER(ClothDescC), C.c_int32, C.c_char_p, C.c_int32, C.c_char_p, C.c_int32]),
    "oc_tune_key_of": (C.c_int32, [_P, C.c_char_p, C.c_int32]),
    "oc_tune_cache_lookup": (C.c_int32, [C.c_char_p, C.c_char_p, C.POINTER(LaunchConfigC), C.POINTER(C.c_int32)]),
    "oc_tune_cache_store": (C.c_int32, [C.c_char_p, C.c_char_p, C.POINTER(LaunchConfigC), C.c_double]),
    "oc_pcg_solve_noalloc": (C.c_int32, [_P, _P, _P, _P, C.c_int32, C.c_int32, C.c_float, C.POINTER(C.c_int32),
                                         C.POINTER(C.c_uint32), _P]),
    "oc_bsr_create": (C.c_int32, [C.POINTER(BsrDescC), C.c_int32, C.POINTER(OptionsC), C.POINTER(_P)]),
    "oc_bsr_destroy": (None, [_P]),
    "oc_bsr_last_error": (C.c_char_p, [_P]),
    "oc_bsr_get_counts": (C.c_int32, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "oc_bsr_set_system": (C.c_int32, [_P, _P, _P, _P]),
    "oc_bsr_solve": (C.c_int32, [_P]),
    "oc_bsr_get_solution": (C.c_int32, [_P, _P, _P]),
    "oc_bsr_get_launch_count": (C.c_int32, [_P, C.POINTER(C.c_int64)]),
    "oc_bsr_synchronize": (C.c_int32, [_P]),
    "oc_bsr_profile": (C.c_int32, [_P, C.c_int32, C.c_int32, _P, _P, _P, _P, _P]),
    "oc_describe_instances": (C.c_int32, [C.POINTER(ClothDescC), C.c_int32, _P, _P]),
    "oc_grid_spring_count": (C.c_int32, [C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
    "oc_grid_build": (C.c_int32, [C.c_int32, C.c_int32, C.c_float, _P, _P, C.c_float, C.c_uint64, _P, _P]),
}

_lib = None


def load() -> C.CDLL:
    """Load the native library (built by ``opencloth_gb300.build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"native library {LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)"
        )
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class OcError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


def ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data
