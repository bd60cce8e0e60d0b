"""ctypes binding of libcm_fe.so (the C ABI of include/cm_fe.h).

The library is built in-tree (``cm_gb300/_build/libcm_fe.so``).  There is no
fallback: if the shared library is missing or cannot be loaded, every call
raises.  Errors returned by the C ABI become :class:`FEError`, the counterpart
of the reference's ``CMISSError`` raised by ``wrap_cmiss_routine``
(bindings/python/opencmiss/_iron_utils.py:23-78).
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcm_fe.so")

FE_NO_ERROR = 0
FE_ERR_INVALID_ARGUMENT = -1
FE_ERR_CUDA = -2
FE_ERR_OUT_OF_MEMORY = -3
FE_ERR_NOT_SUPPORTED = -4
FE_ERR_NUMERICAL = -5
FE_ERR_PATTERN = -6

FE_LAW_MOONEY_RIVLIN = 1
FE_LAW_GUCCIONE = 15
FE_HIGH_PRECISION_FP64 = 0
FE_HIGH_PRECISION_DOUBLE_FLOAT = 1
FE_ASSEMBLY_STAGED = 0
FE_ASSEMBLY_COLOURED = 1
FE_HOST_OUTPUT_STREAMED = 0
FE_HOST_OUTPUT_IN_PLACE = 1
FE_HOST_OUTPUT_AFTER = 2
FE_PRESSURE_ELEMENT_BASED = 0
FE_PRESSURE_NODE_BASED = 1
FE_NOALLOC_MAX_DOFS = 1048576


class FEError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("libcm_fe error %d: %s" % (code, message))
        self.code = code


class FEMeshDesc(C.Structure):
    _fields_ = [
        ("num_elements", C.c_int32), ("num_nodes_u", C.c_int32), ("num_nodes_p", C.c_int32),
        ("nodes_per_xi_u", C.c_int32), ("pressure_interpolation", C.c_int32), ("law", C.c_int32),
        ("num_material_components", C.c_int32), ("materials_per_element", C.c_int32),
        ("element_nodes_u", C.c_void_p), ("element_nodes_p", C.c_void_p), ("geometry", C.c_void_p),
        ("materials", C.c_void_p), ("fibre_angles", C.c_void_p),
    ]


class FENewtonOptions(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int32), ("atol", C.c_double), ("alpha", C.c_double), ("max_step", C.c_double),
        ("min_lambda", C.c_double), ("ksp_rtol", C.c_double), ("ksp_restart", C.c_int32),
        ("ksp_max_iterations", C.c_int32), ("forcing", C.c_int32),
    ]


class FENewtonReport(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32), ("converged", C.c_int32), ("linear_iterations", C.c_int64),
        ("residual_norm_initial", C.c_double), ("residual_norm", C.c_double), ("last_lambda", C.c_double),
        ("line_search_failed", C.c_int32),
    ]


# Every symbol include/cm_fe.h declares, with its argument types.
_vp, _i32, _i64 = C.c_void_p, C.c_int32, C.c_int64
SIGNATURES = {
    "fe_create": [C.POINTER(FEMeshDesc), C.POINTER(_vp)],
    "fe_destroy": [_vp],
    "fe_structure_calculate": [C.POINTER(FEMeshDesc), _i32, C.POINTER(_i64), C.POINTER(_i64), _vp, _vp],
    "fe_sizes": [_vp, C.POINTER(_i64), C.POINTER(_i64)],
    "fe_structure_calculate_device": [C.POINTER(FEMeshDesc), _i32, C.POINTER(_i64), C.POINTER(_i64), _vp, _vp, _vp],
    "fe_csr_pattern": [_vp, _i32, _vp, _vp],
    "fe_residual_evaluate": [_vp, _vp, _vp, _vp],
    "fe_residual_evaluate_noalloc": [_vp, _vp, _vp, _vp],
    "fe_jacobian_evaluate": [_vp, _vp, _vp, _vp, _vp],
    "fe_jacobian_evaluate_mixed": [_vp, _vp, _vp, _vp, _vp, _vp],
    "fe_mixed_layout": [_vp, C.POINTER(_i64), C.POINTER(_i64), _vp, _vp],
    "fe_element_size": [_vp, C.POINTER(_i32)],
    "fe_element_residuals": [_vp, _vp, _i32, _i32, _vp, _vp],
    "fe_element_jacobians": [_vp, _vp, _i32, _i32, _vp, _vp],
    "fe_set_high_precision": [_vp, _i32],
    "fe_set_assembly_order": [_vp, _i32],
    "fe_set_host_output": [_vp, _i32, _i32],
    "fe_clone": [_vp, C.POINTER(_vp)],
    "fe_set_surface_pressure": [_vp, _vp],
    "fe_set_materials": [_vp, _vp],
    "fe_newton_options_default": [C.POINTER(FENewtonOptions)],
    "fe_newton_load_step": [_vp, _vp, _vp, _i64, _vp, C.POINTER(FENewtonOptions), C.POINTER(FENewtonReport), _vp],
    "fe_check": [_vp, _vp],
    "fe_launch_count": [_vp, C.POINTER(_i64)],
    "fe_last_error": [C.c_char_p, _i32],
    "fe_batch_create": [_vp, _i32, C.POINTER(_vp)],
    "fe_batch_destroy": [_vp],
    "fe_batch_jacobian_evaluate_mixed": [_vp, _vp, _vp, _vp, _vp, _vp],
    "fe_batch_check": [_vp, _vp],
    "fe_batch_set_config": [_vp, _i32, _i32, _i32],
    "fe_batch_set_barrier_limits": [_vp, C.c_uint32, C.c_uint32],
    "fe_batch_get_config": [_vp, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32), C.POINTER(C.c_double)],
    "fe_batch_autotune": [_vp, _vp, _vp, _vp, _vp, _i32, _vp],
    "fe_batch_capture": [_vp, _vp, _vp, _vp, _vp, _vp],
    "fe_batch_replay": [_vp, _vp],
    "fe_batch_launch_count": [_vp, C.POINTER(_i64)],
    # include/cm_warmstart.h
    "ws_gemm_f32": [_i32, _i32, _i32, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, C.c_float, _vp],
    "ws_bias_act": [_vp, _vp, _i32, _i32, _i32, _vp],
    "ws_act_backward": [_vp, _vp, _vp, _i64, _i32, _vp],
    "ws_column_sum": [_vp, _vp, _i32, _i32, _vp],
    "ws_mse": [_vp, _vp, _vp, _vp, _i64, _vp],
    "ws_adam": [_vp, _vp, _vp, _vp, _i64, C.c_float, C.c_float, C.c_float, C.c_float, _i32, _vp],
    "ws_to_bf16": [_vp, _vp, _i64, _vp],
    "ws_mlp_forward_bf16": [_i32, _i32, _vp, _vp, _vp, _vp, _vp, _i32, _vp],
}

# Functions of the C ABI that return nothing.
VOID_FUNCTIONS = {"fe_newton_options_default"}

WS_ACT_IDENTITY = 0
WS_ACT_TANH = 1

_lib = None


def load(path: str | None = None):
    """Loads libcm_fe.so (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if path is None:
        from . import build as _build
        if _build._stale():
            _build.build()
    L = C.CDLL(p)
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = None if name in VOID_FUNCTIONS else C.c_int
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().fe_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int):
    if rc != FE_NO_ERROR:
        raise FEError(rc, last_error())
