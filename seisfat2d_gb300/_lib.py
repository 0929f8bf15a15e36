"""ctypes binding of the engine's C ABI (include/seisfat2d.h).

The shared library is built in-tree by ``seisfat2d_gb300.build``; loading fails
loudly when it is missing (there is no CPU fallback).
"""
import ctypes as C
import os

from . import build as _build

SF_OK = 0
SF_ERR_ARG = 1
SF_ERR_CUDA = 2
SF_ERR_TIMEOUT = 3
SF_ERR_RANGE = 4
SF_ERR_STATE = 5
SF_ERR_NOMEM = 6

SF_MEM_HOST = 0
SF_MEM_DEVICE = 1
SF_LAYOUT_MODEL = 0
SF_LAYOUT_PADDED = 1
SF_ARITH_REFERENCE = 0
SF_ARITH_IEEE = 1
SF_ARITH_COMPENSATED = 2
SF_KEEP_TAPE = 1
SF_KEEP_TABLES = 2


class sf_shot(C.Structure):
    _fields_ = [("sx", C.c_float), ("sz", C.c_float), ("c0", C.c_int), ("ncols", C.c_int)]


VP = C.c_void_p
FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int)

# name -> (restype, argtypes); the set of exported entry points of the ABI
SIGNATURES = {
    "sf_status_string": (C.c_char_p, [C.c_int]),
    "sf_ctx_last_error": (C.c_char_p, [VP]),
    "sf_ctx_create": (C.c_int, [C.POINTER(VP), C.c_int, C.c_int, C.c_float, C.c_float, C.c_int]),
    "sf_ctx_destroy": (C.c_int, [VP]),
    "sf_ctx_dims": (C.c_int, [VP, IP, IP, IP]),
    "sf_set_slowness": (C.c_int, [VP, VP, C.c_int, C.c_int]),
    "sf_get_slowness": (C.c_int, [VP, VP, C.c_int]),
    "sf_set_stiffness": (C.c_int, [VP, VP * 6, C.c_int]),
    "sf_set_stiffness_codes": (C.c_int, [VP, VP * 6, VP, C.c_int]),
    "sf_time_propagation": (C.c_int, [VP, C.c_int, C.c_float, C.c_float, VP, C.c_int, VP]),
    "sf_compute_seismogram": (C.c_int, [VP, VP, VP, VP, C.c_int, VP, C.c_int, VP]),
    "sf_batch_forward": (C.c_int, [VP, C.c_int, C.POINTER(sf_shot), C.c_int, VP, VP, C.c_int, VP,
                                   C.c_int, C.c_int, VP]),
    "sf_batch_table": (C.c_int, [VP, C.c_int, VP, C.c_int, VP]),
    "sf_batch_adjoint": (C.c_int, [VP, VP, C.c_int, VP, C.c_int, VP]),
    "sf_batch_tape_codes": (C.c_int, [VP, C.c_int, VP, C.c_int, VP]),
    "sf_batch_misfit_gradient": (C.c_int, [VP, VP, C.c_int, C.POINTER(C.c_double), VP, C.c_int, VP]),
    "sf_batch_stiffness_gradient": (C.c_int, [VP, VP, VP, C.c_int, VP]),
    "sf_synchronize": (C.c_int, [VP, VP]),
    "sf_set_wait_limit": (C.c_int, [VP, C.c_double]),
    "sf_test_stall_next_batch": (C.c_int, [VP]),
    "sf_set_launch": (C.c_int, [VP, C.c_int, C.c_int]),
    "sf_set_arithmetic": (C.c_int, [VP, C.c_int]),
    "sf_get_arithmetic": (C.c_int, [VP, IP]),
    "sf_get_launch": (C.c_int, [VP, IP, IP]),
    "sf_set_strip_loop": (C.c_int, [VP, C.c_int]),
    "sf_set_fused_gather": (C.c_int, [VP, C.c_int]),
    "sf_get_fused_gather": (C.c_int, [VP, IP, IP]),
    "sf_get_strip_loop": (C.c_int, [VP, IP, IP]),
    "sf_time_propagation_noalloc": (C.c_int, [VP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                              C.c_float, VP, VP]),
    "sf_plan_batch": (C.c_int, [VP, C.POINTER(sf_shot), C.c_int, VP, VP, C.c_int, VP]),
    "sf_plan_iteration": (C.c_int, [VP, VP, VP, VP, VP, VP]),
    "sf_plan_graph_launch": (C.c_int, [VP, VP, VP, VP, VP, VP]),
    "sf_plan_autotune": (C.c_int, [VP, VP, VP, VP, VP, C.c_int, VP, IP, IP, FP]),
    "sf_set_kernel_timing": (C.c_int, [VP, C.c_int]),
    "sf_kernel_times": (C.c_int, [VP, FP, C.c_int]),
    "sf_smooth_model": (C.c_int, [VP, VP, VP, C.c_float, C.c_int, C.c_int, VP]),
    "sf_update_slowness": (C.c_int, [VP, VP, C.c_int, C.c_float, C.c_float, C.c_int, VP, C.c_int, VP]),
    "sf_adjoint_convolution": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, VP]),
    "sf_kirchhoff_image": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, VP, VP, VP, C.c_int, C.c_int, C.c_float,
                                     C.c_float, C.c_float, VP, C.c_int, VP]),
    "sf_kirchhoff_angle_gathers": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, VP, VP, VP, C.c_int, C.c_int,
                                             C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, VP, C.c_int,
                                             IP, IP, VP]),
    "sf_forward_convolution": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, VP]),
    "sf_kirchhoff_image_forward": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, VP, VP, VP, C.c_int, C.c_int,
                                             C.c_float, C.c_float, C.c_float, VP, C.c_int, VP]),
    "sf_kirchhoff_angle_forward": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, VP, VP, VP, C.c_int, C.c_int,
                                             C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, VP, C.c_int,
                                             VP]),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load libseisfat2d.so (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(
                "libseisfat2d.so is not built; run seisfat2d_gb300.build.build() "
                "(the engine has no CPU fallback)")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class EngineError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status
