"""ctypes binding of libvfsm103.so (include/volumefluxes_sm103.h).

The library is the only compute path: if it is missing or fails to load, every
entry point raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(os.environ.get("VF_SM103_LIB", Path(__file__).resolve().parent / "lib" / "libvfsm103.so"))

VF_ABI_VERSION = 2
VF_MAX_SOURCES = 8
VF_OK, VF_EINVAL, VF_ENOMEM, VF_ECUDA, VF_ESTATE = 0, -1, -2, -3, -4
VF_SRC_BOTTOM, VF_SRC_CONST_RAIN, VF_SRC_CONST_INFIL = 1, 2, 3
VF_SRC_TIME_RAIN, VF_SRC_HORTON, VF_SRC_RAIN_FIELD = 4, 5, 6
VF_FRICTION_NONE, VF_FRICTION_BSA2012, VF_FRICTION_FCG2016, VF_FRICTION_BH2021 = 0, 1, 2, 3
VF_STEPPER_FE, VF_STEPPER_RK2 = 1, 2
VF_BC_WALL, VF_BC_PERIODIC, VF_BC_NEUMANN = 1, 2, 3
VF_REC_LINEAR, VF_REC_NONE = 1, 2
VF_ARITH_REFERENCE, VF_ARITH_FAITHFUL = 0, 1

# Every symbol include/volumefluxes_sm103.h declares.
EXPORTED_SYMBOLS = (
    "vf_create", "vf_destroy", "vf_upload_bottom", "vf_set_source_table", "vf_set_source_field",
    "vf_set_interior_state", "vf_upload_state",
    "vf_download_state", "vf_get_interior_state", "vf_step", "vf_set_arithmetic", "vf_simulate", "vf_water_volume",
    "vf_device_state", "vf_stream", "vf_time_steps", "vf_time_kernels", "vf_selftest_tile_wait", "vf_selftest_quotients",
    "vf_selftest_near_dry_quotients",
    "vf_last_error",
    "vf_launch_count",
    "vf_water_volume_static",
    "vf_batch_launch", "vf_batch_poll", "vf_batch_is_done", "vf_batch_collect", "vf_batch_wait", "vf_batch_free",
    "vf_batch_simulate", "vf_batch_cluster_size", "vf_batch_last_error",
    "vf_server_create", "vf_server_submit", "vf_server_poll", "vf_server_result", "vf_server_timing",
    "vf_server_release",
    "vf_server_stats", "vf_server_destroy", "vf_server_last_error",
    "vf_sample_cells", "vf_step_fixed", "vf_adjoint_create", "vf_adjoint_forward", "vf_adjoint_backward", "vf_adjoint_destroy",
    "vf_adjoint_last_error",
)
VF_BATCH_OK, VF_BATCH_TIMEOUT, VF_BATCH_STALLED, VF_BATCH_MAX_STEPS = 0, 1, 2, 3
VF_STATIC_MAX_ROWS = 16384


class VfConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("gc", C.c_int32),
        ("extent", C.c_double * 4),
        ("real_bytes", C.c_int32),
        ("g", C.c_double), ("rho", C.c_double), ("depth_cutoff", C.c_double), ("desingularizing_kappa", C.c_double),
        ("reconstruction", C.c_int32),
        ("theta", C.c_double),
        ("n_sources", C.c_int32),
        ("source_kind", C.c_int32 * VF_MAX_SOURCES),
        ("source_rate", C.c_double * VF_MAX_SOURCES),
        ("source_aux", (C.c_double * 2) * VF_MAX_SOURCES),
        ("friction", C.c_int32), ("friction_Cz", C.c_double),
        ("stepper", C.c_int32), ("bc", C.c_int32), ("cfl", C.c_double),
        ("bottom_is_constant", C.c_int32), ("bottom_constant", C.c_double),
        ("device", C.c_int32),
    ]


class VfBatchOptions(C.Structure):
    _fields_ = [("tiles_per_cta", C.c_int32), ("max_cluster", C.c_int32), ("time_limit_s", C.c_double),
                ("seg_rows", C.c_int32), ("wide_cells", C.c_int64)]


class NativeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def library_path() -> Path:
    return LIB_PATH


def load(build_if_missing: bool = False):
    """Load libvfsm103.so once. Raises if it is absent (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() and build_if_missing:
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "_vf_build_native", Path(__file__).resolve().parent.parent / "build_native.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    if not LIB_PATH.exists():
        raise ImportError(
            f"libvfsm103.so not found at {LIB_PATH}; build it with volumefluxes.jl_gb300/build_native.py "
            "(the sm_103a library is the only compute path)")
    lib = C.CDLL(os.fspath(LIB_PATH))
    H = C.c_void_p
    sig = {
        "vf_create": (C.c_int, [C.POINTER(VfConfig), C.POINTER(C.c_void_p)]),
        "vf_destroy": (None, [H]),
        "vf_upload_bottom": (C.c_int, [H, C.c_void_p]),
        "vf_set_interior_state": (C.c_int, [H, C.c_void_p, C.c_void_p, C.c_void_p]),
        "vf_upload_state": (C.c_int, [H, C.c_void_p]),
        "vf_download_state": (C.c_int, [H, C.c_void_p]),
        "vf_get_interior_state": (C.c_int, [H, C.c_void_p, C.c_void_p, C.c_void_p]),
        "vf_step": (C.c_int, [H, C.c_double, C.c_double, C.POINTER(C.c_double)]),
        "vf_set_arithmetic": (C.c_int, [H, C.c_int32]),
        "vf_set_source_table": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
        "vf_set_source_field": (C.c_int, [H, C.c_int32, C.c_void_p]),
        "vf_simulate": (C.c_int, [H, C.c_double, C.c_double, C.c_int32, C.c_double, C.c_double, C.c_int64,
                                  C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
        "vf_water_volume": (C.c_int, [H, C.POINTER(C.c_double)]),
        "vf_device_state": (C.c_int, [H, C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]),
        "vf_stream": (C.c_int, [H, C.POINTER(C.c_void_p)]),
        "vf_time_steps": (C.c_int, [H, C.c_int64, C.POINTER(C.c_float)]),
        "vf_selftest_tile_wait": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32)]),
        "vf_selftest_quotients": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
        "vf_selftest_near_dry_quotients": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                                     C.c_void_p]),
        "vf_time_kernels": (C.c_int, [H, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "vf_last_error": (C.c_char_p, [H]),
        "vf_water_volume_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                             C.c_double, C.c_double, C.c_int32, C.c_double, C.c_void_p,
                                             C.c_void_p]),
        "vf_launch_count": (C.c_int64, [H]),
        "vf_batch_launch": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_double,
                                      C.c_int64, C.POINTER(VfBatchOptions), C.POINTER(C.c_void_p)]),
        "vf_batch_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
        "vf_batch_is_done": (C.c_int, [C.c_void_p, C.c_int32]),
        "vf_batch_collect": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
        "vf_batch_wait": (C.c_int, [C.c_void_p]),
        "vf_batch_free": (C.c_int, [C.c_void_p]),
        "vf_batch_simulate": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                        C.c_double, C.c_int64, C.POINTER(VfBatchOptions), C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
        "vf_batch_cluster_size": (C.c_int, [H, C.POINTER(VfBatchOptions), C.POINTER(C.c_int32)]),
        "vf_batch_last_error": (C.c_char_p, [C.c_void_p]),
        "vf_server_create": (C.c_int, [C.c_int32, C.c_int64, C.POINTER(VfBatchOptions), C.c_int64,
                                       C.POINTER(C.c_void_p)]),
        "vf_server_submit": (C.c_int, [C.c_void_p, C.POINTER(VfConfig), C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(C.c_int64)]),
        "vf_server_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32)]),
        "vf_server_result": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
        "vf_server_timing": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
        "vf_server_release": (C.c_int, [C.c_void_p, C.c_int64]),
        "vf_server_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int64)]),
        "vf_server_destroy": (C.c_int, [C.c_void_p]),
        "vf_server_last_error": (C.c_char_p, [C.c_void_p]),
        "vf_sample_cells": (C.c_int, [H, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
        "vf_step_fixed": (C.c_int, [H, C.c_double, C.c_double]),
        "vf_adjoint_create": (C.c_int, [H, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
        "vf_adjoint_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
        "vf_adjoint_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                          C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_double)]),
        "vf_adjoint_destroy": (None, [C.c_void_p]),
        "vf_adjoint_last_error": (C.c_char_p, [C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(lib, h, rc: int):
    if rc != VF_OK:
        msg = lib.vf_last_error(h)
        text = msg.decode() if msg else ""
        if rc == VF_EINVAL:
            from .api import ArgumentError
            raise ArgumentError(text)
        if rc == VF_ENOMEM:
            raise MemoryError(text)
        raise NativeError(rc, text)


def check_batch(lib, b, rc: int):
    if rc != VF_OK:
        msg = lib.vf_batch_last_error(b)
        text = msg.decode() if msg else ""
        if rc == VF_EINVAL:
            from .api import ArgumentError
            raise ArgumentError(text)
        if rc == VF_ENOMEM:
            raise MemoryError(text)
        raise NativeError(rc, text)


def check_server(lib, s, rc: int):
    if rc != VF_OK:
        msg = lib.vf_server_last_error(s)
        text = msg.decode() if msg else ""
        if rc == VF_EINVAL:
            from .api import ArgumentError
            raise ArgumentError(text)
        if rc == VF_ENOMEM:
            raise MemoryError(text)
        raise NativeError(rc, text)


def check_adjoint(lib, a, rc: int):
    if rc != VF_OK:
        msg = lib.vf_adjoint_last_error(a)
        text = msg.decode() if msg else ""
        if rc == VF_EINVAL:
            from .api import ArgumentError
            raise ArgumentError(text)
        if rc == VF_ENOMEM:
            raise MemoryError(text)
        raise NativeError(rc, text)


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)
