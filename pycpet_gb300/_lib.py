"""ctypes binding of libcpetgb.so (the C ABI in include/cpetgb.h).

The library is loaded from the package directory, where
``pycpet_gb300.build.build_library()`` puts it.  There is no fallback: if the
library is missing or no CUDA device is usable, calls raise ``CpetgbError``.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

OK = 0
EINVAL, ENOMEM, ECUDA, ETIMEOUT, ENODEV, ERANGE, EAGAIN = -1, -2, -3, -4, -5, -6, -7
FP64, FP32C = 0, 1
HOST, DEVICE = 0, 1
FIELD, ESP = 0, 1

_CODES = {EINVAL: "EINVAL", ENOMEM: "ENOMEM", ECUDA: "ECUDA", ETIMEOUT: "ETIMEOUT",
          ENODEV: "ENODEV", ERANGE: "ERANGE", EAGAIN: "EAGAIN"}

_lib = None
_path = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_f = ctypes.c_float
_sz = ctypes.c_size_t

# name -> argument types (all return int status)
SIGNATURES = {
    "cpetgb_version": [],
    "cpetgb_last_error": [ctypes.c_char_p, _sz],
    "cpetgb_device_sms": [],
    "cpetgb_synchronize": [_vp],
    "cpetgb_set_default_precision": [_i],
    "cpetgb_get_default_precision": [],
    "cpetgb_measure_peak": [_i, ctypes.POINTER(ctypes.c_double)],
    "cpetgb_compute_looped_field": [_i, _i, _vp, _vp, _vp, _vp],
    "cpetgb_calc_esp_base": [_vp, _vp, _i, _vp, _vp],
    "cpetgb_calc_field": [_vp, _vp, _i, _vp, _vp],
    "cpetgb_thread_operation": [_i, _i, _f, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_thread_operation_batch": [_i, _i, _vp, _f, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_thread_operation_dipole": [_i, _i, _f, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_compute_esp_grid": [_i, _i, _vp, _vp, _vp, _vp],
    "cpetgb_compute_looped_field_p": [_i, _i, _i, _vp, _vp, _vp, _vp],
    "cpetgb_calc_esp_base_p": [_i, _vp, _vp, _i, _vp, _vp],
    "cpetgb_calc_field_p": [_i, _vp, _vp, _i, _vp, _vp],
    "cpetgb_thread_operation_p": [_i, _i, _i, _f, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_thread_operation_batch_p": [_i, _i, _i, _vp, _f, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_thread_operation_dipole_p": [_i, _i, _i, _f, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_compute_esp_grid_p": [_i, _i, _i, _vp, _vp, _vp, _vp],
    "cpetgb_set_field_refinement": [_d],
    "cpetgb_check_wait_limit": [_d],
    "cpetgb_field_grid": [_i, _i, _i, _i, _vp, _vp, _vp, _i, _vp, _vp],
    "cpetgb_esp_grid": [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_grid_batch": [_i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_topo_lines": [_i, _i, _i, _i, _vp, _vp, _d, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_topo_batch": [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_topo_dipole_lines": [_i, _i, _i, _i, _vp, _vp, _d, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_tune_key": [_i, _i, _i, _d],
    "cpetgb_tune_variants": [_i],
    "cpetgb_tune_set": [_i, _i],
    "cpetgb_tune_get": [_i],
    "cpetgb_topo_resident_limit": [_i, _i],
    "cpetgb_grid_plan_create": [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_topo_plan_create": [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_plan_launch": [_vp, _vp],
    "cpetgb_plan_destroy": [_vp],
    "cpetgb_engine_create": [_vp, _i, ctypes.c_int64, ctypes.c_int64, _i, _i, _i],
    "cpetgb_engine_destroy": [_vp],
    "cpetgb_engine_add_frame": [_vp, _i, _vp, _vp, _vp],
    "cpetgb_engine_remove_frame": [_vp, _i],
    "cpetgb_engine_submit": [_vp, _i, _i, _vp, _vp, _d, _vp, _vp],
    "cpetgb_engine_poll": [_vp, _i],
    "cpetgb_engine_collect": [_vp, _i, _vp, _vp],
    "cpetgb_engine_drain": [_vp],
    "cpetgb_engine_set_ctas_per_sm": [_vp, _i],
    "cpetgb_topo_lines_noalloc": [_i, _i, _i, _vp, _vp, _d, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_topo_hist2d": [_i, _i, _vp, _i, _i, _vp, _vp, _vp, _vp],
    "cpetgb_prepare_frame": [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _d, _vp, _vp, _vp, _vp, _vp, _vp],
    "cpetgb_format_fixed3": [_i, ctypes.c_int64, _i, _vp, _vp, ctypes.c_int64, _vp, _vp],
    "cpetgb_format_sci18": [_i, ctypes.c_int64, _i, _vp, _vp, ctypes.c_int64, _vp, _vp],
    "cpetgb_topo_hist2d_sets": [_i, _i, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp],
    "cpetgb_chi2_distance_matrix": [_i, _i, _i, _i, _vp, _vp, _vp],
    "cpetgb_field_distance_matrix": [_i, _i, _i, _i, _vp, _vp, _vp],
}


class CpetgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cpetgb error {_CODES.get(code, code)}: {msg}")
        self.code = code


def lib(path: str | None = None):
    """Load (once) and return the ctypes handle of libcpetgb.so."""
    global _lib, _path
    if _lib is not None and (path is None or path == _path):
        return _lib
    so = path or LIB
    if not os.path.exists(so):
        raise CpetgbError(ENODEV, f"{so} is not built (run pycpet_gb300.build.build_library())")
    L = ctypes.CDLL(so)
    for name, argtypes in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int
    L.cpetgb_field_refinement.argtypes = []
    L.cpetgb_field_refinement.restype = ctypes.c_double
    _lib, _path = L, so
    _load_tuned_table()
    return L


def _load_tuned_table():
    """Loads the autotuner table for this GPU (the user's cache, else the one
    shipped for the model), when a CUDA device is visible."""
    try:
        import torch

        if not torch.cuda.is_available():
            return
        from . import autotune

        autotune.load_default()
    except Exception:  # a missing or unreadable table only means default shapes
        pass


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().cpetgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != OK:
        raise CpetgbError(rc, last_error())


def measure_peak(kind: int) -> float:
    """Measured throughput: 0 FFMA flop/s, 1 DFMA flop/s, 2 MUFU op/s, 3 FFMA2 flop/s,
    4 pair evaluations/s of the FP32C streamline sweep's inner loop alone."""
    v = ctypes.c_double(0.0)
    check(lib().cpetgb_measure_peak(kind, ctypes.byref(v)))
    return v.value


def set_field_refinement(tau: float) -> float:
    """Sets the FP32C field refinement threshold (0 = off) and returns the old one."""
    old = lib().cpetgb_field_refinement()
    check(lib().cpetgb_set_field_refinement(float(tau)))
    return old


def device_sms() -> int:
    rc = lib().cpetgb_device_sms()
    if rc < 0:
        check(rc)
    return rc
