"""CPU oracle of the GB300 Coulomb library.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py may
import this module.  It loads ``liboracle.so`` (built from oracle.c and
oracle_ref32.c by oracle/Makefile) and exposes numpy-level wrappers:

* ``field_grid_f64`` / ``esp_grid_f64`` / ``topo_lines_f64``: the FP64
  precision oracle of compute_looped_field (CPET/utils/math_module.c:405-451),
  calc_esp_base (math_module.c:453-486) and thread_operation
  (math_module.c:523-591).
* ``*_f32``: the same algorithms in the reference's float arithmetic, used as
  the timed CPU baseline ("port").
* ``histogram2d``: numpy's own histogram2d, the function the reference calls in
  make_histograms (CPET/utils/calculator.py:702-707).
* ``topo_lines_dipole``: thread_operation_dipole (math_module.c:593-659),
  FP64 or the reference's float arithmetic.
* ``chi2_matrix_f64`` / ``field_matrix_f64``: the clustering distance matrices
  construct_distance_matrix (calculator.py:975-978, 1003-1015) and
  construct_distance_matrix_volume (calculator.py:1042-1058) in IEEE double.
* ``load_reference()``: the reference's own math_module.c compiled from source
  into oracle/_ref (present only where the reference checkout exists).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C")
_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C")
_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C")
_c_int = ctypes.c_int


def build(force: bool = False) -> str:
    """Compile liboracle.so (and oracle/_ref when the reference source exists)."""
    so = os.path.join(HERE, "liboracle.so")
    if force or not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        so = build()
        L = ctypes.CDLL(so)
        L.oracle_field_grid_f64_mt.argtypes = [_c_int, _c_int, _d, _d, _d, _d, _c_int, _c_int]
        L.oracle_esp_grid_f64_mt.argtypes = [_c_int, _c_int, _d, _d, _d, _d, _c_int]
        L.oracle_field_grid_f32_mt.argtypes = [_c_int, _c_int, _f, _f, _f, _f, _c_int]
        L.oracle_esp_grid_f32_mt.argtypes = [_c_int, _c_int, _f, _f, _f, _f, _c_int]
        L.oracle_point_field_f32.argtypes = [_c_int, _c_int, _f, _f, _f, _f]
        L.oracle_topo_lines_f64_mt.argtypes = [
            _c_int, _c_int, _i, ctypes.c_double, _d, _d, _d, _d, _d, _d, _i, _c_int]
        L.oracle_topo_lines_f32_mt.argtypes = [
            _c_int, _c_int, _i, ctypes.c_float, _f, _f, _f, _f, _f, _f, _i, _c_int]
        L.oracle_chi2_matrix_f64.argtypes = [_c_int, _c_int, _d, _d, _c_int]
        L.oracle_field_matrix_f64.argtypes = [_c_int, _c_int, _d, _d, _c_int]
        _v = ctypes.c_void_p
        L.oracle_topo_lines_dipole_mt.argtypes = [_c_int, _c_int, _c_int, _i, ctypes.c_double, _v, _v, _v, _v,
                                                  _v, _v, _i, _c_int]
        _LIB = L
    return _LIB


def _threads(n):
    return int(n) if n else (os.cpu_count() or 1)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def field_grid_f64(pts, x, q, clamp=True, threads=None):
    pts, x, q = _c(pts, np.float64).reshape(-1, 3), _c(x, np.float64).reshape(-1, 3), _c(q, np.float64).reshape(-1)
    E = np.empty_like(pts)
    lib().oracle_field_grid_f64_mt(len(pts), len(q), pts, x, q, E, int(bool(clamp)), _threads(threads))
    return E


def esp_grid_f64(pts, x, q, threads=None):
    pts, x, q = _c(pts, np.float64).reshape(-1, 3), _c(x, np.float64).reshape(-1, 3), _c(q, np.float64).reshape(-1)
    phi = np.empty(len(pts))
    lib().oracle_esp_grid_f64_mt(len(pts), len(q), pts, x, q, phi, _threads(threads))
    return phi


def field_grid_f32(pts, x, q, threads=None):
    pts, x, q = _c(pts, np.float32).reshape(-1, 3), _c(x, np.float32).reshape(-1, 3), _c(q, np.float32).reshape(-1)
    E = np.empty_like(pts)
    lib().oracle_field_grid_f32_mt(len(pts), len(q), pts, x, q, E, _threads(threads))
    return E


def esp_grid_f32(pts, x, q, threads=None):
    pts, x, q = _c(pts, np.float32).reshape(-1, 3), _c(x, np.float32).reshape(-1, 3), _c(q, np.float32).reshape(-1)
    phi = np.empty(len(pts), dtype=np.float32)
    lib().oracle_esp_grid_f32_mt(len(pts), len(q), pts, x, q, phi, _threads(threads))
    return phi


def point_field_f32(pts, x, q):
    pts, x, q = _c(pts, np.float32).reshape(-1, 3), _c(x, np.float32).reshape(-1, 3), _c(q, np.float32).reshape(-1)
    E = np.empty_like(pts)
    lib().oracle_point_field_f32(len(pts), len(q), pts, x, q, E)
    return E


def topo_lines_f64(x0, n_iter, x, q, step, dims, threads=None):
    """Returns (ret (L,2) = [dist, curv], ends (L,3), steps (L,))."""
    x0 = _c(x0, np.float64).reshape(-1, 3)
    n_iter = _c(np.broadcast_to(np.asarray(n_iter), (len(x0),)), np.int32)
    x, q = _c(x, np.float64).reshape(-1, 3), _c(q, np.float64).reshape(-1)
    dims = _c(dims, np.float64).reshape(3)
    ret = np.empty((len(x0), 2))
    ends = np.empty((len(x0), 3))
    steps = np.empty(len(x0), dtype=np.int32)
    lib().oracle_topo_lines_f64_mt(len(x0), len(q), n_iter, float(step), x0, dims, x, q, ret, ends, steps,
                                   _threads(threads))
    return ret, ends, steps


def topo_lines_f32(x0, n_iter, x, q, step, dims, threads=None):
    x0 = _c(x0, np.float32).reshape(-1, 3)
    n_iter = _c(np.broadcast_to(np.asarray(n_iter), (len(x0),)), np.int32)
    x, q = _c(x, np.float32).reshape(-1, 3), _c(q, np.float32).reshape(-1)
    dims = _c(dims, np.float32).reshape(3)
    ret = np.empty((len(x0), 2), dtype=np.float32)
    ends = np.empty((len(x0), 3), dtype=np.float32)
    steps = np.empty(len(x0), dtype=np.int32)
    lib().oracle_topo_lines_f32_mt(len(x0), len(q), n_iter, np.float32(step), x0, dims, x, q, ret, ends, steps,
                                   _threads(threads))
    return ret, ends, steps


def histogram2d(dist, curv, bins, rng):
    """The reference's binning call (CPET/utils/calculator.py:702-707): numpy's histogram2d."""
    h, _, _ = np.histogram2d(np.asarray(dist, np.float64), np.asarray(curv, np.float64), bins=bins, range=rng)
    return h


def chi2_matrix_f64(hists, threads=None):
    """construct_distance_matrix / distance_numpy (CPET/utils/calculator.py:975-978,
    1003-1015) in IEEE double: (F, B) histograms -> (F, F)."""
    h = _c(hists, np.float64)
    n = h.shape[0]
    out = np.empty((n, n))
    if n:
        lib().oracle_chi2_matrix_f64(n, h.shape[1], h.reshape(n, -1), out, _threads(threads))
    return out


def field_matrix_f64(fields, threads=None):
    """construct_distance_matrix_volume (CPET/utils/calculator.py:1042-1058) in
    IEEE double: (F, P, 3) fields -> (F, F)."""
    f = _c(fields, np.float64)
    n = f.shape[0]
    out = np.empty((n, n))
    if n:
        lib().oracle_field_matrix_f64(n, f.shape[1], f.reshape(n, -1), out, _threads(threads))
    return out


def topo_lines_dipole(x0, n_iter, x, mu, step, dims, f32=False, threads=None):
    """thread_operation_dipole (CPET/utils/math_module.c:593-659) for every start
    point: FP64 (f32=False) or the reference's float arithmetic (f32=True).
    Returns (ret (L,2) = [dist, curv], ends (L,3), steps (L,))."""
    dt = np.float32 if f32 else np.float64
    x0 = _c(x0, dt).reshape(-1, 3)
    L = len(x0)
    n_iter = _c(np.broadcast_to(np.asarray(n_iter), (L,)), np.int32)
    x, mu, dims = _c(x, dt).reshape(-1, 3), _c(mu, dt).reshape(-1, 3), _c(dims, dt).reshape(3)
    ret, ends = np.empty((L, 2), dtype=dt), np.empty((L, 3), dtype=dt)
    steps = np.empty(L, dtype=np.int32)
    p = lambda a: a.ctypes.data
    lib().oracle_topo_lines_dipole_mt(int(f32), L, len(mu), n_iter, float(np.float32(step) if f32 else step),
                                      p(x0), p(dims), p(x), p(mu), p(ret), p(ends), steps, _threads(threads))
    return ret, ends, steps


def load_reference():
    """The reference's own C library built from source into oracle/_ref, or None."""
    so = os.path.join(HERE, "_ref", "math_module.so")
    if not os.path.exists(so):
        return None
    L = ctypes.CDLL(so)
    f1 = np.ctypeslib.ndpointer(dtype=np.float32, ndim=1, flags="C")
    f2 = np.ctypeslib.ndpointer(dtype=np.float32, ndim=2, flags="C")
    # argument lists as declared by the reference's FFI (CPET/utils/c_ops.py:85-159)
    L.compute_looped_field.argtypes = [_c_int, _c_int, f2, f2, f1, f2]
    L.compute_looped_field.restype = None
    L.calc_esp_base.argtypes = [f1, f1, _c_int, f2, f1]
    L.calc_esp_base.restype = None
    L.calc_field.argtypes = [f1, f1, _c_int, f2, f1]
    L.calc_field.restype = None
    L.thread_operation.argtypes = [_c_int, _c_int, ctypes.c_float, f1, f1, f2, f1, f1]
    L.thread_operation.restype = None
    L.thread_operation_dipole.argtypes = [_c_int, _c_int, ctypes.c_float, f1, f1, f2, f2, f1]
    L.thread_operation_dipole.restype = None
    return L
