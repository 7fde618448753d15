"""Drop-in for PyCPET's ctypes wrapper ``CPET.utils.c_ops.Math_ops``
(CPET/utils/c_ops.py:7-375), backed by libcpetgb.so on the GPU.

Method names, argument order and meaning, return shapes and dtypes follow the
reference wrapper for the hot-path functions:

  compute_looped_field (c_ops.py:250-263)  -> (P,3) float32, r^2 clamped at 1e-6
  calc_esp_base        (c_ops.py:326-341)  -> (1,) float32
  calc_field_base      (c_ops.py:343-358)  -> (3,) float32
  calc_field           (c_ops.py:360-375)  -> (3,) float32
  thread_operation     (c_ops.py:281-302)  -> (2,) float32 [distance, curvature]

plus two batched calls the reference lacks (one launch instead of a Python or
Pool loop): ``thread_operation_batch`` and ``compute_esp_grid``.

Error behaviour mirrors the reference: the methods that convert their inputs
with ``np.array(..., dtype="float32")`` in the reference convert here too;
the ones that pass arrays straight to ctypes ``ndpointer(float32, C)``
arguments raise ``ctypes.ArgumentError`` on other dtypes here too.  Library
failures raise ``pycpet_gb300.CpetgbError``; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np
import numpy.ctypeslib as npct

from . import _lib
from .core import precision_code

_f1 = npct.ndpointer(dtype=np.float32, ndim=1, flags="C")
_f2 = npct.ndpointer(dtype=np.float32, ndim=2, flags="C")
_i1 = npct.ndpointer(dtype=np.int32, ndim=1, flags="C")


class Math_ops:
    """``precision`` (``"fp32c"`` / ``"fp64"``, default: the library default)
    travels with every call (the ``*_p`` entry points), so objects of different
    precisions can be used from several threads at once."""

    def __init__(self, shared_loc=None, precision=None):
        # shared_loc names the GPU library (default: the in-tree libcpetgb.so)
        self.math = _lib.lib(shared_loc)
        self.precision = None if precision is None else precision_code(precision)
        # typed views with the reference's ndpointer checks (c_ops.py:85-138)
        L = ctypes.CDLL(self.math._name)
        _c = ctypes.c_int

        def typed(name, argtypes):
            fn = getattr(L, name)
            fn.argtypes = [_c] + argtypes
            fn.restype = ctypes.c_int
            return fn

        self._thread_op = typed("cpetgb_thread_operation_p",
                                [_c, _c, ctypes.c_float, _f1, _f1, _f2, _f1, _f1])
        self._esp_base = typed("cpetgb_calc_esp_base_p", [_f1, _f1, _c, _f2, _f1])
        self._calc_field = typed("cpetgb_calc_field_p", [_f1, _f1, _c, _f2, _f1])
        self._thread_op_dipole = typed("cpetgb_thread_operation_dipole_p",
                                       [_c, _c, ctypes.c_float, _f1, _f1, _f2, _f2, _f1])

    def _prec(self) -> int:
        return self.math.cpetgb_get_default_precision() if self.precision is None else self.precision

    def _call(self, fn, *args):
        return _lib.check(fn(self._prec(), *args))

    def compute_looped_field(self, x_0, x, Q):
        res = np.zeros_like(x_0, dtype="float32")
        Q = Q.reshape(-1)
        x0 = np.ascontiguousarray(np.array(x_0, dtype="float32"))
        xx = np.ascontiguousarray(np.array(x, dtype="float32"))
        qq = np.ascontiguousarray(np.array(Q, dtype="float32"))
        res = np.ascontiguousarray(res)
        self._call(self.math.cpetgb_compute_looped_field_p, int(x0.shape[0]), len(qq),
                   x0.ctypes.data, xx.ctypes.data, qq.ctypes.data, res.ctypes.data)
        return res

    def compute_esp_grid(self, x_0, x, Q):
        x0 = np.ascontiguousarray(np.array(x_0, dtype="float32")).reshape(-1, 3)
        xx = np.ascontiguousarray(np.array(x, dtype="float32")).reshape(-1, 3)
        qq = np.ascontiguousarray(np.array(Q, dtype="float32")).reshape(-1)
        res = np.zeros(x0.shape[0], dtype="float32")
        self._call(self.math.cpetgb_compute_esp_grid_p, x0.shape[0], len(qq), x0.ctypes.data,
                   xx.ctypes.data, qq.ctypes.data, res.ctypes.data)
        return res

    def thread_operation(self, x_0, n_iter, x, Q, step_size, dimensions):
        res = np.zeros(2, dtype="float32")
        n_charges = len(Q)
        Q = Q.reshape(-1)
        self._call(self._thread_op, n_charges, int(n_iter), step_size, x_0, dimensions, x, Q, res)
        return res

    def thread_operation_dipole(self, x_0, n_iter, x, mu, step_size, dimensions):
        """One streamline through point dipoles (c_ops.py:304-325): res = (dist, curv)."""
        res = np.zeros(2, dtype="float32")
        self._call(self._thread_op_dipole, len(mu), int(n_iter), step_size, x_0, dimensions, x, mu, res)
        return res

    def thread_operation_batch(self, x_0, n_iter, x, Q, step_size, dimensions):
        x0 = np.ascontiguousarray(np.array(x_0, dtype="float32")).reshape(-1, 3)
        it = np.ascontiguousarray(np.broadcast_to(np.asarray(n_iter), (x0.shape[0],)), dtype=np.int32)
        xx = np.ascontiguousarray(np.array(x, dtype="float32")).reshape(-1, 3)
        qq = np.ascontiguousarray(np.array(Q, dtype="float32")).reshape(-1)
        dims = np.ascontiguousarray(np.array(dimensions, dtype="float32")).reshape(3)
        res = np.zeros((x0.shape[0], 2), dtype="float32")
        self._call(self.math.cpetgb_thread_operation_batch_p, x0.shape[0], len(qq), it.ctypes.data,
                   float(step_size), x0.ctypes.data, dims.ctypes.data, xx.ctypes.data, qq.ctypes.data,
                   res.ctypes.data)
        return res

    def calc_esp_base(self, x_0, x, Q):
        res = np.zeros(1, dtype="float32")
        self._call(self._esp_base, res, x_0, len(Q), x, Q.reshape(len(Q)))
        return res

    def calc_field_base(self, x_0, x, Q):
        res = np.zeros(3, dtype="float32")
        self._call(self._calc_field, res, x_0, len(Q), x, Q.reshape(len(Q)))
        return res

    def calc_field(self, x_0, x, Q):
        res = np.zeros(3, dtype="float32")
        self._call(self._calc_field, res, x_0, len(Q), x, Q.reshape(len(Q)))
        return res
