"""pycpet_gb300 -- GB300 (sm_103a) implementation of PyCPET's Coulomb hot path.

Kernels live in libcpetgb.so (pycpet_gb300/csrc, C ABI in include/cpetgb.h);
this package is the host side: ctypes binding (``_lib``), array-level API
(``core``), and drop-ins for PyCPET's ``c_ops.Math_ops`` (``c_ops``), the
math functions of ``CPET.utils.calculator`` (``calculator``) and the
calculator hot-path methods (``drop_in``).
"""
from ._lib import CpetgbError, set_field_refinement  # noqa: F401
from .core import (GridBatch, TopoBatch, chi2_distance_matrix, esp_grid, field_distance_matrix,  # noqa: F401
                   field_grid, point_field, synchronize, topo_dipole_lines, topo_hist2d, topo_hist2d_sets,
                   topo_lines)

__version__ = "1.0.0"
