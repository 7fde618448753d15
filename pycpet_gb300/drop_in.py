"""Calculator-level drop-in for PyCPET's ``CPET.source.calculator.calculator``.

The hot-path methods the reference's dispatcher calls by name
(CPET/source/CPET.py:105-108, 149, 186, 208) are provided as plain functions
of ``self`` so they work both on ``Calculator`` below and, after
``patch_pycpet()``, on the reference class itself:

  compute_point_field             CPET/source/calculator.py:442-463  -> (3,) float32
  compute_box                     calculator.py:489-507  -> ((P,6) float32, mesh.shape)
  compute_box_ESP                 calculator.py:509-528  -> ((P,4) float16, mesh.shape)
  compute_topo_complete_c_shared  calculator.py:675-712  -> (L,2) float32, start order
  compute_topo_GPU_batch_filter   calculator.py:793-978  -> (L,2) float32, start order
                                  (the reference returns finish order; same rows)
  compute_topo_complete_c_shared_dipole  calculator.py:714-749  -> (L,2) float32
                                  (point dipoles self.x / self.mu)

Each reads ``self.x``, ``self.Q``, ``self.mesh``, ``self.random_start_points``,
``self.random_max_samples``, ``self.step_size`` and ``self.dimensions`` at call
time (scripts swap ``x``/``Q`` on live objects,
CPET/source/scripts/residue_breakdown_analysis.py:175-183).  The arithmetic
form comes from ``self.precision`` ("fp32c" default, or "fp64"), an additive
options key.
"""
from __future__ import annotations

import logging

import numpy as np

from .calculator import (box_transformation, initialize_box_points_random, initialize_box_points_uniform,
                         volume_grid_counts)
from .core import esp_grid, field_grid, prepare_frame, topo_dipole_lines, topo_lines

log = logging.getLogger(__name__)

HOT_METHODS = ("compute_point_field", "compute_box", "compute_box_ESP", "compute_topo_complete_c_shared",
               "compute_topo_GPU_batch_filter", "compute_topo_complete_c_shared_dipole")


def _prec(self):
    return getattr(self, "precision", None) or "fp32c"


def compute_point_field(self):
    """Field at the box centre (the origin of the rotated frame)."""
    E = field_grid(np.zeros((1, 3)), np.asarray(self.x, np.float64), np.asarray(self.Q, np.float64),
                   precision=_prec(self), clamp=False)
    return E[0].astype(np.float32)


def compute_box(self):
    x_0 = self.mesh.reshape(-1, 3)
    E = field_grid(x_0, np.asarray(self.x, np.float64), np.asarray(self.Q, np.float64),
                   precision=_prec(self), clamp=True)
    return np.concatenate((x_0, E.astype(np.float32)), axis=1), self.mesh.shape


def compute_box_ESP(self):
    x_0 = self.mesh.reshape(-1, 3)
    phi = esp_grid(x_0, np.asarray(self.x, np.float64), np.asarray(self.Q, np.float64), precision=_prec(self))
    return np.concatenate((x_0, phi.reshape(-1, 1)), axis=1).astype(np.half), self.mesh.shape


def _topo(self):
    starts = np.asarray(self.random_start_points, np.float64).reshape(-1, 3)
    caps = np.asarray(self.random_max_samples).reshape(-1).astype(np.int32)
    res = topo_lines(starts, caps, np.asarray(self.x, np.float64), np.asarray(self.Q, np.float64),
                     float(self.step_size), np.asarray(self.dimensions, np.float64), precision=_prec(self))
    self.hist = res.astype(np.float32)
    return self.hist


def compute_topo_complete_c_shared(self):
    return _topo(self)


def compute_topo_complete_c_shared_dipole(self):
    """Streamlines through point dipoles self.x / self.mu
    (CPET/source/calculator.py:714-749; used by
    CPET/source/scripts/field_topology_dipole.py:136-153)."""
    starts = np.asarray(self.random_start_points, np.float64).reshape(-1, 3)
    caps = np.asarray(self.random_max_samples).reshape(-1).astype(np.int32)
    res = topo_dipole_lines(starts, caps, np.asarray(self.x, np.float64), np.asarray(self.mu, np.float64),
                            float(self.step_size), np.asarray(self.dimensions, np.float64), precision=_prec(self))
    self.hist = res.astype(np.float32)
    return self.hist


def compute_topo_GPU_batch_filter(self):
    return _topo(self)


class _NumpyWithGpuSavetxt:
    """numpy as the dispatcher module sees it, with savetxt formatted on the GPU."""

    def __init__(self, savetxt):
        self.savetxt = savetxt

    def __getattr__(self, name):
        return getattr(np, name)


def patch_pycpet(precision: str = "fp32c", gpu_writers: bool = False):
    """Route an installed PyCPET's calculator hot-path methods to the GPU.

    Returns the patched class.  With ``gpu_writers`` the dispatcher's output
    writers run on the GPU too: save_numpy_as_dat (CPET/source/CPET.py:162,
    221) and the np.savetxt of .top files (CPET.py:123) in the module
    CPET.source.CPET, with byte-identical files.  Everything else of PyCPET
    (file parsing, filters, frames, clustering) is unchanged."""
    from CPET.source import calculator as ref

    cls = ref.calculator
    for name in HOT_METHODS:
        setattr(cls, name, globals()[name])
    cls.precision = precision
    if gpu_writers:
        from CPET.source import CPET as dispatcher

        from .calculator import save_numpy_as_dat, savetxt

        dispatcher.save_numpy_as_dat = save_numpy_as_dat
        dispatcher.np = _NumpyWithGpuSavetxt(savetxt)
    return cls


class Calculator:
    """The hot-path state of PyCPET's calculator built from arrays.

    ``options`` uses the reference keys (CPET_method, dimensions, step_size,
    n_samples, initializer, max_streamline_init, dtype, center / x / y given
    as coordinates, box_shift, filter_radius, filter_in_box) plus the
    additive ``precision``.  ``x`` and ``Q`` are the charges in the input
    frame; ``resid`` / ``resnum`` (per atom) are needed for filter_radius.
    The radius filter, the rotation into the box frame, the box filter and
    the shift run on the GPU (prepare_frame) with the reference's rules
    (CPET/source/calculator.py:239-251, 341-371).  Parsing and atom-spec
    filtering of PDB files stay PyCPET's job.
    """

    compute_point_field = compute_point_field
    compute_box = compute_box
    compute_box_ESP = compute_box_ESP
    compute_topo_complete_c_shared = compute_topo_complete_c_shared
    compute_topo_GPU_batch_filter = compute_topo_GPU_batch_filter
    compute_topo_complete_c_shared_dipole = compute_topo_complete_c_shared_dipole

    def __init__(self, options, x, Q, resid=None, resnum=None):
        opts = dict(options)
        self.precision = opts.get("precision", "fp32c")
        self.step_size = opts.get("step_size")
        self.dimensions = np.array(opts["dimensions"]) if opts.get("dimensions") is not None else None
        self.n_samples = opts.get("n_samples")
        self.dtype = opts.get("dtype", "float32")
        self.max_streamline_init = opts.get("max_streamline_init", "true_rand")
        self.box_shift = opts.get("box_shift", [0, 0, 0])
        method = opts["CPET_method"]
        self.center = np.asarray(opts.get("center", [0.0, 0.0, 0.0]), dtype=np.float64)
        x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
        self.Q = np.asarray(Q, dtype=np.float64).reshape(-1)
        has_axes = "x" in opts and "y" in opts
        if has_axes:
            self.x_vec_pt = np.asarray(opts["x"], dtype=np.float64)
            self.y_vec_pt = np.asarray(opts["y"], dtype=np.float64)
        if method in ("volume", "volume_ESP") and has_axes:
            N_cr = volume_grid_counts(self.dimensions, self.step_size)
            self.mesh, self.transformation_matrix = initialize_box_points_uniform(
                center=self.center, x=self.x_vec_pt, y=self.y_vec_pt, N_cr=N_cr, dimensions=self.dimensions,
                dtype=self.dtype, inclusive=True)
        elif method in ("topo", "topo_GPU") and has_axes:
            self.max_steps = round(2 * np.linalg.norm(self.dimensions) / self.step_size)
            if opts.get("initializer", "uniform") == "random":
                (self.random_start_points, self.random_max_samples, self.transformation_matrix,
                 self.max_streamline_len) = initialize_box_points_random(
                    self.center, self.x_vec_pt, self.y_vec_pt, self.dimensions, self.n_samples, dtype=self.dtype,
                    max_steps=self.max_steps)
            else:
                num_per_dim = round(self.n_samples ** (1 / 3))
                if num_per_dim ** 3 < self.n_samples:
                    num_per_dim += 1
                seed = 42 if self.max_streamline_init == "fixed_rand" else None
                (self.random_start_points, self.random_max_samples,
                 self.transformation_matrix) = initialize_box_points_uniform(
                    center=self.center, x=self.x_vec_pt, y=self.y_vec_pt, dimensions=self.dimensions,
                    N_cr=[num_per_dim] * 3, dtype=self.dtype, max_steps=self.max_steps, ret_rand_max=True,
                    inclusive=False, seed=seed)
                self.random_start_points = self.random_start_points.reshape(-1, 3)
                self.n_samples = len(self.random_start_points)
        elif has_axes:
            self.transformation_matrix = box_transformation(self.center, self.x_vec_pt, self.y_vec_pt)
        # residue radius filter, rotation, box filter and shift on the GPU
        # (CPET/source/calculator.py:239-251, 341-371)
        radius = float(opts["filter_radius"]) if "filter_radius" in opts else None
        box = self.dimensions if bool(opts.get("filter_in_box", False)) else None
        shift = self.box_shift if list(self.box_shift) != [0, 0, 0] else None
        inv = np.linalg.inv(self.transformation_matrix) if has_axes else None
        self.x, self.Q = prepare_frame(x, self.Q, self.center, inv_basis=inv, radius=radius, resid=resid,
                                       resnum=resnum, box_half=box, box_shift=shift)
        if self.dtype == "float32":
            self.x = self.x.astype(np.float32)
            self.Q = self.Q.astype(np.float32)
            self.center = self.center.astype(np.float32)
            if self.dimensions is not None:
                self.dimensions = self.dimensions.astype(np.float32)
