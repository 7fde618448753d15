"""GPU-backed mirror of the hot-path functions of ``CPET.utils.calculator``
(CPET/utils/calculator.py).  Same names, arguments and return arrays; the
Coulomb arithmetic runs in libcpetgb.so.

Box/grid construction (host, numpy) is restated so the coordinates are the
reference's own:
  initialize_box_points_random   CPET/utils/calculator.py:123-168
  initialize_box_points_uniform  CPET/utils/calculator.py:171-248
Math wrappers (GPU):
  compute_field_on_grid                      calculator.py:430-447  -> (P,6) float32
  compute_ESP_on_grid                        calculator.py:450-475  -> (P,4) float16
  calculate_electric_field_c_shared_full_alt calculator.py:296-310  -> (3,) float32
  calculate_esp_c_shared_full                calculator.py:330-341  -> (1,) float32
  calculate_thread_c_shared                  calculator.py:344-348  -> (2,) float32
  calculate_thread_c_shared_dipole           calculator.py:351-358  -> (2,) float32
Streamline post-processing and histograms:
  curv / compute_curv_and_dist               calculator.py:501-561  (numpy, host)
  make_histograms                            calculator.py:596-718  (GPU binning, one launch)
Output (GPU text formatting):
  save_numpy_as_dat                          CPET/utils/io.py:50-109
  savetxt (the .top writer)                  numpy.savetxt as called at CPET/source/CPET.py:123
Clustering front end (GPU distance matrices):
  distance_numpy                             calculator.py:975-978  (numpy, per pair)
  construct_distance_matrix                  calculator.py:1003-1015
  make_fields                                calculator.py:846-857  (host parser)
  construct_distance_matrix_volume           calculator.py:1042-1058
"""
from __future__ import annotations

import logging
import warnings

import numpy as np

from . import _lib
from .c_ops import Math_ops
from .core import chi2_distance_matrix, field_distance_matrix, format_fixed3, format_sci18, topo_hist2d_sets

log = logging.getLogger(__name__)

_MATH = None


def math_ops() -> Math_ops:
    global _MATH
    if _MATH is None:
        _MATH = Math_ops()
    return _MATH


def box_transformation(center, x, y):
    """Orthonormal box basis as rows (x_hat, y_hat, z_hat): x_hat along x-center,
    z_hat = x_hat cross y_hat, y_hat = z_hat cross x_hat
    (CPET/utils/calculator.py:200-215)."""
    x = np.asarray(x, dtype=np.float64) - np.asarray(center, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64) - np.asarray(center, dtype=np.float64)
    x_unit = x / np.linalg.norm(x)
    y_unit = y / np.linalg.norm(y)
    z_unit = np.cross(x_unit, y_unit)
    z_unit = z_unit / np.linalg.norm(z_unit)
    y_unit = np.cross(z_unit, x_unit)
    y_unit = y_unit / np.linalg.norm(y_unit)
    return np.column_stack([x_unit, y_unit, z_unit]).T


def initialize_box_points_random(center, x, y, dimensions, n_samples, max_steps=10, dtype="float32"):
    """Random start points in the box and per-line step caps (same RNG calls
    and order as the reference, so a seeded numpy global state gives the
    same points and caps)."""
    half_length, half_width, half_height = dimensions
    transformation_matrix = box_transformation(center, x, y)
    random_x = np.random.uniform(-half_length, half_length, n_samples)
    random_y = np.random.uniform(-half_width, half_width, n_samples)
    random_z = np.random.uniform(-half_height, half_height, n_samples)
    random_points_local = np.column_stack([random_x, random_y, random_z])
    if dtype == "float32":
        random_points_local = random_points_local.astype(np.float32)
    random_max_samples = np.random.randint(1, max_steps, n_samples)
    return random_points_local, random_max_samples, transformation_matrix, max_steps


def initialize_box_points_uniform(center, x, y, N_cr, dimensions, dtype="float32", max_steps=10,
                                  ret_rand_max=False, inclusive=True, seed=None):
    """Uniform ij-indexed mesh: linspace(-d, d, N_cr+1) per axis, faces
    included (volume grids) or excluded (streamline starts)."""
    half_length, half_width, half_height = dimensions
    transformation_matrix = box_transformation(center, x, y)
    if inclusive:
        xs = np.linspace(-half_length, half_length, N_cr[0] + 1)
        ys = np.linspace(-half_width, half_width, N_cr[1] + 1)
        zs = np.linspace(-half_height, half_height, N_cr[2] + 1)
    else:
        xs = np.linspace(-half_length, half_length, N_cr[0] + 1, endpoint=False)[1:]
        ys = np.linspace(-half_width, half_width, N_cr[1] + 1, endpoint=False)[1:]
        zs = np.linspace(-half_height, half_height, N_cr[2] + 1, endpoint=False)[1:]
    xm, ym, zm = np.meshgrid(xs, ys, zs, indexing="ij")
    local_coords = np.stack([xm, ym, zm], axis=-1, dtype=dtype)
    if seed is not None:
        np.random.seed(seed)
    if ret_rand_max:
        n_samples = local_coords.shape[0] * local_coords.shape[1] * local_coords.shape[2]
        random_max_samples = np.random.randint(1, max_steps, n_samples)
        return local_coords, random_max_samples, transformation_matrix
    return local_coords, transformation_matrix


def volume_grid_counts(dimensions, step_size):
    """N_cr = int(2 * d / step) per axis, truncated as in
    CPET/source/calculator.py:258-259."""
    n = 2 * np.asarray(dimensions) / step_size
    return [int(n[0]), int(n[1]), int(n[2])]


def calculate_electric_field_c_shared_full_alt(x_0, x, Q):
    x_0 = x_0.astype(np.float32)
    x = x.astype(np.float32)
    Q = Q.astype(np.float32)
    return math_ops().calc_field(x_0=np.ascontiguousarray(x_0.reshape(3)), x=np.ascontiguousarray(x.reshape(-1, 3)),
                                 Q=np.ascontiguousarray(Q.reshape(-1)))


def calculate_esp_c_shared_full(x_0, x, Q):
    return math_ops().calc_esp_base(x_0=x_0, x=x, Q=Q)


def calculate_thread_c_shared(x_0, n_iter, x, Q, step_size, dimensions):
    return math_ops().thread_operation(x_0=x_0, n_iter=n_iter, x=x, Q=Q, step_size=step_size,
                                       dimensions=dimensions)


def calculate_thread_c_shared_dipole(x_0, n_iter, x, mu, step_size, dimensions):
    """One dipole streamline (CPET/utils/calculator.py:351-358)."""
    return math_ops().thread_operation_dipole(x_0=x_0, n_iter=n_iter, x=x, mu=mu, step_size=step_size,
                                              dimensions=dimensions)


def compute_field_on_grid(grid_coords, x, Q):
    """(M,M,M,3) mesh -> (P,6) float32 [x, y, z, Ex, Ey, Ez]."""
    x_0 = grid_coords.reshape(-1, 3)
    E = math_ops().compute_looped_field(x_0, x, Q)
    return np.concatenate((x_0, E), axis=1)


def compute_ESP_on_grid(grid_coords, x, Q):
    """(M,M,M,3) mesh -> (P,4) float16 [x, y, z, phi], one GPU launch for all
    points (the reference loops over points in Python)."""
    reshaped = grid_coords.reshape(-1, 3)
    esp = math_ops().compute_esp_grid(reshaped, x, Q).astype(float).reshape(-1, 1)
    return np.concatenate((reshaped, esp), axis=1).astype(np.half)


def curv(v_prime, v_prime_prime, eps=10e-6):
    denominator = np.linalg.norm(v_prime, axis=0) ** 3
    curvature = np.linalg.norm(np.cross(v_prime, v_prime_prime), axis=0)
    if denominator == 0:
        return curvature / eps
    return curvature / denominator


def compute_curv_and_dist(x_init, x_init_plus, x_init_plus_plus, x_0, x_0_plus, x_0_plus_plus):
    curv_init = curv(x_init_plus - x_init, x_init_plus_plus - 2 * x_init_plus + x_init)
    curv_final = curv(x_0_plus - x_0, x_0_plus_plus - 2 * x_0_plus + x_0)
    curv_mean = (curv_init + curv_final) / 2
    dist = np.linalg.norm(x_init - x_0, axis=-1)
    return [dist, curv_mean]


def _read_top(path):
    d, c = [], []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                continue
            parts = line.split()
            d.append(float(parts[0]))
            c.append(float(parts[1]))
    return np.asarray(d), np.asarray(c)


def histogram_bins(dist_list, curv_list, len_dist_curv):
    """Freedman-Diaconis bin counts and ranges of make_histograms
    (CPET/utils/calculator.py:664-685)."""
    from scipy.stats import iqr

    dmax, cmax = np.max(dist_list), np.max(curv_list)
    dmin, cmin = np.min(dist_list), np.min(curv_list)
    d_res = 2 * iqr(dist_list) / (len_dist_curv ** (1 / 3))
    c_res = 2 * iqr(curv_list) / (len_dist_curv ** (1 / 3))
    nd = int((dmax - dmin) / d_res)
    nc = int((cmax - cmin) / c_res)
    return (nd, nc), ((dmin, dmax), (cmin, cmax))


def make_histograms(topo_files, plot=False):
    """Normalised, flattened 2-D (distance, curvature) histograms of .top
    files, binned on the GPU with numpy.histogram2d's rules."""
    data = [_read_top(f) for f in topo_files]
    lens = np.array([len(d) for d, _ in data], dtype=int)
    if lens.size and not np.all(lens == lens[0]):
        warnings.warn(f"Topologies provided are of different sizes, using the mean value of {np.mean(lens)} "
                      f"to represent binning for {lens}")
        n_ref = np.mean(lens)
    else:
        n_ref = lens[0] if lens.size else 0
    dist_all = np.concatenate([d for d, _ in data])
    curv_all = np.concatenate([c for _, c in data])
    bins, rng = histogram_bins(dist_all, curv_all, n_ref)
    offsets = np.concatenate([[0], np.cumsum(lens)])
    # every file's histogram in one launch, each divided by its own total
    return topo_hist2d_sets(np.column_stack([dist_all, curv_all]), offsets, bins, rng, normalize=True)


def distance_numpy(hist1, hist2):
    """Chi-square distance of two histograms (CPET/utils/calculator.py:975-978),
    numpy on the host: the per-pair metric; whole matrices go to the GPU
    through construct_distance_matrix."""
    a = (hist1 - hist2) ** 2
    b = hist1 + hist2
    return np.sum(np.divide(a, b, out=np.zeros_like(a), where=b != 0)) / 2.0


def construct_distance_matrix(histograms, precision=None):
    """All-pairs distance_numpy matrix of the rows of `histograms`
    (CPET/utils/calculator.py:1003-1015), one GPU launch; zero diagonal.
    precision: "fp64" (IEEE double) or "fp32c" (FP32 terms, compensated sums);
    default: the library's default precision."""
    return chi2_distance_matrix(np.asarray(histograms, np.float64), _precision(precision))


def make_fields(field_files):
    """The (Ex, Ey, Ez) columns of volume .dat files, one (P,3) array per file
    (CPET/utils/calculator.py:846-857)."""
    fields = []
    for field_file in field_files:
        rows = []
        with open(field_file) as fh:
            for line in fh:
                if line.startswith("#"):
                    continue
                parts = line.split()
                rows.append([float(parts[3]), float(parts[4]), float(parts[5])])
        fields.append(np.array(rows))
    return fields


def construct_distance_matrix_volume(fields, precision=None):
    """Matrix of sum_p |f_i[p] - f_j[p]| over a common grid
    (CPET/utils/calculator.py:1042-1058), one GPU launch; zero diagonal."""
    return field_distance_matrix(np.stack([np.asarray(f, np.float64).reshape(-1, 3) for f in fields]),
                                 _precision(precision))


def save_numpy_as_dat(meta_data, volume, name):
    """Volume output file of CPET/utils/io.py:50-109: the same seven header
    lines, then the rows of `volume` as numpy.savetxt(fmt="%.3f") writes them,
    formatted on the GPU for float32 / float16 volumes (the arrays
    compute_box and compute_box_ESP return); other dtypes go through
    numpy.savetxt itself, as the reference does."""
    dimensions = meta_data["dimensions"]
    num_steps_list = meta_data["num_steps"]
    trans_mat = meta_data["transformation_matrix"].transpose()
    center = meta_data["center"]
    header = "#Sample Density: {} {} {}; Volume: Box: {} {} {}\n".format(
        num_steps_list[0], num_steps_list[1], num_steps_list[2], dimensions[0], dimensions[1], dimensions[2])
    header += "#Frame 0\n"
    header += "#Center: {} {} {}\n".format(center[0], center[1], center[2])
    header += "#Basis Matrix:\n# {} {} {}\n# {} {} {}\n# {} {} {}\n".format(
        trans_mat[0][0], trans_mat[0][1], trans_mat[0][2], trans_mat[1][0], trans_mat[1][1], trans_mat[1][2],
        trans_mat[2][0], trans_mat[2][1], trans_mat[2][2])
    volume = np.asarray(volume)
    if volume.dtype in (np.float32, np.float16) and volume.ndim in (1, 2):
        body = format_fixed3(volume)
    else:
        import io

        sink = io.BytesIO()
        np.savetxt(sink, volume, fmt="%.3f")
        body = sink.getvalue()
    with open(name, "wb") as fh:
        fh.write(header.encode())
        fh.write(body)


def savetxt(fname, X, *args, **kwargs):
    """numpy.savetxt, with the default call numpy.savetxt(fname, X) -- how the
    topology dispatcher writes every .top file (CPET/source/CPET.py:123) --
    formatted on the GPU for float32 matrices (the (L,2) streamline results):
    the same bytes, "%.18e" values joined by spaces, one row per line.  Any
    other dtype or argument goes to numpy.savetxt itself."""
    a = np.asarray(X)
    if args or kwargs or a.dtype != np.float32 or a.ndim not in (1, 2):
        return np.savetxt(fname, X, *args, **kwargs)
    body = format_sci18(a.reshape(-1, 1) if a.ndim == 1 else a)
    if hasattr(fname, "write"):
        try:
            fname.write(body)
        except TypeError:
            fname.write(body.decode("latin-1"))
        return None
    with open(fname, "wb") as fh:
        fh.write(body)
    return None


def _precision(p):
    if p is not None:
        return p
    return "fp64" if _lib.lib().cpetgb_get_default_precision() == _lib.FP64 else "fp32c"
