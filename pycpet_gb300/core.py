"""Array-level API over libcpetgb.so.

Every function accepts either numpy arrays (host memory: the library copies in,
computes on the GPU and copies out) or CUDA torch tensors (device memory: the
call is enqueued on the tensor's current stream and returns device tensors;
``synchronize()`` waits and raises device-side errors).  Torch is used only as
a device-buffer container; all arithmetic runs in the library's kernels.

Precision names: ``"fp64"`` (every operation in IEEE double, the plain form)
and ``"fp32c"`` (FP32 pair terms with Kahan-compensated accumulation across
charge tiles; FP64 streamline positions, curvature and distance).
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import DEVICE, ESP, FIELD, FP32C, FP64, HOST, check, lib

PRECISIONS = {"fp64": FP64, "fp32c": FP32C, FP64: FP64, FP32C: FP32C}


def precision_code(p) -> int:
    try:
        return PRECISIONS[p.lower() if isinstance(p, str) else p]
    except KeyError:
        raise ValueError(f"precision must be 'fp64' or 'fp32c', got {p!r}") from None


def _is_torch(a) -> bool:
    return type(a).__module__.split(".")[0] == "torch"


def _host(a, dtype, shape_tail=None):
    a = np.ascontiguousarray(a, dtype=dtype)
    if shape_tail is not None:
        a = a.reshape((-1,) + tuple(shape_tail))
    return a


def _dev(t, dtype, shape_tail=None):
    import torch

    if not (isinstance(t, torch.Tensor) and t.is_cuda):
        raise TypeError("device calls need CUDA torch tensors for every array argument")
    t = t.to(dtype).contiguous()
    if shape_tail is not None:
        t = t.reshape((-1,) + tuple(shape_tail))
    return t


def _stream_of(t):
    import torch

    return torch.cuda.current_stream(t.device).cuda_stream


def synchronize(stream=None) -> None:
    """Wait for `stream` (a torch stream, a raw handle or None for the current
    torch stream) and raise any device-side error recorded by the kernels."""
    if stream is None:
        try:
            import torch

            stream = torch.cuda.current_stream().cuda_stream if torch.cuda.is_available() else 0
        except ImportError:
            stream = 0
    elif hasattr(stream, "cuda_stream"):
        stream = stream.cuda_stream
    check(lib().cpetgb_synchronize(stream))


# ---------------------------------------------------------------------------
# Grids (K1 field, K2 potential)
# ---------------------------------------------------------------------------

def field_grid(points, x, q, precision="fp32c", clamp=True):
    """E[p] = k sum_j q_j (p - x_j) / |p - x_j|^3 at every point (P,3) -> (P,3) float64.

    clamp=True applies compute_looped_field's r^2 >= 1e-6 softening
    (CPET/utils/math_module.c:431-436); clamp=False is calc_field
    (math_module.c:255-293)."""
    prec = precision_code(precision)
    if _is_torch(points):
        import torch

        points, x, q = _dev(points, torch.float64, (3,)), _dev(x, torch.float64, (3,)), _dev(q, torch.float64)
        out = torch.empty((points.shape[0], 3), dtype=torch.float64, device=points.device)
        with torch.cuda.device(points.device):
            check(lib().cpetgb_field_grid(prec, DEVICE, points.shape[0], q.numel(), points.data_ptr(),
                                          x.data_ptr(), q.data_ptr(), int(bool(clamp)), out.data_ptr(),
                                          _stream_of(points)))
        return out
    points, x, q = _host(points, np.float64, (3,)), _host(x, np.float64, (3,)), _host(q, np.float64)
    out = np.empty((points.shape[0], 3))
    check(lib().cpetgb_field_grid(prec, HOST, points.shape[0], q.size, points.ctypes.data, x.ctypes.data,
                                  q.ctypes.data, int(bool(clamp)), out.ctypes.data, None))
    return out


def esp_grid(points, x, q, precision="fp32c"):
    """phi[p] = k sum_j q_j / |p - x_j| (calc_esp_base, math_module.c:453-486) -> (P,) float64."""
    prec = precision_code(precision)
    if _is_torch(points):
        import torch

        points, x, q = _dev(points, torch.float64, (3,)), _dev(x, torch.float64, (3,)), _dev(q, torch.float64)
        out = torch.empty((points.shape[0],), dtype=torch.float64, device=points.device)
        with torch.cuda.device(points.device):
            check(lib().cpetgb_esp_grid(prec, DEVICE, points.shape[0], q.numel(), points.data_ptr(),
                                        x.data_ptr(), q.data_ptr(), out.data_ptr(), _stream_of(points)))
        return out
    points, x, q = _host(points, np.float64, (3,)), _host(x, np.float64, (3,)), _host(q, np.float64)
    out = np.empty(points.shape[0])
    check(lib().cpetgb_esp_grid(prec, HOST, points.shape[0], q.size, points.ctypes.data, x.ctypes.data,
                                q.ctypes.data, out.ctypes.data, None))
    return out


def point_field(points, x, q, precision="fp32c"):
    """calc_field at one or more points (unsoftened field) -> (P,3) float64."""
    return field_grid(np.asarray(points, dtype=np.float64).reshape(-1, 3) if not _is_torch(points) else points,
                      x, q, precision=precision, clamp=False)


class GridBatch:
    """Many frames evaluated in one launch through a frame descriptor table.

    frames: sequence of (points (P_f,3), x (N_f,3), q (N_f,)).  The arrays are
    concatenated once; ``run()`` may then be called repeatedly (it reuses the
    concatenated inputs).  With ``device=True`` the inputs are uploaded once
    into torch CUDA tensors and ``run()`` stays on the device.
    """

    def __init__(self, frames, kind="field", precision="fp32c", clamp=True, device=False, graph=False):
        self.kind = FIELD if kind == "field" else ESP
        self.prec = precision_code(precision)
        self.clamp = int(bool(clamp))
        pts, xs, qs, desc = [], [], [], []
        po = co = 0
        for p, x, q in frames:
            p = np.asarray(p, np.float64).reshape(-1, 3)
            x = np.asarray(x, np.float64).reshape(-1, 3)
            q = np.asarray(q, np.float64).reshape(-1)
            desc.append((co, len(q), po, len(p)))
            pts.append(p), xs.append(x), qs.append(q)
            po += len(p)
            co += len(q)
        self.desc = np.ascontiguousarray(np.array(desc, dtype=np.int64).reshape(-1, 4))
        self.points = np.ascontiguousarray(np.concatenate(pts) if pts else np.zeros((0, 3)))
        self.x = np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros((0, 3)))
        self.q = np.ascontiguousarray(np.concatenate(qs) if qs else np.zeros(0))
        self.n_points = po
        self.n_charges = co
        self.nc = 3 if self.kind == FIELD else 1
        self.device = device
        if device:
            import torch

            self.points = torch.from_numpy(self.points).cuda()
            self.x = torch.from_numpy(self.x).cuda()
            self.q = torch.from_numpy(self.q).cuda()
            self.out = torch.empty((po, self.nc), dtype=torch.float64, device=self.points.device)
        self.plan = None
        if graph:
            if not device:
                raise ValueError("graph=True needs device=True (a plan binds device buffers)")
            self.plan = _Plan.grid(self.kind, self.prec, self.clamp, self.desc, self.points, self.x, self.q,
                                   self.out)

    @property
    def pair_evals(self) -> int:
        return int(np.sum(self.desc[:, 1] * self.desc[:, 3]))

    def run(self, out=None):
        if self.plan is not None and out is None:
            self.plan.launch(self.points)
            return self.out
        if self.device:
            out = self.out if out is None else out
            with __import__("torch").cuda.device(self.points.device):
                check(lib().cpetgb_grid_batch(self.kind, self.prec, DEVICE, self.clamp, len(self.desc),
                                              self.desc.ctypes.data, self.points.data_ptr(), self.x.data_ptr(),
                                              self.q.data_ptr(), out.data_ptr(), _stream_of(self.points)))
            return out
        out = np.empty((self.n_points, self.nc)) if out is None else out
        check(lib().cpetgb_grid_batch(self.kind, self.prec, HOST, self.clamp, len(self.desc), self.desc.ctypes.data,
                                      self.points.ctypes.data, self.x.ctypes.data, self.q.ctypes.data,
                                      out.ctypes.data, None))
        return out

    def split(self, out):
        """Per-frame views of a run() output."""
        return [out[po:po + P] for _, _, po, P in self.desc]


# ---------------------------------------------------------------------------
# Streamlines (K3) and histogram (K4)
# ---------------------------------------------------------------------------

def topo_lines(starts, n_iter, x, q, step, half_dims, precision="fp32c", return_ends=False,
               return_steps=False):
    """thread_operation (CPET/utils/math_module.c:523-591) for every start point.

    Returns result (L,2) = [distance, mean curvature] in start order, and
    optionally the end points (L,3) and the Euler step counts (L,)."""
    return _topo_lines(lib().cpetgb_topo_lines, 1, starts, n_iter, x, q, step, half_dims, precision, return_ends,
                       return_steps)


def topo_dipole_lines(starts, n_iter, x, mu, step, half_dims, precision="fp32c", return_ends=False,
                      return_steps=False):
    """thread_operation_dipole (CPET/utils/math_module.c:593-659) for every start
    point: streamlines through the field of point dipoles at x (N,3) with
    moments mu (N,3).  Outputs as topo_lines."""
    return _topo_lines(lib().cpetgb_topo_dipole_lines, 3, starts, n_iter, x, mu, step, half_dims, precision,
                       return_ends, return_steps)


def _topo_lines(fn, src_tail, starts, n_iter, x, q, step, half_dims, precision, return_ends, return_steps):
    prec = precision_code(precision)
    half = np.ascontiguousarray(np.asarray(half_dims, dtype=np.float64).reshape(3))
    if _is_torch(starts):
        import torch

        starts, x = _dev(starts, torch.float64, (3,)), _dev(x, torch.float64, (3,))
        q = _dev(q, torch.float64, (3,) if src_tail == 3 else ())
        if q.shape[0] != x.shape[0]:
            raise ValueError(f"{x.shape[0]} positions but {q.shape[0]} charges / moments")
        L = starts.shape[0]
        n_iter = _dev(n_iter if _is_torch(n_iter) else torch.as_tensor(np.broadcast_to(n_iter, (L,)).copy(),
                                                                       device=starts.device),
                      torch.int32)
        dev = starts.device
        res = torch.empty((L, 2), dtype=torch.float64, device=dev)
        ends = torch.empty((L, 3), dtype=torch.float64, device=dev) if return_ends else None
        steps = torch.empty((L,), dtype=torch.int32, device=dev) if return_steps else None
        with torch.cuda.device(dev):
            check(fn(prec, DEVICE, L, x.shape[0], starts.data_ptr(), n_iter.data_ptr(),
                     float(step), half.ctypes.data, x.data_ptr(), q.data_ptr(),
                     res.data_ptr(), ends.data_ptr() if ends is not None else None,
                     steps.data_ptr() if steps is not None else None, _stream_of(starts)))
    else:
        starts = _host(starts, np.float64, (3,))
        L = starts.shape[0]
        n_iter = np.ascontiguousarray(np.broadcast_to(np.asarray(n_iter), (L,)), dtype=np.int32)
        x, q = _host(x, np.float64, (3,)), _host(q, np.float64, (3,) if src_tail == 3 else None)
        if src_tail == 1:
            q = q.reshape(-1)
        if len(q) != len(x):
            raise ValueError(f"{len(x)} positions but {len(q)} charges / moments")
        res = np.empty((L, 2))
        ends = np.empty((L, 3)) if return_ends else None
        steps = np.empty(L, dtype=np.int32) if return_steps else None
        check(fn(prec, HOST, L, len(x), starts.ctypes.data, n_iter.ctypes.data, float(step),
                 half.ctypes.data, x.ctypes.data, q.ctypes.data, res.ctypes.data,
                 ends.ctypes.data if ends is not None else None,
                 steps.ctypes.data if steps is not None else None, None))
    out = [res]
    if return_ends:
        out.append(ends)
    if return_steps:
        out.append(steps)
    return out[0] if len(out) == 1 else tuple(out)


class _Plan:
    """A CUDA-graph plan of the library (cpetgb_plan) bound to device tensors."""

    def __init__(self, handle, keep):
        self.handle = handle
        self._keep = keep  # tensors the graph reads / writes

    @classmethod
    def grid(cls, kind, prec, clamp, desc, points, x, q, out):
        import ctypes

        h = ctypes.c_void_p()
        with __import__("torch").cuda.device(points.device):
            check(lib().cpetgb_grid_plan_create(ctypes.byref(h), kind, prec, clamp, len(desc), desc.ctypes.data,
                                                points.data_ptr(), x.data_ptr(), q.data_ptr(), out.data_ptr()))
        return cls(h, (desc, points, x, q, out))

    @classmethod
    def topo(cls, prec, desc, params, starts, n_iter, x, q, result, steps):
        import ctypes

        h = ctypes.c_void_p()
        with __import__("torch").cuda.device(starts.device):
            check(lib().cpetgb_topo_plan_create(ctypes.byref(h), prec, len(desc), desc.ctypes.data,
                                                params.ctypes.data, starts.data_ptr(), n_iter.data_ptr(),
                                                x.data_ptr(), q.data_ptr(), result.data_ptr(), None,
                                                steps.data_ptr() if steps is not None else None))
        return cls(h, (desc, params, starts, n_iter, x, q, result, steps))

    def launch(self, like):
        import torch

        with torch.cuda.device(like.device):
            check(lib().cpetgb_plan_launch(self.handle, _stream_of(like)))

    def __del__(self):
        if getattr(self, "handle", None):
            try:
                lib().cpetgb_plan_destroy(self.handle)
            except Exception:
                pass
            self.handle = None


class TopoBatch:
    """Streamlines of many frames in one persistent launch (frame descriptor table).

    frames: sequence of dicts with keys starts (L_f,3), n_iter (L_f,) or scalar,
    x (N_f,3), q (N_f,), step, half_dims (3,).  Inputs are concatenated once;
    ``run()`` returns (L_total, 2) results (split per frame with ``split``).
    With ``device=True`` the inputs live in torch CUDA tensors.
    """

    def __init__(self, frames, precision="fp32c", device=False, graph=False):
        self.prec = precision_code(precision)
        starts, caps, xs, qs, desc, params = [], [], [], [], [], []
        lo = co = 0
        for fr in frames:
            st = np.asarray(fr["starts"], np.float64).reshape(-1, 3)
            L = len(st)
            it = np.broadcast_to(np.asarray(fr["n_iter"]), (L,)).astype(np.int32)
            x = np.asarray(fr["x"], np.float64).reshape(-1, 3)
            q = np.asarray(fr["q"], np.float64).reshape(-1)
            h = np.asarray(fr["half_dims"], np.float64).reshape(3)
            desc.append((co, len(q), lo, L))
            params.append((float(fr["step"]), h[0], h[1], h[2]))
            starts.append(st), caps.append(it), xs.append(x), qs.append(q)
            lo += L
            co += len(q)
        self.desc = np.ascontiguousarray(np.array(desc, dtype=np.int64).reshape(-1, 4))
        self.params = np.ascontiguousarray(np.array(params, dtype=np.float64).reshape(-1, 4))
        self.starts = np.ascontiguousarray(np.concatenate(starts) if starts else np.zeros((0, 3)))
        self.n_iter = np.ascontiguousarray(np.concatenate(caps) if caps else np.zeros(0, np.int32))
        self.x = np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros((0, 3)))
        self.q = np.ascontiguousarray(np.concatenate(qs) if qs else np.zeros(0))
        self.n_lines = lo
        self.device = device
        if device:
            import torch

            self.starts = torch.from_numpy(self.starts).cuda()
            self.n_iter = torch.from_numpy(self.n_iter).cuda()
            self.x = torch.from_numpy(self.x).cuda()
            self.q = torch.from_numpy(self.q).cuda()
        self.plan = None
        if graph:
            if not device:
                raise ValueError("graph=True needs device=True (a plan binds device buffers)")
            import torch

            self.result = torch.empty((self.n_lines, 2), dtype=torch.float64, device=self.starts.device)
            self.steps = torch.empty((self.n_lines,), dtype=torch.int32, device=self.starts.device)
            self.plan = _Plan.topo(self.prec, self.desc, self.params, self.starts, self.n_iter, self.x, self.q,
                                   self.result, self.steps)

    def run(self, return_steps=False):
        if self.plan is not None:
            self.plan.launch(self.starts)
            return (self.result, self.steps) if return_steps else self.result
        if self.device:
            import torch

            dev = self.starts.device
            res = torch.empty((self.n_lines, 2), dtype=torch.float64, device=dev)
            steps = torch.empty((self.n_lines,), dtype=torch.int32, device=dev) if return_steps else None
            with torch.cuda.device(dev):
                check(lib().cpetgb_topo_batch(self.prec, DEVICE, len(self.desc), self.desc.ctypes.data,
                                              self.params.ctypes.data, self.starts.data_ptr(),
                                              self.n_iter.data_ptr(), self.x.data_ptr(), self.q.data_ptr(),
                                              res.data_ptr(), None, steps.data_ptr() if steps is not None else None,
                                              _stream_of(self.starts)))
        else:
            res = np.empty((self.n_lines, 2))
            steps = np.empty(self.n_lines, dtype=np.int32) if return_steps else None
            check(lib().cpetgb_topo_batch(self.prec, HOST, len(self.desc), self.desc.ctypes.data,
                                          self.params.ctypes.data, self.starts.ctypes.data, self.n_iter.ctypes.data,
                                          self.x.ctypes.data, self.q.ctypes.data, res.ctypes.data, None,
                                          steps.ctypes.data if steps is not None else None, None))
        return (res, steps) if return_steps else res

    def split(self, out):
        return [out[lo:lo + L] for _, _, lo, L in self.desc]


def topo_hist2d(result, bins=(20, 20), range=((0.0, 5.2), (0.0, None)), return_edges=False):
    """2-D histogram of (distance, curvature) rows with numpy.histogram2d's
    edges and binning (CPET/utils/calculator.py:702-707).  A range bound of
    None is taken from the data (column min or max).  Returns int64 counts of
    shape bins (and the two edge arrays)."""
    nb0, nb1 = (int(bins), int(bins)) if np.isscalar(bins) else (int(bins[0]), int(bins[1]))
    rng = np.array([math.nan if v is None else float(v) for pair in range for v in pair], dtype=np.float64)
    if _is_torch(result):
        import torch

        result = _dev(result, torch.float64, (2,))
        counts = torch.empty((nb0, nb1), dtype=torch.int64, device=result.device)
        edges = torch.empty((nb0 + nb1 + 2,), dtype=torch.float64, device=result.device)
        with torch.cuda.device(result.device):
            check(lib().cpetgb_topo_hist2d(DEVICE, result.shape[0], result.data_ptr(), nb0, nb1, rng.ctypes.data,
                                           counts.data_ptr(), edges.data_ptr(), _stream_of(result)))
    else:
        result = _host(result, np.float64, (2,))
        counts = np.empty((nb0, nb1), dtype=np.uint64)
        edges = np.empty(nb0 + nb1 + 2)
        check(lib().cpetgb_topo_hist2d(HOST, result.shape[0], result.ctypes.data, nb0, nb1, rng.ctypes.data,
                                       counts.ctypes.data, edges.ctypes.data, None))
        counts = counts.astype(np.int64)
    if return_edges:
        return counts, edges[:nb0 + 1], edges[nb0 + 1:]
    return counts


# ---------------------------------------------------------------------------
# Clustering front end: histogram sets and distance matrices
# ---------------------------------------------------------------------------

def topo_hist2d_sets(values, offsets, bins, range, normalize=True):
    """Histograms of many (distance, curvature) sets with one binning, in one
    launch (the per-file np.histogram2d loop of make_histograms,
    CPET/utils/calculator.py:689-711).  values (L,2); set f is rows
    offsets[f]:offsets[f+1].  range ((d_lo, d_hi), (c_lo, c_hi)) finite.
    Returns (F, nb0*nb1) float64 histograms each divided by its total
    (normalize=True, make_histograms' output rows) or int64 counts."""
    nb0, nb1 = (int(bins), int(bins)) if np.isscalar(bins) else (int(bins[0]), int(bins[1]))
    rng = np.array([float(v) for pair in range for v in pair], dtype=np.float64)
    off = np.ascontiguousarray(offsets, dtype=np.int64).reshape(-1)
    n_sets = len(off) - 1
    if _is_torch(values):
        import torch

        values = _dev(values, torch.float64, (2,))
        dev = values.device
        out = torch.empty((n_sets, nb0 * nb1), dtype=torch.float64 if normalize else torch.int64, device=dev)
        with torch.cuda.device(dev):
            check(lib().cpetgb_topo_hist2d_sets(DEVICE, n_sets, off.ctypes.data, values.data_ptr(), nb0, nb1,
                                                rng.ctypes.data, None if normalize else out.data_ptr(),
                                                out.data_ptr() if normalize else None, _stream_of(values)))
        return out
    values = _host(values, np.float64, (2,))
    out = np.empty((n_sets, nb0 * nb1), dtype=np.float64 if normalize else np.uint64)
    check(lib().cpetgb_topo_hist2d_sets(HOST, n_sets, off.ctypes.data, values.ctypes.data, nb0, nb1,
                                        rng.ctypes.data, None if normalize else out.ctypes.data,
                                        out.ctypes.data if normalize else None, None))
    return out if normalize else out.astype(np.int64)


def _distance_matrix(fn, rows, tail, precision):
    prec = precision_code(precision)
    if _is_torch(rows):
        import torch

        rows = _dev(rows, torch.float64)
        n = rows.shape[0]
        feat = rows[0].numel() // tail if n else 0
        out = torch.empty((n, n), dtype=torch.float64, device=rows.device)
        with torch.cuda.device(rows.device):
            check(fn(prec, DEVICE, n, feat, rows.data_ptr(), out.data_ptr(), _stream_of(rows)))
        return out
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    n = rows.shape[0]
    feat = rows[0].size // tail if n else 0
    out = np.empty((n, n))
    check(fn(prec, HOST, n, feat, rows.ctypes.data, out.ctypes.data, None))
    return out


def chi2_distance_matrix(hists, precision="fp32c"):
    """(F, B) histograms -> (F, F) matrix of 1/2 sum (a-b)^2/(a+b) over bins
    with a+b != 0 (construct_distance_matrix with distance_numpy,
    CPET/utils/calculator.py:975-978, 1003-1015); zero diagonal."""
    hists = hists if _is_torch(hists) else np.asarray(hists, np.float64)
    if hists.ndim != 2:
        raise ValueError("hists must be (n_histograms, n_bins)")
    return _distance_matrix(lib().cpetgb_chi2_distance_matrix, hists, 1, precision)


def field_distance_matrix(fields, precision="fp32c"):
    """(F, P, 3) vector fields on one grid -> (F, F) matrix of sum_p |f_i[p] -
    f_j[p]| (construct_distance_matrix_volume, CPET/utils/calculator.py:1042-1058)."""
    fields = fields if _is_torch(fields) else np.asarray(fields, np.float64)
    if fields.ndim != 3 or fields.shape[2] != 3:
        raise ValueError("fields must be (n_fields, n_points, 3)")
    return _distance_matrix(lib().cpetgb_field_distance_matrix, fields, 3, precision)


# ---------------------------------------------------------------------------
# Output text
# ---------------------------------------------------------------------------

def format_fixed3(values) -> bytes:
    """Rows of a float32 (or float16) matrix as numpy.savetxt(fmt="%.3f")
    writes them, formatted on the GPU (cpetgb_format_fixed3): each value
    correctly rounded to 3 decimals, single spaces, "\\n" after each row."""
    import ctypes

    v = np.asarray(values)
    if v.dtype not in (np.float32, np.float16):
        raise TypeError("format_fixed3 formats float32 / float16 values exactly; got " + str(v.dtype))
    cols = int(np.prod(v.shape[1:])) if v.ndim > 1 else 1
    v = np.ascontiguousarray(v.reshape(v.shape[0] if v.ndim else 1, cols), dtype=np.float32)
    n, m = v.shape
    if n == 0:
        return b""
    length = ctypes.c_int64(0)
    check(lib().cpetgb_format_fixed3(HOST, n, m, v.ctypes.data, None, 0, ctypes.byref(length), None))
    buf = ctypes.create_string_buffer(max(length.value, 1))
    check(lib().cpetgb_format_fixed3(HOST, n, m, v.ctypes.data, buf, length.value, ctypes.byref(length), None))
    return buf.raw[:length.value]


def format_sci18(values) -> bytes:
    """Rows of a float32 matrix as numpy.savetxt(fname, X) writes them with
    its default fmt "%.18e" (the .top files of the topology dispatcher,
    CPET/source/CPET.py:123), formatted on the GPU (cpetgb_format_sci18):
    every value exactly rounded to 19 significant digits, single spaces, "\n"
    after each row."""
    import ctypes

    v = np.asarray(values)
    if v.dtype != np.float32:
        raise TypeError("format_sci18 formats float32 values exactly; got " + str(v.dtype))
    cols = int(np.prod(v.shape[1:])) if v.ndim > 1 else 1
    v = np.ascontiguousarray(v.reshape(v.shape[0] if v.ndim else 1, cols))
    n, m = v.shape
    if n == 0:
        return b""
    cap = n * m * 26
    buf = ctypes.create_string_buffer(cap)
    length = ctypes.c_int64(0)
    check(lib().cpetgb_format_sci18(HOST, n, m, v.ctypes.data, buf, cap, ctypes.byref(length), None))
    return buf.raw[:length.value]


# ---------------------------------------------------------------------------
# Frame preparation
# ---------------------------------------------------------------------------

def residue_codes(resid, resnum):
    """int32 codes for the residue radius filter: equal (resid, resnum) give
    equal codes (resid names such as 'ALA' are mapped to integers)."""
    resid = np.asarray(resid)
    if resid.dtype.kind in "iu":
        codes = resid.astype(np.int32)
    else:
        _, codes = np.unique(resid.astype(str), return_inverse=True)
    return np.ascontiguousarray(codes, dtype=np.int32), np.ascontiguousarray(resnum, dtype=np.int32)


def prepare_frame(x, q, center, inv_basis=None, radius=None, resid=None, resnum=None, box_half=None,
                  box_shift=None):
    """The calculator's per-frame preparation on the GPU (cpetgb_prepare_frame;
    CPET/source/calculator.py:239-251, 341-371): optional residue radius
    filter (io.py:283-338), rotation (x - center) @ inv_basis, optional box
    filter (io.py:422-475, with the reference's second recentring), optional
    box shift.  Returns (x_box (M,3), q (M,)) float64 of the kept atoms in
    input order (torch tensors when x is one)."""
    import ctypes

    c = np.ascontiguousarray(np.asarray(center, np.float64).reshape(3))
    inv = None if inv_basis is None else np.ascontiguousarray(np.asarray(inv_basis, np.float64).reshape(9))
    half = None if box_half is None else np.ascontiguousarray(np.asarray(box_half, np.float64).reshape(3))
    shift = None if box_shift is None else np.ascontiguousarray(np.asarray(box_shift, np.float64).reshape(3))
    r = 0.0 if radius is None else float(radius)
    n_out = ctypes.c_int(0)
    ptr = lambda a: None if a is None else a.ctypes.data
    if r > 0.0:
        if resid is None or resnum is None:
            raise ValueError("the residue radius filter needs resid and resnum")
        rc_, rn_ = residue_codes(resid, resnum)
    if _is_torch(x):
        import torch

        x, q = _dev(x, torch.float64, (3,)), _dev(q, torch.float64, ())
        n = x.shape[0]
        xo = torch.empty_like(x)
        qo = torch.empty_like(q)
        dr = dn = None
        if r > 0.0:
            dr, dn = torch.from_numpy(rc_).to(x.device), torch.from_numpy(rn_).to(x.device)
        with torch.cuda.device(x.device):
            check(lib().cpetgb_prepare_frame(DEVICE, n, x.data_ptr(), q.data_ptr(),
                                             dr.data_ptr() if dr is not None else None,
                                             dn.data_ptr() if dn is not None else None, ptr(c), ptr(inv), r,
                                             ptr(half), ptr(shift), xo.data_ptr(), qo.data_ptr(),
                                             ctypes.byref(n_out), _stream_of(x)))
        return xo[:n_out.value], qo[:n_out.value]
    x, q = _host(x, np.float64, (3,)), _host(q, np.float64).reshape(-1)
    n = x.shape[0]
    xo, qo = np.empty_like(x), np.empty_like(q)
    check(lib().cpetgb_prepare_frame(HOST, n, x.ctypes.data, q.ctypes.data, ptr(rc_) if r > 0 else None,
                                     ptr(rn_) if r > 0 else None, ptr(c), ptr(inv), r, ptr(half), ptr(shift),
                                     xo.ctypes.data, qo.ctypes.data, ctypes.byref(n_out), None))
    return xo[:n_out.value], qo[:n_out.value]
