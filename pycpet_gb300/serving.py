"""Serving loop: continuous batching of Coulomb requests on one GPU.

Requests (``point_field``, ``volume``, ``volume_esp``, ``topo``) arrive over
time against frames whose charges stay resident on the device.

* Streamlines go to the library's engine (``cpetgb_engine_*``): a persistent
  kernel whose warps claim chunks of lines from a ring the host appends to, so
  a request arriving while others run is admitted as line slots free up and
  its lines are swept by the same warps, overlapping on the device.
* Grid and point requests that are waiting are batched into one
  descriptor-table launch per kind (field with the r^2 clamp, unclamped point
  fields, potential) on one of two side streams, beside the engine kernel
  (which, at one CTA per SM, leaves half of every SM's registers free for
  them; a streamline-only server gives the engine two).
* Admission: a request is started only while the memory it needs fits an HBM
  budget (80% of the device by default) next to the resident frames; the
  engine also refuses (and the loop retries) when its line store is full.
* Refusals and the watchdog: a request that can never run -- an unknown kind
  or frame, no points or lines, non-finite coordinates, a step cap outside
  [0, 2^24], more memory than the budget leaves beside the resident frames --
  is refused at submit() with status "rejected" and a message, and counts as
  completed; with ``pending_deadline_s`` set, a request still waiting for
  admission that long after its arrival is cancelled with status "expired".
  Frames with no charges or with non-finite positions or charges are refused
  by add_frame().  The reference has no request loop; its only recovery is to
  skip inputs whose output file exists (CPET/source/CPET.py:119-126).

Latency is measured from a request's arrival to its results on the host.
"""
from __future__ import annotations

import ctypes
import heapq
import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import DEVICE, EAGAIN, ESP, FIELD, check, lib
from .core import precision_code

KINDS = ("point_field", "volume", "volume_esp", "topo")


@dataclass
class Request:
    kind: str
    frame: int
    arrival: float = 0.0
    points: np.ndarray | None = None      # grid / point requests (P,3)
    starts: np.ndarray | None = None      # topo (L,3)
    n_iter: np.ndarray | int | None = None
    step: float = 0.001
    half_dims: tuple = (1.5, 1.5, 1.5)
    result: np.ndarray | None = None
    t_start: float | None = None
    t_done: float | None = None
    status: str = "new"                   # pending, running, done, rejected, expired
    error: str | None = None
    _rid: int = -1

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival

    def bytes_needed(self) -> int:
        if self.kind == "topo":
            return int(len(self.starts) * 48)
        return int(len(self.points) * 48)


MAX_STEP_CAP = 1 << 24   # the library's largest per-line step cap


def validate_request(req: Request, frames, max_bytes: int) -> str | None:
    """Why `req` can never be served (a message), or None.  `frames` holds the
    resident frame ids; `max_bytes` is what the budget leaves beside them."""
    if req.kind not in KINDS:
        return f"unknown request kind {req.kind!r}"
    if req.frame not in frames:
        return f"frame {req.frame} is not resident"
    if req.kind == "topo":
        if req.starts is None:
            return "a topo request needs start points"
        st = np.asarray(req.starts, np.float64).reshape(-1, 3)
        if len(st) == 0:
            return "a topo request needs at least one start point"
        if not np.all(np.isfinite(st)):
            return "start points must be finite"
        caps = np.asarray(req.n_iter if req.n_iter is not None else 0)
        if caps.size not in (1, len(st)) or np.any(caps < 0) or np.any(caps > MAX_STEP_CAP):
            return f"step caps must be one value or one per line, in [0, {MAX_STEP_CAP}]"
        if not np.isfinite(req.step):
            return "the step must be finite"
        half = np.asarray(req.half_dims, np.float64)
        if half.size != 3 or not np.all(np.isfinite(half)) or np.any(half < 0):
            return "half_dims must be three finite values >= 0"
    else:
        if req.points is None:
            return "a grid or point request needs points"
        pts = np.asarray(req.points, np.float64).reshape(-1, 3)
        if len(pts) == 0:
            return "a grid or point request needs at least one point"
        if not np.all(np.isfinite(pts)):
            return "points must be finite"
    if req.bytes_needed() > max_bytes:
        return f"needs {req.bytes_needed()} bytes, more than the {max_bytes} the HBM budget leaves"
    return None


def expire_pending(pending, now: float, deadline_s: float | None):
    """Splits waiting requests into (kept, expired) by the pending deadline."""
    if deadline_s is None:
        return list(pending), []
    kept, expired = [], []
    for r in pending:
        (expired if now - r.arrival > deadline_s else kept).append(r)
    return kept, expired


@dataclass
class _GridLaunch:
    event: object
    reqs: list
    out: object
    nc: int
    nbytes: int
    keep: list = field(default_factory=list)


class Server:
    def __init__(self, precision="fp32c", hbm_budget_frac=0.8, line_capacity=2_000_000,
                 charge_capacity=4_000_000, max_frames=64, max_requests=4096, chunk_lines=32,
                 engine_ctas_per_sm=1, pending_deadline_s=None):
        """``engine_ctas_per_sm``: 1 keeps half of every SM free for grid and
        point requests (mixed serving); 2 gives the streamline engine whole SMs
        (streamline-only serving: about 1.5x the line throughput, but a grid
        request then waits until the engine's launch ends).
        ``pending_deadline_s``: cancel requests not admitted that long after
        their arrival (None: wait indefinitely)."""
        import torch

        self.torch = torch
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.prec_name = precision
        self.prec = precision_code(precision)
        free, total = torch.cuda.mem_get_info(self.dev)
        self.budget = int(hbm_budget_frac * total)
        self.resident_bytes = 0
        self.inflight_bytes = 0
        h = ctypes.c_void_p()
        check(lib().cpetgb_engine_create(ctypes.byref(h), self.prec, int(charge_capacity), int(line_capacity),
                                         int(max_frames), int(max_requests), int(chunk_lines)))
        self.engine = h
        check(lib().cpetgb_engine_set_ctas_per_sm(h, int(engine_ctas_per_sm)))
        self.resident_bytes += int(charge_capacity * 32 + line_capacity * 56)
        self.frames = {}          # frame id -> dict(engine id, offset in the grid pool, n)
        self._gx, self._gq = [], []
        self._pool_x = self._pool_q = None
        self.grid_streams = [torch.cuda.Stream(self.dev), torch.cuda.Stream(self.dev)]
        self.grid_inflight: list[_GridLaunch] = []
        self.pending: list[Request] = []
        self.topo_running: list[Request] = []
        self.completed: list[Request] = []
        self.max_topo_inflight = 0
        self.pending_deadline_s = pending_deadline_s

    # ---- frames ---------------------------------------------------------------
    def add_frame(self, frame_id, x, q):
        x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 3))
        q = np.ascontiguousarray(np.asarray(q, np.float64).reshape(-1))
        if len(q) == 0 or len(x) != len(q):
            raise ValueError(f"frame {frame_id}: needs one position per charge and at least one charge")
        if not (np.all(np.isfinite(x)) and np.all(np.isfinite(q))):
            raise ValueError(f"frame {frame_id}: positions and charges must be finite")
        fid = ctypes.c_int(-1)
        check(lib().cpetgb_engine_add_frame(self.engine, len(q), x.ctypes.data, q.ctypes.data, ctypes.byref(fid)))
        off = sum(len(a) for a in self._gq)
        self._gx.append(x)
        self._gq.append(q)
        self._pool_x = self._pool_q = None  # grid pool rebuilt lazily
        self.frames[frame_id] = {"engine": fid.value, "off": off, "n": len(q)}
        self.resident_bytes += 32 * len(q) * 2

    def _grid_pool(self):
        if self._pool_x is None:
            t = self.torch
            self._pool_x = t.from_numpy(np.concatenate(self._gx)).to(self.dev)
            self._pool_q = t.from_numpy(np.concatenate(self._gq)).to(self.dev)
        return self._pool_x, self._pool_q

    # ---- requests ---------------------------------------------------------------
    def submit(self, req: Request) -> bool:
        """Queues `req` (True) or refuses it at once (False: status
        "rejected", the reason in ``req.error``, counted as completed)."""
        why = validate_request(req, self.frames, self.budget - self.resident_bytes)
        if why is not None:
            req.status, req.error = "rejected", why
            req.t_done = time.perf_counter()
            self.completed.append(req)
            return False
        req.status = "pending"
        self.pending.append(req)
        return True

    def _fits(self, nbytes):
        return self.resident_bytes + self.inflight_bytes + nbytes <= self.budget

    def _admit_topo(self, req, now):
        starts = np.ascontiguousarray(np.asarray(req.starts, np.float64).reshape(-1, 3))
        L = len(starts)
        caps = np.ascontiguousarray(np.broadcast_to(np.asarray(req.n_iter), (L,)), dtype=np.int32)
        half = np.ascontiguousarray(np.asarray(req.half_dims, np.float64).reshape(3))
        rid = ctypes.c_int(-1)
        rc = lib().cpetgb_engine_submit(self.engine, self.frames[req.frame]["engine"], L, starts.ctypes.data,
                                        caps.ctypes.data, float(req.step), half.ctypes.data, ctypes.byref(rid))
        if rc == EAGAIN:
            return False
        check(rc)
        req._rid = rid.value
        req.t_start = now
        req.status = "running"
        self.topo_running.append(req)
        self.max_topo_inflight = max(self.max_topo_inflight, len(self.topo_running))
        return True

    def _launch_grid(self, reqs, kind_code, clamp, now):
        t = self.torch
        px, pq = self._grid_pool()
        desc, pts, po = [], [], 0
        for r in reqs:
            f = self.frames[r.frame]
            p = np.asarray(r.points, np.float64).reshape(-1, 3)
            desc.append((f["off"], f["n"], po, len(p)))
            pts.append(p)
            po += len(p)
            r.t_start = now
            r.status = "running"
        desc = np.ascontiguousarray(np.array(desc, dtype=np.int64))
        host_pts = t.from_numpy(np.concatenate(pts)).pin_memory()
        nc = 3 if kind_code == FIELD else 1
        stream = min(self.grid_streams, key=lambda s: sum(1 for g in self.grid_inflight if g.keep[0] is s))
        with t.cuda.stream(stream):
            d_pts = host_pts.to(self.dev, non_blocking=True)
            out = t.empty((po, nc), dtype=t.float64, device=self.dev)
            check(lib().cpetgb_grid_batch(kind_code, self.prec, DEVICE, int(clamp), len(desc), desc.ctypes.data,
                                          d_pts.data_ptr(), px.data_ptr(), pq.data_ptr(), out.data_ptr(),
                                          stream.cuda_stream))
            host_out = t.empty((po, nc), dtype=t.float64, pin_memory=True)
            host_out.copy_(out, non_blocking=True)
            ev = t.cuda.Event()
            ev.record(stream)
        nbytes = po * 48
        self.inflight_bytes += nbytes
        self.grid_inflight.append(_GridLaunch(ev, list(reqs), host_out, nc, nbytes,
                                              keep=[stream, d_pts, out, host_pts, desc]))

    def step(self, now=None):
        """One pass of the loop: admit, launch, poll.  Returns True if anything moved."""
        now = time.perf_counter() if now is None else now
        moved = False
        self.pending, expired = expire_pending(self.pending, now, self.pending_deadline_s)
        for r in expired:
            r.status, r.error = "expired", f"not admitted within {self.pending_deadline_s} s"
            r.t_done = now
            self.completed.append(r)
            moved = True
        # streamlines: into the engine while it accepts them
        still = []
        for r in self.pending:
            if r.kind == "topo":
                if self._fits(r.bytes_needed()) and self._admit_topo(r, now):
                    moved = True
                    continue
            still.append(r)
        self.pending = still
        # grid / point requests: one batched launch per kind, at most 2 in flight
        if len(self.grid_inflight) < 2:
            groups = {"volume": [], "volume_esp": [], "point_field": []}
            rest = []
            for r in self.pending:
                if r.kind in groups and self._fits(r.bytes_needed()):
                    groups[r.kind].append(r)
                else:
                    rest.append(r)
            self.pending = rest
            for kind, reqs in groups.items():
                if not reqs:
                    continue
                if kind == "volume":
                    self._launch_grid(reqs, FIELD, True, now)
                elif kind == "volume_esp":
                    self._launch_grid(reqs, ESP, False, now)
                else:
                    self._launch_grid(reqs, FIELD, False, now)
                moved = True
        # completions
        done_now = time.perf_counter()
        keep = []
        for g in self.grid_inflight:
            if g.event.query():
                out = g.out.numpy()
                po = 0
                for r in g.reqs:
                    n = len(np.asarray(r.points).reshape(-1, 3))
                    r.result = out[po:po + n].copy() if g.nc == 3 else out[po:po + n, 0].copy()
                    po += n
                    r.t_done = done_now
                    r.status = "done"
                    self.completed.append(r)
                self.inflight_bytes -= g.nbytes
                moved = True
            else:
                keep.append(g)
        self.grid_inflight = keep
        still = []
        for r in self.topo_running:
            st = lib().cpetgb_engine_poll(self.engine, r._rid)
            if st < 0:
                check(st)
            if st == 1:
                L = len(np.asarray(r.starts).reshape(-1, 3))
                res = np.empty((L, 2))
                check(lib().cpetgb_engine_collect(self.engine, r._rid, res.ctypes.data, None))
                r.result = res
                r.t_done = time.perf_counter()
                r.status = "done"
                self.completed.append(r)
                moved = True
            else:
                still.append(r)
        self.topo_running = still
        return moved

    def busy(self):
        return bool(self.pending or self.topo_running or self.grid_inflight)

    def run(self, schedule, timeout_s=600.0):
        """Replays `schedule` (requests with arrival offsets in seconds) in real
        time and serves until all are done.  Returns the completed requests."""
        t0 = time.perf_counter()
        heap = [(r.arrival, i, r) for i, r in enumerate(schedule)]
        heapq.heapify(heap)
        while heap or self.busy():
            now = time.perf_counter()
            if now - t0 > timeout_s:
                raise TimeoutError("serving loop did not finish in time")
            while heap and heap[0][0] <= now - t0:
                _, _, r = heapq.heappop(heap)
                r.arrival = t0 + r.arrival
                self.submit(r)
            if not self.step(now) and not heap:
                time.sleep(2e-5)
            elif not self.busy() and heap:
                time.sleep(max(0.0, min(1e-3, heap[0][0] - (time.perf_counter() - t0))))
        return schedule

    def close(self):
        if getattr(self, "engine", None):
            lib().cpetgb_engine_drain(self.engine)
            lib().cpetgb_engine_destroy(self.engine)
            self.engine = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def latency_stats(reqs):
    """p50 / p99 latency (ms) per kind and overall."""
    out = {}
    for kind in KINDS + ("all",):
        lat = [r.latency for r in reqs
               if r.latency is not None and r.status == "done" and (kind == "all" or r.kind == kind)]
        if lat:
            out[kind] = {"n": len(lat), "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                         "p99_ms": 1e3 * float(np.percentile(lat, 99))}
    return out


def synthetic_schedule(frames, n_requests, rate_hz, seed=0, topo_lines=(1_000, 10_000), volume_sides=(11, 51),
                       step=0.001, cap=6000, half=1.5):
    """Poisson arrivals mixing point_field (1-64 points), volume / volume_esp
    (cubic grids of volume_sides points per side, 0.1 A spacing) and topo
    (topo_lines lines) over the given frame ids."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        kind = KINDS[rng.integers(0, 4)]
        f = int(rng.choice(frames))
        if kind == "point_field":
            out.append(Request(kind, f, t, points=rng.uniform(-half, half, (int(rng.integers(1, 65)), 3))))
        elif kind in ("volume", "volume_esp"):
            side = int(rng.integers(volume_sides[0] // 10, volume_sides[1] // 10 + 1)) * 10 + 1
            h = (side - 1) * 0.05
            g = np.linspace(-h, h, side)
            pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
            out.append(Request(kind, f, t, points=pts))
        else:
            L = int(rng.integers(topo_lines[0], topo_lines[1] + 1))
            st = np.column_stack([rng.uniform(-half, half, L) for _ in range(3)])
            out.append(Request(kind, f, t, starts=st, n_iter=cap, step=step, half_dims=(half, half, half)))
    return out
