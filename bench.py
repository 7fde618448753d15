#!/usr/bin/env python
"""Benchmark of the Coulomb streamline hot path on GB300.

Workload (one step = one pass over one frame, inputs resident in HBM):
  'topo', 1 frame: 8,000 synthetic charges (50 A cube, >= 1 A apart, none
  within 2 A of the centre, q ~ N(0, 0.4) clipped, integer net charge),
  100,000 seeded uniform start points in a box of half-width 1.5 A, Euler
  step 0.001 A, at most 6,000 steps per line; per line the start-to-end
  distance and mean curvature; a 20x20 histogram over distance [0, 5.2] and
  curvature [0, max].  Computed in the FP32-compensated form.

Printed (rank 0, one JSON line): streamlines/s (value), pair-evaluations/s,
per-step latency p50/p99, the same workload end to end through the C ABI with
host buffers (e2e), the roofline of the streamline kernel against the FP32
pipe peak measured in this run, the plain FP64 form and the batched grid
workload for comparison, the CPU baseline (the oracle's restatement of the
reference's float arithmetic on all host cores) and the SM clocks seen.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Multi-GPU: one process per GPU (torchrun); each rank processes its own frame
and lines, no data-path collective ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair-evals/s & streamlines/s, FP32-comp vs FP64 plain at stated err; p50/p99"
N_CHARGES, N_LINES, HALF, STEP, CAP = 8000, 100_000, 1.5, 0.001, 6000
FLOPS_PER_PAIR = 17        # 3 sub, r^2 (1 mul + 2 fma), r^-3 (2 mul), q (1 mul), 3 fma accumulate
L2_FLUSH_BYTES = 256 << 20


def workload_config():
    """The workload (identical in both arms; the arithmetic form is the line's
    top-level "precision")."""
    return {
        "workload": "topo, 1 frame: 8,000 charges, 100,000 seeded uniform start points, half-width 1.5 A, "
                    "step 0.001 A, cap 6,000 steps, 20x20 (distance 0-5.2 A, curvature 0-max) histogram",
        "n_charges": N_CHARGES, "n_lines": N_LINES, "half_width_A": HALF, "step_A": STEP, "cap": CAP,
        "histogram": [20, 20],
        "l2": "flushed between timed steps (256 MiB device write)",
    }


PRECISION_DETAIL = ("FP32C: FP32 pair terms, Kahan across charge tiles, TwoSum warp reduction; "
                    "FP64 positions, box test, curvature and distance")
# CPU legs (our cpu_baseline and the --impl reference arm) time the same sample:
# every CPU_STRIDE-th line of the 100,000, all of it in one call, the lines
# spread over all host threads by an atomic counter (the oracle's _mt driver).
CPU_STRIDE = 100


def cpu_sample(starts, caps):
    idx = np.arange(0, len(starts), CPU_STRIDE)
    return starts[idx], caps[idx]


def make_inputs(rank: int):
    from pycpet_gb300.synth import topo_workload

    return topo_workload(rank)


def pair_evals(steps, n_charges):
    s = np.asarray(steps, dtype=np.int64)
    return int(np.sum(np.maximum(s, 2) + 2) * n_charges)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for name, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_pass(x, q, st, cp, threads):
    """One pass of the reference's float arithmetic (the oracle's restatement
    of thread_operation, math_module.c:523-591) over the sample lines."""
    from oracle import oracle

    t0 = time.perf_counter()
    _, _, steps = oracle.topo_lines_f32(st, cp, x, q, STEP, [HALF] * 3, threads=threads)
    return time.perf_counter() - t0, steps


def cpu_baseline(x, q, starts, caps, min_s=10.0, threads=None):
    """The CPU leg of this arm: the sample of cpu_sample() on all host cores,
    repeated until at least `min_s` seconds have passed."""
    threads = threads or os.cpu_count() or 1
    st, cp = cpu_sample(starts, caps)
    total, passes, steps = 0.0, 0, None
    while total < min_s or passes == 0:
        dt, steps = cpu_pass(x, q, st, cp, threads)
        total += dt
        passes += 1
    return {"lines": len(st) * passes, "seconds": total, "streamlines_per_s": len(st) * passes / total,
            "pair_evals_per_s": pair_evals(steps, len(q)) * passes / total, "cores": threads, "passes": passes}


def cpu_sample_text(n):
    return (f"every {CPU_STRIDE}th of the 100,000 lines ({n} lines, same frame, starts and caps) per pass, "
            "one call spreading lines over all host threads; the oracle's restatement of the reference's "
            "float C (thread_operation)")


def run_reference(args, world):
    """--impl reference: the reference's CPU implementation of the path (the
    oracle's port of its float C; the reference library itself cannot be
    built on the GPU host) timed on the host cores: each step is one pass over
    the same strided sample the other arm's cpu_baseline times."""
    from oracle import oracle

    oracle.lib()
    x, q, starts, caps = make_inputs(0)
    threads = os.cpu_count() or 1
    st, cp = cpu_sample(starts, caps)
    times, pe = [], 0
    for i in range(args.warmup + args.steps):
        dt, steps = cpu_pass(x, q, st, cp, threads)
        if i >= args.warmup:
            times.append(dt)
            pe = pair_evals(steps, len(q))
    total = sum(times)
    value = len(st) * len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "streamlines/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; no dataset ships with the benchmark)", "config": workload_config(),
        "precision": "reference float arithmetic (float storage and sums, double pow/sqrt)",
        "pair_evals_per_s": pe * len(times) / total,
        "cpu_baseline": {"value": value, "unit": "streamlines/s", "cores": threads, "kind": "port",
                         "sample": cpu_sample_text(len(st))},
        "e2e": {"value": value, "unit": "streamlines/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64 / grid / CPU comparison legs")
    ap.add_argument("--lines", type=int, default=N_LINES, help="streamlines per step (smaller cases for ncu)")
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"],
                    help="topo workload: arithmetic form of the timed step (fp64: the plain drop-in form)")
    ap.add_argument("--workload", default="topo", choices=["topo", "grid", "topo-batch", "serve", "cluster", "topo-dipole", "dat", "prep"],
                    help="grid: the 64-frame batched volume + volume_ESP workload; topo-batch: "
                         "frames of 5,000-20,000 charges with uneven line counts in one launch")
    ap.add_argument("--requests", type=int, default=400, help="serve: number of requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: mean arrival rate (requests/s)")
    ap.add_argument("--line-scale", type=float, default=0.1,
                    help="topo-batch: fraction of the 100,000-1,000,000 lines per frame")
    ap.add_argument("--frames", type=int, default=64, help="frames of the grid workload")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, world)
        return

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local_rank)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    from pycpet_gb300 import build as gbuild
    from pycpet_gb300 import _lib, topo_hist2d, topo_lines
    from pycpet_gb300.core import GridBatch

    gbuild.build_library()
    dev = torch.device("cuda", local_rank)
    if args.workload == "grid":
        return grid_main(args, rank, world, dev, torch, dist)
    if args.workload == "topo-batch":
        return topo_batch_main(args, rank, world, dev, torch, dist)
    if args.workload == "serve":
        return serve_main(args, rank, world, dev, torch, dist)
    if args.workload == "cluster":
        return cluster_main(args, rank, world, dev, torch, dist)
    if args.workload == "topo-dipole":
        return dipole_main(args, rank, world, dev, torch, dist)
    if args.workload == "dat":
        return dat_main(args, rank, world, dev, torch, dist)
    if args.workload == "prep":
        return prep_main(args, rank, world, dev, torch, dist)
    x, q, starts, caps = make_inputs(rank)
    if args.lines != N_LINES:
        starts, caps = starts[:args.lines], caps[:args.lines]
    d_x = torch.from_numpy(x).to(dev)
    d_q = torch.from_numpy(q).to(dev)
    d_starts = torch.from_numpy(starts).to(dev)
    d_caps = torch.from_numpy(caps).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    hist_range = ((0.0, 5.2), (0.0, None))

    # step counts (deterministic) for the pair-evaluation count
    prec = args.precision
    res, steps = topo_lines(d_starts, d_caps, d_x, d_q, STEP, [HALF] * 3, precision=prec, return_steps=True)
    torch.cuda.synchronize()
    pe_step = pair_evals(steps.cpu().numpy(), N_CHARGES)

    def step(ev_k0=None, ev_k1=None):
        if ev_k0 is not None:
            ev_k0.record(stream)
        r = topo_lines(d_starts, d_caps, d_x, d_q, STEP, [HALF] * 3, precision=prec)
        if ev_k1 is not None:
            ev_k1.record(stream)
        return r, topo_hist2d(r, bins=(20, 20), range=hist_range)

    for _ in range(args.warmup):
        step()
    # FP32 pipe peak of this GPU, measured now: the higher of scalar FFMA and packed FFMA2
    ffma_scalar, ffma2 = _lib.measure_peak(0), _lib.measure_peak(3)
    ffma = max(ffma_scalar, ffma2)
    loop_rate = _lib.measure_peak(4)  # the sweep's inner loop alone (pair evaluations/s)
    peak = ffma if prec == "fp32c" else _lib.measure_peak(1)  # FP64 form: the DFMA pipe
    torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    sampler = ClockSampler(local_rank)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    for k in range(args.steps):
        e0, ek0, ek1, e1 = evs[k]
        e0.record(stream)
        res, counts = step(ek0, ek1)
        e1.record(stream)
        flush.fill_(k & 0xFF)  # evict L2 between timed steps (outside the events)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    _lib.check(_lib.lib().cpetgb_synchronize(stream.cuda_stream))
    step_ms = [e[0].elapsed_time(e[3]) for e in evs]
    kern_ms = [e[1].elapsed_time(e[2]) for e in evs]
    total_s = sum(step_ms) * 1e-3
    if world > 1:
        t = torch.tensor([total_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())

    n_lines = len(starts)
    value = n_lines * world * args.steps / total_s
    pe_per_s = pe_step * world * args.steps / total_s
    avg_kern_s = statistics.mean(kern_ms) * 1e-3
    achieved = pe_step * FLOPS_PER_PAIR / avg_kern_s
    traffic = None
    try:  # DRAM bytes per line from the committed ncu capture, scaled to this launch
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as fh:
            traffic = json.load(fh)["topo_kernel FP32C"]["dram_bytes_per_line"] * len(starts)
    except (OSError, KeyError, ValueError):
        pass
    out = {
        "metric": METRIC, "value": value, "unit": "streamlines/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; no dataset ships with the benchmark)",
        "config": dict(workload_config(), n_lines=n_lines),
        "precision": prec, "precision_detail": PRECISION_DETAIL if prec == "fp32c" else "IEEE double throughout",
        "pair_evals_per_s": pe_per_s,
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "roofline": {"bound": "fp32" if prec == "fp32c" else "fp64", "achieved": achieved / 1e12,
                     "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": traffic if prec == "fp32c" else None,
                     "traffic_note": ("DRAM bytes per launch (ncu capture of 20,000 lines scaled by lines); "
                                      "the kernel is FP32-pipe bound, the charges stay in shared memory")
                     if prec == "fp32c" else "FP64-pipe bound; charges read from L2",
                     "frac_ceiling": 17 / 24,
                     "sweep_loop_pair_evals_per_s": loop_rate,
                     "frac_of_sweep_loop": (pe_step / avg_kern_s) / loop_rate,
                     "kernel": ("topo_kernel (FP32C, charges resident in shared memory)" if prec == "fp32c"
                                else "topo_kernel (FP64, charges from L2)"),
                     "work": f"{FLOPS_PER_PAIR} flop per pair evaluation x sum_lines N*(max(s,2)+2)",
                     "peak_source": ("FP32 pipe measured in this run (cpetgb_measure_peak): the higher of "
                                     f"FFMA {ffma_scalar / 1e12:.1f} and packed FFMA2 {ffma2 / 1e12:.1f} TFLOP/s"
                                     if prec == "fp32c" else "DFMA throughput measured in this run")
                                    + "; MEASURED_PEAKS.json holds HBM and bf16 figures only"},
        "gpu_launches": 4 * args.steps,
        "clocks": clocks,
    }

    if rank == 0:
        # e2e: the same step through the C ABI with host buffers in pinned memory,
        # every one of the --steps repetitions timed
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        h_starts, h_caps, h_x, h_q = pin(starts), pin(caps), pin(x), pin(q)
        topo_lines(h_starts[:1024], h_caps[:1024], h_x, h_q, STEP, [HALF] * 3, precision=prec)
        e2e_t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = topo_lines(h_starts, h_caps, h_x, h_q, STEP, [HALF] * 3, precision=prec)
            c = topo_hist2d(r, bins=(20, 20), range=hist_range)
            e2e_t.append(time.perf_counter() - t0)
        # in: starts, caps, charges; the histogram call uploads the (L,2) result again
        h2d = h_starts.nbytes + h_caps.nbytes + h_x.nbytes + h_q.nbytes + r.nbytes
        d2h = r.nbytes + c.nbytes + 8 * 42       # result, counts, bin edges
        out["e2e"] = {"value": n_lines * len(e2e_t) / sum(e2e_t), "unit": "streamlines/s",
                      "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                      "steps": len(e2e_t),
                      "path": "cpetgb_topo_lines then cpetgb_topo_hist2d, CPETGB_HOST, pinned buffers "
                              "(the histogram call copies the result back in)"}
        if not args.no_extras and world == 1:
            dfma = _lib.measure_peak(1)
            out.update(extras(d_starts, d_caps, d_x, d_q, torch, topo_lines, GridBatch, dfma))
            tb = topo_batch_measure(rank, world, dev, torch, dist, 32, 0.1, steps=1, warmup=1)
            out["topo_batch"] = tb
            frames, serving = serve_measure(rank, world, torch, dist, 400, 200.0)
            out["serving"] = dict(serving, config=dict(SERVE_CONFIG, rate_hz=200.0))
            out["streamline_throughput"] = engine_throughput(frames, rank, torch)
            cb = cpu_baseline(x, q, starts, caps)
            out["cpu_baseline"] = {"value": cb["streamlines_per_s"], "unit": "streamlines/s",
                                   "cores": cb["cores"], "kind": "port",
                                   "pair_evals_per_s": cb["pair_evals_per_s"],
                                   "sample": cpu_sample_text(cb["lines"] // cb["passes"]) +
                                             f"; {cb['passes']} passes, {cb['seconds']:.1f} s"}
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def grid_frames(n_frames, seed=2024):
    """Batched volume workload: N ~ U[3,000, 40,000] charges (cube edge scaled
    to keep the density), grids of 11^3, 21^3 or 31^3 points at 0.1 A."""
    from pycpet_gb300.synth import volume_batch_frames

    return volume_batch_frames(n_frames, seed)


def grid_main(args, rank, world, dev, torch, dist):
    """--workload grid: field + potential of a frame batch in one descriptor-
    table launch each (FP32C), device-resident inputs, per-step events."""
    from pycpet_gb300 import _lib
    from pycpet_gb300.core import GridBatch

    frames = grid_frames(args.frames, seed=2024 + rank)
    gbs = [GridBatch(frames, kind=k, precision="fp32c", device=True, graph=True) for k in ("field", "esp")]
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        for gb in gbs:
            gb.run()
    ffma = max(_lib.measure_peak(0), _lib.measure_peak(3))  # FP32 pipe: FFMA or packed FFMA2
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        evs[k][0].record(stream)
        gbs[0].run()
        evs[k][1].record(stream)
        gbs[1].run()
        evs[k][2].record(stream)
        flush.fill_(k & 0xFF)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    _lib.check(_lib.lib().cpetgb_synchronize(stream.cuda_stream))
    f_ms = [e[0].elapsed_time(e[1]) for e in evs]
    e_ms = [e[1].elapsed_time(e[2]) for e in evs]
    pe = gbs[0].pair_evals
    total_s = (sum(f_ms) + sum(e_ms)) * 1e-3
    out = {"metric": METRIC, "value": 2 * pe * world * args.steps / total_s, "unit": "pair-evals/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": f"batched volume + volume_ESP, {args.frames} frames, FP32C, "
                                  "one descriptor-table launch per kind captured in a CUDA graph",
                      "pair_evals_per_kind": pe},
           "field_pair_evals_per_s": pe / (statistics.mean(f_ms) * 1e-3),
           "esp_pair_evals_per_s": pe / (statistics.mean(e_ms) * 1e-3),
           "roofline": {"bound": "fp32", "achieved": pe * FLOPS_PER_PAIR / (statistics.mean(f_ms) * 1e-3) / 1e12,
                        "peak": ffma / 1e12, "unit": "TFLOP/s",
                        "frac": pe * FLOPS_PER_PAIR / (statistics.mean(f_ms) * 1e-3) / ffma,
                        "traffic": None, "kernel": "grid_kernel (FP32C field)"}}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def engine_throughput(frames, rank, torch, n_req=100):
    """Streamline-only burst through the serving engine: n_req requests of
    500-1,500 lines (step 0.001 A, cap 6,000), all queued at once, on the
    10,000-charge frame and on the mix of 2,000-100,000-charge frames; the
    engine at one CTA per SM (half of every SM, the mixed-serving setting) and
    at two (whole SMs), beside one batched launch of the same lines
    (cpetgb_topo_batch).  Lines/s and pair evaluations/s from the step counts."""
    from dataclasses import replace

    from pycpet_gb300.core import TopoBatch
    from pycpet_gb300.serving import Request, Server

    out = {}
    for name, fids in (("10000_charges", [2]), ("2000-100000_charges", list(frames))):
        rng = np.random.default_rng(4242 + rank)
        reqs = []
        for i in range(n_req):
            f = int(fids[int(rng.integers(0, len(fids)))])
            L = int(rng.integers(500, 1501))
            reqs.append(Request("topo", f, 0.0, starts=rng.uniform(-1.5, 1.5, (L, 3)), n_iter=6000, step=0.001))
        tb = TopoBatch([{"x": frames[r.frame]["x"], "q": frames[r.frame]["q"], "starts": r.starts,
                         "n_iter": 6000, "step": 0.001, "half_dims": [1.5] * 3} for r in reqs],
                       precision="fp32c", device=True)
        res, steps = tb.run(return_steps=True)
        torch.cuda.synchronize()
        steps = steps.cpu().numpy()
        n_of = np.concatenate([np.full(len(r.starts), len(frames[r.frame]["q"]), np.int64) for r in reqs])
        pe = int(np.sum((np.maximum(steps, 2) + 2).astype(np.int64) * n_of))
        n_lines = len(steps)
        t0 = time.perf_counter()
        tb.run()
        torch.cuda.synchronize()
        t_batch = time.perf_counter() - t0
        row = {"requests": n_req, "lines": n_lines, "pair_evals": pe,
               "batch_launch": {"s": t_batch, "lines_per_s": n_lines / t_batch, "pair_evals_per_s": pe / t_batch}}
        ref = res.cpu().numpy()
        for cps in (1, 2):
            srv = Server(precision="fp32c", line_capacity=2_000_000, charge_capacity=400_000, max_requests=4096,
                         engine_ctas_per_sm=cps)
            for fid, fr in frames.items():
                srv.add_frame(fid, fr["x"], fr["q"])
            srv.run([Request("topo", r.frame, 0.0, starts=r.starts[:64], n_iter=6000, step=0.001) for r in reqs[:8]])
            burst = [replace(r, result=None, t_start=None, t_done=None, _rid=-1) for r in reqs]
            t0 = time.perf_counter()
            srv.run(burst)
            t = time.perf_counter() - t0
            srv.close()
            same = bool(np.array_equal(np.concatenate([r.result for r in burst]), ref))
            row[f"engine_{cps}_cta_per_sm"] = {"s": t, "lines_per_s": n_lines / t, "pair_evals_per_s": pe / t,
                                               "identical_to_batch": same}
        out[name] = row
    return out


SERVE_FRAME_SIZES = [2000, 5000, 10000, 20000, 40000, 60000, 80000, 100000]


def serve_measure(rank, world, torch, dist, n_requests, rate, fp64_requests=24):
    """Serving loop (config: Poisson arrivals mixing point_field 1-64 points,
    volume / volume_ESP 11^3-51^3 and topo requests on resident frames of
    2,000-100,000 charges; continuous batching): p50/p99 latency per kind for
    FP32C at `rate` requests/s and FP64 at a 50x lower rate.  Streamline
    requests carry 10-500 lines (the config's 10^4-10^6 would offer ~10^3 times
    the device's capacity at 200 requests/s and measure only queueing)."""
    from pycpet_gb300.serving import Server, latency_stats, synthetic_schedule
    from pycpet_gb300.synth import make_frame

    frames = {i: make_frame(n, 600 + i + 100 * rank) for i, n in enumerate(SERVE_FRAME_SIZES)}
    results = {}
    # FP64 runs a smaller mix at a lower rate: its pipe is ~75x narrower on this GPU
    for prec, n_req, r_hz in (("fp32c", n_requests, rate), ("fp64", fp64_requests, rate / 50)):
        lines = (10, 500)
        srv = Server(precision=prec, line_capacity=4_000_000, charge_capacity=400_000, max_requests=8192)
        for fid, fr in frames.items():
            srv.add_frame(fid, fr["x"], fr["q"])
        warm = synthetic_schedule(list(frames), 8, 1e6, seed=99, topo_lines=(100, 1000))
        srv.run(warm)
        sched = synthetic_schedule(list(frames), n_req, r_hz, seed=rank, topo_lines=lines)
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        srv.run(sched)
        wall = time.perf_counter() - t0
        print(f"serve {prec}: {n_req} requests in {wall:.2f} s", file=sys.stderr, flush=True)
        pe = 0
        for r in sched:
            n = len(frames[r.frame]["q"])
            pe += (len(r.points) if r.points is not None else 0) * n
        results[prec] = {"requests": n_req, "rate_hz": r_hz, "topo_lines": list(lines), "wall_s": wall,
                         "requests_per_s": n_req / wall, "completed": sum(r.status == "done" for r in sched),
                         "grid_pair_evals": pe, "latency": latency_stats(sched),
                         "max_topo_requests_in_flight": srv.max_topo_inflight}
        srv.close()
    return frames, results


SERVE_CONFIG = {"workload": "serving: Poisson arrivals, point_field 1-64 points, volume / volume_ESP "
                            "11^3-51^3, topo 10-500 lines (step 0.001 A, cap 6,000), frames of "
                            "2,000-100,000 charges resident on the device",
                "admission": "80% HBM budget; engine line store 4e6 lines"}


def serve_main(args, rank, world, dev, torch, dist):
    """--workload serve: the serving loop at --rate requests/s (serve_measure)
    and the engine's streamline throughput (engine_throughput)."""
    out = {"metric": METRIC, "unit": "requests/s", "n_gpus": world, "steps": 1, "warmup": args.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)"}
    frames, results = serve_measure(rank, world, torch, dist, args.requests, args.rate)
    out["streamline_throughput"] = engine_throughput(frames, rank, torch)
    out["value"] = results["fp32c"]["requests_per_s"]
    out["ms_per_step"] = 1e3 * results["fp32c"]["wall_s"]
    out["config"] = dict(SERVE_CONFIG, rate_hz=args.rate)
    out["serving"] = results
    out["latency_ms"] = {"p50": results["fp32c"]["latency"]["all"]["p50_ms"],
                         "p99": results["fp32c"]["latency"]["all"]["p99_ms"]}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def cluster_inputs(rank, n_hist=4096, n_fields=1024):
    """Synthetic trajectory-scale clustering inputs: n_hist topology histograms
    of 20 x 20 bins (rows normalised to 1, about a third of the bins empty) and
    n_fields vector fields on a 21^3 grid."""
    rng = np.random.default_rng(7070 + rank)
    base = rng.gamma(1.0, 1.0, 400) * (rng.random(400) < 0.7)
    h = base * rng.lognormal(0.0, 0.3, (n_hist, 400))
    h /= h.sum(axis=1, keepdims=True)
    fld = rng.normal(0.0, 1.0, (9261, 3)) + rng.normal(0.0, 0.2, (n_fields, 9261, 3))
    return h, fld


def cluster_main(args, rank, world, dev, torch, dist):
    """--workload cluster: the chi-square distance matrix of 4,096 topology
    histograms (20 x 20 bins) and the field distance matrix of 1,024 vector
    fields on a 21^3 grid, device-resident (FP32C and FP64), against the
    oracle's C restatement of construct_distance_matrix(_volume) on all host
    cores over a sample of rows."""
    from pycpet_gb300 import _lib, chi2_distance_matrix, field_distance_matrix

    h, fld = cluster_inputs(rank)
    dh, df = torch.from_numpy(h).to(dev), torch.from_numpy(fld).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    mufu = _lib.measure_peak(2)

    def timed(fn, arg, prec):
        for _ in range(args.warmup):
            fn(arg, prec)
        torch.cuda.synchronize()
        ts = []
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn(arg, prec)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return statistics.median(ts)

    n_h, n_f = h.shape[0], fld.shape[0]
    terms_h = n_h * (n_h - 1) // 2 * h.shape[1]
    terms_f = n_f * (n_f - 1) // 2 * fld.shape[1]
    res = {}
    for prec in ("fp32c", "fp64"):
        th = timed(chi2_distance_matrix, dh, prec)
        tf = timed(field_distance_matrix, df, prec)
        res[prec] = {"chi2_terms_per_s": terms_h / th, "chi2_ms": th * 1e3,
                     "field_terms_per_s": terms_f / tf, "field_ms": tf * 1e3}
    d32 = chi2_distance_matrix(dh[:512], "fp32c").cpu().numpy()
    d64 = chi2_distance_matrix(dh[:512], "fp64").cpu().numpy()
    err = float(np.max(np.abs(d32 - d64)) / np.max(d64))
    out = {"metric": "chi-square distance-matrix terms/s (histogram pairs x bins)",
           "value": res["fp32c"]["chi2_terms_per_s"], "unit": "terms/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["fp32c"]["chi2_ms"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": f"construct_distance_matrix of {n_h} histograms x 400 bins; "
                                  f"construct_distance_matrix_volume of {n_f} fields x 9,261 points",
                      "l2": "flushed between timed steps"},
           "forms": res, "fp32c_vs_fp64_max_rel_err_512": err,
           "roofline": {"bound": "mufu", "achieved": res["fp32c"]["chi2_terms_per_s"] / 1e12, "peak": mufu / 1e12,
                        "unit": "Tterm/s", "frac": res["fp32c"]["chi2_terms_per_s"] / mufu,
                        "note": "one MUFU reciprocal per chi-square term; peak = MUFU rsqrt rate measured now"}}
    if rank == 0 and world == 1:
        from oracle import oracle

        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        oracle.chi2_matrix_f64(h[:768], threads=threads)
        t1 = time.perf_counter()
        oracle.field_matrix_f64(fld[:128], threads=threads)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"value": 768 * 767 // 2 * 400 / (t1 - t0), "unit": "terms/s", "cores": threads,
                               "kind": "port", "field_terms_per_s": 128 * 127 // 2 * 9261 / (t2 - t1),
                               "sample": "first 768 histograms / first 128 fields, oracle C restatement (FP64)"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def dat_main(args, rank, world, dev, torch, dist):
    """--workload dat: one 51^3-point volume of a 20,000-charge frame, end to
    end as the reference's run_volume does it (CPET/source/CPET.py:129-170):
    the field on the grid (compute_field_on_grid) and the .dat file
    (save_numpy_as_dat, CPET/utils/io.py:50-109) with its body formatted on
    the GPU; beside it numpy.savetxt of the same rows on the host, the
    reference's writer."""
    import io as _io

    from pycpet_gb300 import calculator as calc
    from pycpet_gb300.synth import make_frame

    fr = make_frame(20000, seed=21 + rank)
    g = np.linspace(-2.5, 2.5, 51)
    mesh = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).astype(np.float32)
    meta = {"dimensions": np.array([2.5] * 3, np.float32), "num_steps": [51, 51, 51],
            "transformation_matrix": np.eye(3, dtype=np.float32), "center": np.zeros(3, np.float32)}
    x32, q32 = fr["x"].astype(np.float32), fr["q"].astype(np.float32).reshape(-1, 1)
    tmp = tempfile.mkdtemp()
    path = os.path.join(tmp, "frame_efield.dat")

    def step():
        vol = calc.compute_field_on_grid(mesh, x32, q32)
        calc.save_numpy_as_dat(meta, vol, path)
        return vol

    for _ in range(args.warmup):
        vol = step()
    ts, tf = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        vol = calc.compute_field_on_grid(mesh, x32, q32)
        t1 = time.perf_counter()
        calc.save_numpy_as_dat(meta, vol, path)
        t2 = time.perf_counter()
        ts.append(t2 - t0)
        tf.append(t2 - t1)
    sink = _io.BytesIO()
    t0 = time.perf_counter()
    np.savetxt(sink, vol, fmt="%.3f")
    t_np = time.perf_counter() - t0
    body = calc.format_fixed3(vol)
    assert body == sink.getvalue(), "GPU text differs from numpy.savetxt"
    rows = vol.shape[0]
    t = statistics.median(ts)
    out = {"metric": "volume frames/s end to end (field + .dat file)", "value": 1.0 / t, "unit": "frames/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": "51^3 volume of a 20,000-charge frame: compute_field_on_grid + save_numpy_as_dat",
                      "rows": rows, "bytes": len(body)},
           "writer_ms": statistics.median(tf) * 1e3, "writer_rows_per_s": rows / statistics.median(tf),
           "numpy_savetxt_ms": t_np * 1e3, "numpy_savetxt_rows_per_s": rows / t_np,
           "writer_speedup_vs_numpy": t_np / statistics.median(tf), "bytes_identical": True,
           "e2e": {"value": 1.0 / t, "unit": "frames/s", "h2d_bytes_per_step": int(mesh.nbytes + x32.nbytes + q32.nbytes),
                   "d2h_bytes_per_step": int(vol.nbytes + len(body))}}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def prep_main(args, rank, world, dev, torch, dist):
    """--workload prep: the calculator's frame preparation for a 100,000-atom
    frame in residues of 4-19 atoms (residue radius filter 25 A, rotation,
    box filter, box shift; CPET/source/calculator.py:239-251, 341-371) through
    prepare_frame with host buffers, against a vectorised numpy restatement of
    the same rules on the host."""
    from pycpet_gb300.core import prepare_frame

    rng = np.random.default_rng(51 + rank)
    n = 100000
    x = rng.uniform(-40.0, 40.0, (n, 3))
    q = rng.normal(0.0, 0.4, n)
    sizes = rng.integers(4, 20, n // 4)
    resnum = np.repeat(np.arange(len(sizes)), sizes)[:n].astype(np.int32)
    resid = (resnum % 20).astype(np.int32)
    center = np.array([1.0, -2.0, 0.5])
    T = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    inv = np.linalg.inv(T)
    half, shift = np.array([1.5, 1.5, 1.5]), np.array([0.1, 0.0, -0.1])
    run = lambda: prepare_frame(x, q, center, inv_basis=inv, radius=25.0, resid=resid, resnum=resnum,
                                box_half=half, box_shift=shift)
    for _ in range(args.warmup):
        xo, qo = run()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        xo, qo = run()
        ts.append(time.perf_counter() - t0)

    def host():
        start = np.ones(n, bool)
        start[1:] = (resid[1:] != resid[:-1]) | (resnum[1:] != resnum[:-1])
        runs = np.cumsum(start) - 1
        near = np.linalg.norm(x - center, axis=1) < 25.0
        keep_run = np.zeros(runs[-1] + 1, bool)
        keep_run[runs[near]] = True
        k = keep_run[runs]
        xr = (x[k] - center) @ inv
        inside = np.all((xr - center > -half) & (xr - center < half), axis=1)
        return xr[~inside] - shift, q[k][~inside]

    th = []
    for _ in range(3):
        t0 = time.perf_counter()
        xh, qh = host()
        th.append(time.perf_counter() - t0)
    assert np.array_equal(qh, qo) and np.abs(xh - xo).max() < 1e-12
    t = statistics.median(ts)
    out = {"metric": "frames prepared/s (100,000 atoms, radius + box filters, rotation)", "value": 1.0 / t,
           "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)",
           "config": {"workload": "prepare_frame, 100,000 atoms, residues of 4-19 atoms, radius 25 A",
                      "kept_atoms": int(len(qo))},
           "e2e": {"value": 1.0 / t, "unit": "frames/s", "h2d_bytes_per_step": int(x.nbytes + q.nbytes + 8 * n),
                   "d2h_bytes_per_step": int(xo.nbytes + qo.nbytes)},
           "cpu_baseline": {"value": 1.0 / statistics.median(th), "unit": "frames/s", "cores": 1, "kind": "port",
                            "sample": "the whole frame, vectorised numpy restatement of the same rules"}}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


DIPOLE_FLOPS = 29  # 3 sub, r^2 5, r^-2 r^-3 r^-5 3, dot 5, w 1, 2 x 3 fma 12


def dipole_main(args, rank, world, dev, torch, dist):
    """--workload topo-dipole: streamlines through 8,000 point dipoles
    (thread_operation_dipole; positions as the charge frames, moments
    ~ N(0, 0.3)), --lines seeded start points (default 20,000) in the
    1.5 A box, step 0.001 A, cap 6,000, FP32C device-resident; FP64 and the
    CPU restatement on samples of the same lines."""
    from pycpet_gb300 import _lib, topo_dipole_lines
    from pycpet_gb300.synth import make_dipole_frame, random_start_points

    n_lines = args.lines if args.lines != N_LINES else 20000
    fr = make_dipole_frame(8000, seed=11 + 1000 * rank)
    starts = random_start_points(n_lines, [HALF] * 3, seed=12 + 1000 * rank)
    caps = np.full(n_lines, CAP, np.int32)
    d = [torch.from_numpy(a).to(dev) for a in (starts, caps, fr["x"], fr["mu"])]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    res, steps = topo_dipole_lines(*d[:2], d[2], d[3], STEP, [HALF] * 3, precision="fp32c", return_steps=True)
    torch.cuda.synchronize()
    pe = pair_evals(steps.cpu().numpy(), 8000)
    for _ in range(args.warmup):
        topo_dipole_lines(*d[:2], d[2], d[3], STEP, [HALF] * 3, precision="fp32c")
    ffma = _lib.measure_peak(0)
    torch.cuda.synchronize()
    ts = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        topo_dipole_lines(*d[:2], d[2], d[3], STEP, [HALF] * 3, precision="fp32c")
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = statistics.median(ts)
    sub = slice(0, 1024)
    t0 = time.perf_counter()
    r64, s64 = topo_dipole_lines(starts[sub], caps[sub], fr["x"], fr["mu"], STEP, [HALF] * 3, precision="fp64",
                                 return_steps=True)
    t64 = time.perf_counter() - t0
    r32 = res.cpu().numpy()[sub]
    out = {"metric": "dipole streamlines/s (thread_operation_dipole)", "value": n_lines / t, "unit": "streamlines/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": f"8,000 point dipoles, {n_lines} lines, half-width 1.5 A, step 0.001 A, cap 6,000",
                      "l2": "flushed between timed steps"},
           "pair_evals_per_s": pe / t,
           "roofline": {"bound": "fp32", "achieved": pe * DIPOLE_FLOPS / t / 1e12, "peak": ffma / 1e12,
                        "unit": "TFLOP/s", "frac": pe * DIPOLE_FLOPS / t / ffma,
                        "work": f"{DIPOLE_FLOPS} flop per dipole term (21 FP32-pipe operations + 1 MUFU)"},
           "fp64_first_1024": {"streamlines_per_s": 1024 / t64,
                               "pair_evals_per_s": pair_evals(s64, 8000) / t64},
           "fp32c_vs_fp64_first_1024": {"dist_max_A": float(np.abs(r32[:, 0] - r64[:, 0]).max()),
                                        "curv_rel_p50": float(np.median(np.abs(r32[:, 1] - r64[:, 1]) /
                                                                        np.abs(r64[:, 1]))),
                                        "step_count_mismatch_frac": float(np.mean(steps.cpu().numpy()[sub] != s64))}}
    if rank == 0 and world == 1:
        from oracle import oracle

        threads = os.cpu_count() or 1
        n_cpu = 4 * threads
        t0 = time.perf_counter()
        _, _, sc = oracle.topo_lines_dipole(starts[:n_cpu], caps[:n_cpu], fr["x"], fr["mu"], STEP, [HALF] * 3,
                                            f32=True, threads=threads)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n_cpu / tc, "unit": "streamlines/s", "cores": threads, "kind": "port",
                               "pair_evals_per_s": pair_evals(sc, 8000) / tc,
                               "sample": f"first {n_cpu} lines, the reference's float arithmetic restated"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def topo_batch_measure(rank, world, dev, torch, dist, n_frames, line_scale, steps, warmup):
    """Batched topo (config: frames of 5,000-20,000 charges, density kept,
    100,000-1,000,000 lines per frame scaled by `line_scale`, half-width 1.5 A,
    step 0.001 A, cap 6,000): all frames in one persistent launch (FP32C).
    Returns a dict of streamlines/s, pair evaluations/s and per-launch times."""
    from pycpet_gb300 import _lib
    from pycpet_gb300.core import TopoBatch
    from pycpet_gb300.synth import make_frame, random_start_points

    rng = np.random.default_rng(3030 + rank)
    frames = []
    for f in range(n_frames):
        n = int(rng.integers(5000, 20001))
        L = max(1, int(rng.integers(100_000, 1_000_001) * line_scale))
        fr = make_frame(n, seed=7000 + f + 100 * rank)
        frames.append({"x": fr["x"], "q": fr["q"], "starts": random_start_points(L, [HALF] * 3, 8000 + f),
                       "n_iter": CAP, "step": STEP, "half_dims": [HALF] * 3})
    tb = TopoBatch(frames, precision="fp32c", device=True)
    res, stp = tb.run(return_steps=True)
    torch.cuda.synchronize()
    stp = stp.cpu().numpy()
    pe = sum(pair_evals(s_, len(fr["q"])) for fr, s_ in zip(frames, tb.split(stp)))
    for _ in range(warmup - 1):
        tb.run()
    stream = torch.cuda.current_stream(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    for e0, e1 in evs:
        e0.record(stream)
        tb.run()
        e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    _lib.check(_lib.lib().cpetgb_synchronize(stream.cuda_stream))
    ms = [a.elapsed_time(b) for a, b in evs]
    total_s = sum(ms) * 1e-3
    return {"frames": n_frames, "line_scale": line_scale, "n_lines": tb.n_lines, "steps": steps,
            "streamlines_per_s": tb.n_lines * steps / total_s, "pair_evals_per_s": pe * steps / total_s,
            "ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99))},
            "workload": f"batched topo, {n_frames} frames of 5,000-20,000 charges, "
                        f"{line_scale:g} x (100,000-1,000,000) lines per frame, one launch"}


def topo_batch_main(args, rank, world, dev, torch, dist):
    """--workload topo-batch: topo_batch_measure with --frames (default 32) and --line-scale."""
    n_frames = args.frames if args.frames != 64 else 32
    r = topo_batch_measure(rank, world, dev, torch, dist, n_frames, args.line_scale, args.steps, args.warmup)
    out = {"metric": METRIC, "value": r["streamlines_per_s"] * world, "unit": "streamlines/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": r["ms"]["p50"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": r["workload"], "n_lines": r["n_lines"], "line_scale": args.line_scale},
           "precision": "fp32c",
           "pair_evals_per_s": r["pair_evals_per_s"] * world,
           "latency_ms": r["ms"]}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def extras(d_starts, d_caps, d_x, d_q, torch, topo_lines, GridBatch, dfma):
    """FP64 plain form on a subset of the same lines (same subset in FP32C for
    the speed-up), and the batched volume/ESP grid workload in both forms."""
    from pycpet_gb300 import set_field_refinement, topo_hist2d

    n_sub = 16384
    res, outs = {}, {}
    for prec in ("fp32c", "fp64"):
        topo_lines(d_starts[:1024], d_caps[:1024], d_x, d_q, STEP, [HALF] * 3, precision=prec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r, ends, steps = topo_lines(d_starts[:n_sub], d_caps[:n_sub], d_x, d_q, STEP, [HALF] * 3,
                                    precision=prec, return_ends=True, return_steps=True)
        e1.record()
        torch.cuda.synchronize()
        s = e0.elapsed_time(e1) * 1e-3
        outs[prec] = (r.cpu().numpy(), ends.cpu().numpy(), steps.cpu().numpy())
        res[prec] = {"streamlines_per_s": n_sub / s,
                     "pair_evals_per_s": pair_evals(outs[prec][2], N_CHARGES) / s, "seconds": s}
    (r32, e32, s32), (r64, e64, s64) = outs["fp32c"], outs["fp64"]
    cmax = float(np.nanmax(r64[:, 1]))
    h32 = topo_hist2d(r32, bins=(20, 20), range=((0.0, 5.2), (0.0, cmax))).astype(np.float64)
    h64 = topo_hist2d(r64, bins=(20, 20), range=((0.0, 5.2), (0.0, cmax))).astype(np.float64)
    end_err = np.linalg.norm(e32 - e64, axis=1)
    curv_rel = np.abs(r32[:, 1] - r64[:, 1]) / np.maximum(np.abs(r64[:, 1]), 1e-300)
    topo_cmp = {"sample": f"first {n_sub} lines", "fp32c": res["fp32c"], "fp64": res["fp64"],
                "speedup_fp32c_vs_fp64": res["fp64"]["seconds"] / res["fp32c"]["seconds"],
                "fp64_roofline": {"achieved_tflops": res["fp64"]["pair_evals_per_s"] * FLOPS_PER_PAIR / 1e12,
                                  "peak_tflops": dfma / 1e12,
                                  "frac": res["fp64"]["pair_evals_per_s"] * FLOPS_PER_PAIR / dfma,
                                  "peak_source": "DFMA throughput measured in this run"},
                "error_fp32c_vs_fp64": {
                    "endpoint_A": {"p50": float(np.median(end_err)), "p99": float(np.quantile(end_err, 0.99)),
                                   "max": float(end_err.max())},
                    "distance_A_max": float(np.abs(r32[:, 0] - r64[:, 0]).max()),
                    "curvature_rel": {"p50": float(np.median(curv_rel)), "p99": float(np.quantile(curv_rel, 0.99)),
                                      "max": float(curv_rel.max())},
                    "step_count_mismatch_frac": float(np.mean(s32 != s64)),
                    "histogram_L1": float(np.abs(h32 / h32.sum() - h64 / h64.sum()).sum()),
                    "histogram_range": [[0.0, 5.2], [0.0, cmax]]}}

    # batched volume + volume_ESP: 64 frames, N ~ U[3k, 40k], grids 11^3/21^3/31^3
    frames = grid_frames(64)
    grid = {"pair_evals_per_kind": int(sum(len(p) * len(qq) for p, _, qq in frames))}
    def timed_plan(kind, prec):
        """A CUDA-graph plan of the batch (frame table, pack, grid, reduction
        and refinement kernels), replayed once to warm up and once timed."""
        gb = GridBatch(frames, kind=kind, precision=prec, device=True, graph=True)
        gb.run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = gb.run()
        e1.record()
        torch.cuda.synchronize()
        return gb, out.cpu().numpy().copy(), e0.elapsed_time(e1) * 1e-3

    for kind in ("field", "esp"):
        vals = {}
        for prec in ("fp32c", "fp64"):
            gb, out, s = timed_plan(kind, prec)
            grid[f"{kind}_{prec}"] = {"pair_evals_per_s": gb.pair_evals / s, "ms": s * 1e3,
                                      "launch": "CUDA-graph plan (cpetgb_grid_plan_create) replay"}
            vals[prec] = [o.copy() for o in gb.split(out)]
            del gb
            if kind == "field" and prec == "fp32c":
                # the same launch without the FP64 refinement of ill-conditioned points
                tau = set_field_refinement(0.0)
                gb, raw, s0 = timed_plan(kind, prec)
                del gb
                set_field_refinement(tau)
                refined = int(np.sum(np.any(raw != out, axis=1)))
                grid["field_fp32c"]["refinement"] = {
                    "threshold": tau, "points_refined": refined, "ms_without": s0 * 1e3,
                    "pair_evals_per_s_without": grid["pair_evals_per_kind"] / s0,
                    "rule": "points with |E| < threshold x the frame's median |E| recomputed in "
                            "double-float arithmetic (about 1e-12 per term)"}
        # FP32C error against the FP64 form (itself within 1e-11 of the CPU FP64 oracle), per frame
        worst_rel, worst_norm, rels = 0.0, 0.0, []
        for a, b in zip(vals["fp32c"], vals["fp64"]):
            nb = np.linalg.norm(b, axis=1)
            err = np.linalg.norm(a - b, axis=1)
            mask = nb >= 1e-6 * np.median(nb)          # tiny |ref| points are flagged, not scored
            rel = err[mask] / nb[mask]
            rels.append(rel)
            worst_rel = max(worst_rel, float(rel.max()))
            worst_norm = max(worst_norm, float(err.max() / nb.max()))
        rels = np.concatenate(rels)
        grid[f"{kind}_fp32c_error"] = {
            "max_rel_per_point": worst_rel, "p999_rel_per_point": float(np.quantile(rels, 0.999)),
            "frac_points_above_1e-5": float(np.mean(rels > 1e-5)),
            "max_normwise_rel": worst_norm, "frames": len(frames), "points": int(rels.size),
            "rule": "per point |dE|/|E_ref| (points with |E_ref| < 1e-6 * frame median flagged); normwise "
                    "= max|dE| / max|E_ref| per frame; reference = the FP64 form"}
    grid["workload"] = ("64 frames, 3,000-40,000 charges, 11^3/21^3/31^3 grids, one descriptor-table "
                        "launch captured in a CUDA graph")
    return {"topo_fp64_vs_fp32c": topo_cmp, "grid_batch": grid}


if __name__ == "__main__":
    main()
