"""Autotuner for the library's tile shapes.

The library picks a kernel variant per (operation, precision, class, size
bucket) from a table (see ``cpetgb_tune_*`` in include/cpetgb.h):

* grid sums (op 0): points per thread {4, 8} x work items per SM {4, 8, 16, 32, 64}
  (variants 0-9) and {128, 256} (variants 10-13);
  class = field / potential; size = pair evaluations of the launch;
* streamlines (op 1): line slots per warp {4, 2}; class = charges resident
  in shared memory or streamed from L2; size = number of lines.

``tune_grid`` / ``tune_topo`` time every candidate on the caller's actual
batch (CUDA events, device-resident inputs) and store the fastest.
``tune_default`` tunes a set of representative shapes.  ``save`` / ``load``
keep the table as JSON, one file per GPU model; a table measured on a GB300
ships with the package (``tuned/``) and is loaded by ``load_default()``.
"""
from __future__ import annotations

import json
import os

import numpy as np

from ._lib import ESP, FIELD, check, lib
from .core import GridBatch, TopoBatch, precision_code

OP_GRID, OP_TOPO = 0, 1
_TABLE: dict[int, int] = {}
PKG_TUNED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned")


def _gpu_name() -> str:
    import torch

    return torch.cuda.get_device_name(torch.cuda.current_device())


def _slug(name: str) -> str:
    return "".join(ch if ch.isalnum() else "_" for ch in name).strip("_").lower()


def cache_path(gpu_name: str | None = None) -> str:
    env = os.environ.get("CPETGB_TUNE_CACHE")
    if env:
        return env
    base = os.path.join(os.path.expanduser("~"), ".cache", "pycpet_gb300")
    return os.path.join(base, f"tune-{_slug(gpu_name or _gpu_name())}.json")


def set_variant(key: int, variant: int) -> None:
    check(lib().cpetgb_tune_set(int(key), int(variant)))
    if variant < 0:
        _TABLE.pop(int(key), None)
    else:
        _TABLE[int(key)] = int(variant)


def key(op: int, precision, cls: int, size: float) -> int:
    k = lib().cpetgb_tune_key(op, precision_code(precision), int(cls), float(size))
    if k < 0:
        check(k)
    return k


def save(path: str | None = None) -> str:
    path = path or cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    with open(path, "w") as fh:
        json.dump({"gpu": _gpu_name(), "table": {str(k): v for k, v in sorted(_TABLE.items())}}, fh, indent=1)
    return path


def load(path: str | None = None) -> int:
    """Loads a saved table into the library; returns the number of entries."""
    path = path or cache_path()
    if not os.path.exists(path):
        return 0
    with open(path) as fh:
        data = json.load(fh)
    for k, v in data.get("table", {}).items():
        set_variant(int(k), int(v))
    return len(data.get("table", {}))


def load_default() -> int:
    """The user's cache for this GPU if present, else the shipped table for it."""
    n = load()
    if n:
        return n
    return load(os.path.join(PKG_TUNED, f"{_slug(_gpu_name())}.json"))


def _time_ms(run, reps: int) -> float:
    import torch

    run()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune_grid(frames, kind="field", precision="fp32c", reps=3, verbose=False):
    """Times the grid variants on `frames` ((points, x, q) per frame); keeps the
    fastest.  Each variant is timed as a CUDA-graph plan replay, so the host's
    planning of the work items (which grows with their number) stays out of the
    device time being compared."""
    gb = GridBatch(frames, kind=kind, precision=precision, device=True)
    k = key(OP_GRID, precision, FIELD if kind == "field" else ESP, gb.pair_evals)
    n_var = lib().cpetgb_tune_variants(OP_GRID)
    times = []
    for v in range(n_var):
        set_variant(k, v)
        plan = GridBatch(frames, kind=kind, precision=precision, device=True, graph=True)
        times.append(_time_ms(plan.run, reps))
        del plan
    best = int(np.argmin(times))
    set_variant(k, best)
    if verbose:
        print(f"grid {kind} {precision} pairs={gb.pair_evals:.3g} key={k}: " +
              " ".join(f"v{v}={t:.3f}ms" for v, t in enumerate(times)) + f" -> v{best}")
    return best, times


def tune_topo(frames, precision="fp32c", reps=2, verbose=False):
    """Times the streamline variants on `frames` (TopoBatch frame dicts); keeps the fastest."""
    tb = TopoBatch(frames, precision=precision, device=True)
    from ._lib import FP32C

    resident_limit = lib().cpetgb_topo_resident_limit(precision_code(precision), 0)
    check(min(resident_limit, 0))
    pad = 64  # FP32C streamline frames are padded to a multiple of 64 charges
    n_max = max(len(np.asarray(fr["q"]).reshape(-1)) for fr in frames)
    cls = 1 if (precision_code(precision) == FP32C and -(-n_max // pad) * pad <= resident_limit) else 0
    k = key(OP_TOPO, precision, cls, tb.n_lines)
    n_var = lib().cpetgb_tune_variants(OP_TOPO)
    times = []
    for v in range(n_var):
        set_variant(k, v)
        times.append(_time_ms(tb.run, reps))
    best = int(np.argmin(times))
    set_variant(k, best)
    if verbose:
        print(f"topo {precision} lines={tb.n_lines} class={cls} key={k}: " +
              " ".join(f"v{v}={t:.3f}ms" for v, t in enumerate(times)) + f" -> v{best}")
    return best, times


def tune_default(verbose=True, quick=False):
    """Tunes representative shapes: single volumes and point fields, frame
    batches, and streamline sets of several sizes (FP32C)."""
    from .synth import make_frame, random_start_points

    results = {}

    def grid_frames(specs):
        out = []
        for i, (n, half, n_pts) in enumerate(specs):
            fr = make_frame(n, 900 + i)
            if n_pts is None:
                g = np.linspace(-half, half, int(round(2 * half / 0.1)) + 1)
                pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
            else:
                pts = np.random.default_rng(i).uniform(-half, half, (n_pts, 3))
            out.append((pts, fr["x"], fr["q"]))
        return out

    grid_cases = [
        [(5000, 1.0, None)],                                   # one 21^3 volume, 5,000 charges
        [(100000, 0.5, 64)],                                   # a 64-point request on a large frame
        [(20000, 1.5, None)] * 4,                              # a few 31^3 volumes
        [(int(n), h, None) for n, h in zip(np.linspace(3000, 40000, 16 if quick else 64),
                                           [0.5, 1.0, 1.5] * 22)],  # frame batch
    ]
    rng = np.random.default_rng(2024)  # 48 frames of random sizes: the size bucket below
    grid_cases.append([(int(n), float(h), None) for n, h in zip(rng.integers(3000, 40001, 48),
                                                                rng.choice([0.5, 1.0, 1.5], 48))])
    for case in grid_cases:
        frames = grid_frames(case)
        for kind in ("field", "esp"):
            results[f"grid-{kind}-{len(case)}x{case[0][0]}"] = tune_grid(frames, kind, verbose=verbose)
    topo_cases = [(8000, 2000), (8000, 20000), (8000, 100000), (16000, 20000), (2000, 5000)]
    if quick:
        topo_cases = topo_cases[:3]
    for n, L in topo_cases:
        fr = make_frame(n, 950)
        frames = [{"x": fr["x"], "q": fr["q"], "starts": random_start_points(L, [1.5] * 3, 951),
                   "n_iter": 6000, "step": 0.001, "half_dims": [1.5] * 3}]
        results[f"topo-{n}x{L}"] = tune_topo(frames, verbose=verbose)
    return results


if __name__ == "__main__":
    import sys

    from .build import build_library

    build_library()
    tune_default(quick="--quick" in sys.argv)
    print("saved", save(sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else None))
