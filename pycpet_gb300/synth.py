"""Seeded synthetic frames with the shapes and value distributions of the
benchmark workloads (no protein files ship with the benchmarks).

A frame is a set of point charges already expressed in the box frame (centre at
the origin, axes from three seeded atoms), exactly what PyCPET's ``calculator``
holds in ``self.x`` / ``self.Q`` after its rotation step
(CPET/source/calculator.py:341-346):

* positions uniform in a cube of edge 50 A (5,000 charges) scaled as
  50 * (N/5000)^(1/3) A for other N, i.e. a density of 0.04 charges / A^3;
* a minimum pair separation of 1.0 A (rejection sampling with a k-d tree);
* no charge within 2.0 A of the box centre;
* partial charges ~ N(0, 0.4) clipped to +-1, then shifted by one constant so
  the net charge is the nearest integer.

All randomness comes from ``numpy.random.default_rng(seed)`` so the same frame
is produced on every machine.
"""
from __future__ import annotations

import numpy as np

from .calculator import box_transformation


def cube_edge(n_charges: int) -> float:
    return 50.0 * (n_charges / 5000.0) ** (1.0 / 3.0)


def _sample_positions(rng, n, edge, min_sep, exclude_r):
    from scipy.spatial import cKDTree

    accepted = np.empty((0, 3))
    half = edge / 2.0
    while len(accepted) < n:
        need = n - len(accepted)
        cand = rng.uniform(-half, half, size=(int(need * 1.3) + 16, 3))
        cand = cand[np.linalg.norm(cand, axis=1) >= exclude_r]
        if len(accepted):
            d, _ = cKDTree(accepted).query(cand, k=1)
            cand = cand[d >= min_sep]
        # resolve conflicts inside the batch: keep the earlier candidate of each pair
        if len(cand) > 1:
            pairs = cKDTree(cand).query_pairs(min_sep, output_type="ndarray")
            if len(pairs):
                drop = np.zeros(len(cand), bool)
                for a, b in pairs[np.argsort(pairs[:, 1], kind="stable")]:
                    if not drop[a]:
                        drop[b] = True
                cand = cand[~drop]
        accepted = np.concatenate([accepted, cand[:need]])
    return accepted


def make_charges(n_charges: int, seed: int, edge: float | None = None, min_sep: float = 1.0,
                 exclude_r: float = 2.0, sigma: float = 0.4):
    """Returns (x (N,3) float64, q (N,) float64) in the lab frame, centre at origin."""
    rng = np.random.default_rng(seed)
    edge = cube_edge(n_charges) if edge is None else edge
    x = _sample_positions(rng, n_charges, edge, min_sep, exclude_r)
    q = np.clip(rng.normal(0.0, sigma, n_charges), -1.0, 1.0)
    q = q + (np.round(q.sum()) - q.sum()) / n_charges
    return x, q


def make_frame(n_charges: int, seed: int, edge: float | None = None):
    """Charges rotated into the box frame built from three seeded atoms.

    Returns dict(x=(N,3) f64, q=(N,) f64, T=(3,3) box basis, seed=seed).
    """
    x, q = make_charges(n_charges, seed, edge)
    rng = np.random.default_rng(seed + 7919)
    a, b = rng.choice(n_charges, size=2, replace=False)
    T = box_transformation(np.zeros(3), x[a], x[b])
    x_local = x @ np.linalg.inv(T)
    return {"x": np.ascontiguousarray(x_local), "q": q, "T": T, "seed": seed}


def random_start_points(n_lines: int, half_widths, seed: int):
    """Seeded uniform start points inside the box (the 'random' initializer,
    CPET/utils/calculator.py:155-159, with a seeded generator)."""
    rng = np.random.default_rng(seed)
    hw = np.asarray(half_widths, dtype=np.float64)
    return np.column_stack([rng.uniform(-hw[k], hw[k], n_lines) for k in range(3)])


def make_dipole_frame(n_dipoles: int, seed: int, sigma: float = 0.3):
    """Point dipoles for the dipole streamline path: positions as make_frame's
    charges (density 0.04 / A^3, >= 1 A apart, none within 2 A of the centre,
    box frame), moments with components ~ N(0, sigma) e*A.

    Returns dict(x=(N,3) f64, mu=(N,3) f64, seed=seed)."""
    fr = make_frame(n_dipoles, seed)
    mu = np.random.default_rng(seed + 104729).normal(0.0, sigma, (n_dipoles, 3))
    return {"x": fr["x"], "mu": mu, "seed": seed}


def volume_batch_specs(n_frames: int, seed: int = 2024, frame_seed0: int = 5000):
    """Frame shapes of the batched volume workload: per frame (n_charges,
    half_width, frame_seed) with N ~ U[3,000, 40,000] and half-widths 0.5, 1.0
    or 1.5 A (11^3, 21^3 or 31^3 points at 0.1 A); frame f's charges come from
    seed frame_seed0 + f."""
    rng = np.random.default_rng(seed)
    specs = []
    for f in range(n_frames):
        n = int(rng.integers(3000, 40001))
        half = float(rng.choice([0.5, 1.0, 1.5]))
        specs.append((n, half, frame_seed0 + f))
    return specs


def cube_points(half: float, step: float = 0.1):
    """The (2*half/step + 1)^3 grid points of a cube centred at the origin, ij order."""
    g = np.linspace(-half, half, int(round(2 * half / step)) + 1)
    return np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)


def volume_batch_frames(n_frames: int, seed: int = 2024, only=None, frame_seed0: int = 5000):
    """[(points, x, q)] of the batched volume workload (volume_batch_specs);
    ``only`` restricts it to the listed frame indices."""
    out = []
    for f, (n, half, fs) in enumerate(volume_batch_specs(n_frames, seed, frame_seed0)):
        if only is not None and f not in only:
            continue
        fr = make_frame(n, seed=fs)
        out.append((cube_points(half), fr["x"], fr["q"]))
    return out


# The streamline workload the headline benchmark is quoted on: one frame of
# 8,000 charges, 100,000 seeded uniform start points in a box of half-width
# 1.5 A, at most 6,000 Euler steps of 0.001 A per line.
TOPO_N_CHARGES, TOPO_N_LINES, TOPO_HALF, TOPO_STEP, TOPO_CAP = 8000, 100_000, 1.5, 0.001, 6000


def topo_workload(rank: int = 0):
    """(x, q, starts, caps) of the headline streamline workload; rank r > 0
    gets its own frame and start points (seeds offset by 1000 r)."""
    fr = make_frame(TOPO_N_CHARGES, seed=1 + 1000 * rank)
    starts = random_start_points(TOPO_N_LINES, [TOPO_HALF] * 3, seed=2 + 1000 * rank)
    caps = np.full(TOPO_N_LINES, TOPO_CAP, dtype=np.int32)
    return fr["x"], fr["q"], starts, caps
