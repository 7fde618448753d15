"""Per-point accuracy of the FP32C field on the batched volume workload's
largest frames, and the FP64 refinement of ill-conditioned points.

Tolerance (stated here): at every grid point whose FP64-oracle field has
|E_ref| >= 1e-6 * the frame's median |E_ref| (smaller ones are flagged, not
scored), the FP32C field satisfies |E - E_ref| / |E_ref| <= 1e-5.  The oracle
is the CPU FP64 restatement of compute_looped_field
(CPET/utils/math_module.c:405-451).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def _largest_volume_frames(k):
    from pycpet_gb300.synth import volume_batch_frames, volume_batch_specs

    specs = volume_batch_specs(64)
    size = [(int(round(2 * h / 0.1)) + 1) ** 3 * n for n, h, _ in specs]
    idx = sorted(range(len(specs)), key=lambda i: -size[i])[:k]
    return volume_batch_frames(64, only=set(idx))


def _per_point_rel(E, ref):
    nb = np.linalg.norm(ref, axis=1)
    scored = nb >= 1e-6 * np.median(nb)
    return np.linalg.norm(E - ref, axis=1)[scored] / nb[scored]


def test_field_fp32c_per_point_on_largest_volume_frames(gpu_lib, oracle):
    """The three largest frames of the 64-frame batched volume workload (31^3
    points, 36,622-39,771 charges), through one batched launch."""
    from pycpet_gb300 import GridBatch

    frames = _largest_volume_frames(3)
    gb = GridBatch(frames, kind="field", precision="fp32c")
    outs = gb.split(gb.run())
    for (pts, x, q), E in zip(frames, outs):
        assert len(pts) == 31 ** 3 and len(q) > 36000
        ref = oracle.field_grid_f64(pts, x, q, clamp=True)
        rel = _per_point_rel(E, ref)
        assert rel.max() <= REL, (len(q), rel.max(), np.mean(rel > REL))


def test_refined_points_equal_fp64(gpu_lib, oracle):
    """Points below the refinement threshold come out of the FP32C call
    recomputed in double-float arithmetic (within 1e-9 of the oracle per
    point), the rest unchanged;
    with the refinement off the same call is plain FP32C."""
    from pycpet_gb300 import field_grid, set_field_refinement
    from pycpet_gb300.synth import cube_points, make_frame

    fr = make_frame(12000, seed=77)
    pts = cube_points(1.5)
    ref = oracle.field_grid_f64(pts, fr["x"], fr["q"], clamp=True)
    old = set_field_refinement(0.3)
    try:
        E = field_grid(pts, fr["x"], fr["q"], precision="fp32c")
        set_field_refinement(0.0)
        E_plain = field_grid(pts, fr["x"], fr["q"], precision="fp32c")
    finally:
        set_field_refinement(old)
    m = np.linalg.norm(E_plain, axis=1)
    # the threshold is 0.3 x the lower edge of the median's 1/16-octave bin
    low = m < 0.3 * np.median(m) * 2.0 ** (-1 / 16)
    high = m >= 0.3 * np.median(m)
    assert 0 < low.sum() < len(m) // 4
    nb = np.linalg.norm(ref, axis=1)
    d_low = np.linalg.norm(E[low] - ref[low], axis=1) / nb[low]
    assert d_low.max() <= 1e-9, d_low.max()
    np.testing.assert_array_equal(E[high], E_plain[high])
    assert _per_point_rel(E, ref).max() <= REL


def test_refinement_setting_is_validated(gpu_lib):
    from pycpet_gb300 import CpetgbError, set_field_refinement

    old = set_field_refinement(0.1)
    try:
        for bad in (-0.1, 1.5, float("nan"), float("inf")):
            with pytest.raises(CpetgbError):
                set_field_refinement(bad)
    finally:
        set_field_refinement(old)


def test_clamp_near_tiles(gpu_lib, oracle):
    """Points closer than 1e-3 A to a charge (the r^2 >= 1e-6 clamp acts),
    points 0.005-0.02 A away, and far points.  FP64 must match the oracle to
    1e-11 everywhere -- a tile that needed the clamp but skipped it would be
    off by a factor of up to 1e6 there.  FP32C: within 1e-5 at the far points;
    at the near ones the FP32 rounding of coordinates (about 4e-7 A at 6 A)
    limits it to about r_round / r, so the bound there is 1e-2 (an unclamped
    term would be 6-16 times the clamped one)."""
    from pycpet_gb300 import field_grid

    rng = np.random.default_rng(12)
    x = rng.uniform(-6, 6, (3000, 3))
    q = rng.normal(0, 0.4, 3000)
    offs = np.array([[0, 0, 0], [4e-4, 0, 0], [0, 7e-4, 2e-4], [0.005, 0, 0], [0, 0.012, 0], [0.02, 0.01, 0]])
    near = np.concatenate([x[k] + offs for k in range(0, 600, 50)])
    far = rng.uniform(-1, 1, (2000, 3))
    pts = np.concatenate([far[:700], near, far[700:]])
    is_near = np.zeros(len(pts), bool)
    is_near[700:700 + len(near)] = True
    ref = oracle.field_grid_f64(pts, x, q, clamp=True)
    nb = np.linalg.norm(ref, axis=1)
    E64 = field_grid(pts, x, q, precision="fp64")
    assert np.all(np.linalg.norm(E64 - ref, axis=1) <= 1e-11 * nb)
    E32 = field_grid(pts, x, q, precision="fp32c")
    assert np.all(np.isfinite(E32))
    rel = np.linalg.norm(E32 - ref, axis=1) / nb
    assert rel[~is_near].max() <= REL
    assert rel[is_near].max() <= 1e-2


def test_field_fp32c_per_point_on_other_seeded_frames(gpu_lib, oracle):
    """The same bound on frames the refinement threshold was not chosen on:
    the batched volume workload's distribution drawn with another seed (16
    frames, 3,000-40,000 charges, 11^3 / 21^3 / 31^3 grids)."""
    from pycpet_gb300 import GridBatch
    from pycpet_gb300.synth import volume_batch_frames

    frames = volume_batch_frames(16, seed=777, frame_seed0=90_000)
    gb = GridBatch(frames, kind="field", precision="fp32c")
    outs = gb.split(gb.run())
    worst = 0.0
    for (pts, x, q), E in zip(frames, outs):
        ref = oracle.field_grid_f64(pts, x, q, clamp=True)
        worst = max(worst, float(_per_point_rel(E, ref).max()))
    assert worst <= REL, worst
