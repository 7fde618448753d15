"""GPU parity of the streamline kernel (K3) against the FP64 oracle of
thread_operation (CPET/utils/math_module.c:523-591) and the reference's own
compute_topo_complete_c_shared output.

Tolerances (stated here):
  FP64 form   same step count; |d end| <= 1e-9 A; |d dist| <= 1e-9 A;
              |d curv| <= 1e-6 * |curv| + 1e-9 on lines that are not chaotic
              (identical step counts); at most 1% of lines may diverge
  FP32C form  |d dist| <= 1e-4 A on 99% of lines; curvature relative error
              <= 1e-2 on 99% of lines (FP32 field directions)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(n_charges, n_lines, seed, half=1.5, step=0.01, caps=None):
    from pycpet_gb300.synth import make_frame, random_start_points

    fr = make_frame(n_charges, seed)
    starts = random_start_points(n_lines, [half] * 3, seed + 1)
    if caps is None:
        max_steps = round(2 * np.linalg.norm([half] * 3) / step)
        caps = np.random.default_rng(seed + 2).integers(1, max_steps, n_lines)
    return fr["x"], fr["q"], starts, np.asarray(caps, np.int32), [half] * 3, step


def test_fp64_matches_oracle(gpu_lib, oracle):
    from pycpet_gb300 import topo_lines

    x, q, starts, caps, dims, step = _case(600, 300, 41)
    caps[:6] = [0, 1, 2, 3, 1, 0]                       # the short-line paths
    ref, ref_end, ref_steps = oracle.topo_lines_f64(starts, caps, x, q, step, dims)
    res, ends, steps = topo_lines(starts, caps, x, q, step, dims, precision="fp64", return_ends=True,
                                  return_steps=True)
    same = steps == ref_steps
    assert same.mean() >= 0.99
    assert np.abs(ends[same] - ref_end[same]).max() <= 1e-9
    assert np.abs(res[same, 0] - ref[same, 0]).max() <= 1e-9
    assert np.all(np.abs(res[same, 1] - ref[same, 1]) <= 1e-6 * np.abs(ref[same, 1]) + 1e-9)
    np.testing.assert_array_equal(steps[:6], ref_steps[:6])
    assert steps[0] == 0 and steps[5] == 0


def test_fp32c_matches_oracle(gpu_lib, oracle):
    from pycpet_gb300 import topo_lines

    x, q, starts, caps, dims, step = _case(2000, 400, 51)
    ref, ref_end, ref_steps = oracle.topo_lines_f64(starts, caps, x, q, step, dims)
    res, ends, steps = topo_lines(starts, caps, x, q, step, dims, precision="fp32c", return_ends=True,
                                  return_steps=True)
    dd = np.abs(res[:, 0] - ref[:, 0])
    assert np.quantile(dd, 0.99) <= 1e-4
    rel = np.abs(res[:, 1] - ref[:, 1]) / np.maximum(np.abs(ref[:, 1]), 1e-12)
    assert np.quantile(rel, 0.99) <= 1e-2
    assert (steps == ref_steps).mean() >= 0.98


def test_reference_topology_golden(gpu_lib, golden):
    """Against the reference's compute_topo_complete_c_shared (FP32 C)."""
    from pycpet_gb300 import topo_lines

    t = golden("ref_topo.npz")
    R = t["result"]
    for prec in ("fp64", "fp32c"):
        res = topo_lines(t["starts"], t["caps"], t["x"], t["Q"], float(t["step"]), t["dims"], precision=prec)
        assert np.abs(res[:, 0] - R[:, 0]).max() < 1e-5
        rel = np.abs(res[:, 1] - R[:, 1]) / np.abs(R[:, 1])
        assert np.median(rel) < 5e-3 and rel.max() < 5e-2     # reference curvature is FP32 noise


def test_refill_and_streamed_charges(gpu_lib, oracle):
    """Many more lines than slots (refill from the queue), and a frame too
    large for shared memory (charges streamed from L2)."""
    from pycpet_gb300 import topo_lines

    x, q, starts, caps, dims, step = _case(16000, 40, 61, step=0.02)
    ref, _, ref_steps = oracle.topo_lines_f64(starts, caps, x, q, step, dims)
    for prec in ("fp64", "fp32c"):
        res, steps = topo_lines(starts, caps, x, q, step, dims, precision=prec, return_steps=True)
        assert (steps == ref_steps).mean() >= 0.95
        assert np.quantile(np.abs(res[:, 0] - ref[:, 0]), 0.9) <= 1e-4
    x, q, starts, caps, dims, step = _case(300, 20000, 71, step=0.05)
    res, steps = topo_lines(starts, caps, x, q, step, dims, precision="fp32c", return_steps=True)
    sub = np.arange(0, 20000, 97)
    ref, _, ref_steps = oracle.topo_lines_f64(starts[sub], caps[sub], x, q, step, dims)
    assert (steps[sub] == ref_steps).mean() >= 0.98
    assert np.quantile(np.abs(res[sub, 0] - ref[:, 0]), 0.98) <= 1e-4


def test_topo_edge_cases(gpu_lib):
    from pycpet_gb300 import topo_lines

    x = np.array([[0.0, 0.0, 10.0]])
    q = np.array([1.0])
    res, ends, steps = topo_lines(np.array([[0.0, 0.0, 0.0]]), [1000], x, q, 0.1, [1.0, 1.0, 1.0],
                                  precision="fp64", return_ends=True, return_steps=True)
    assert steps[0] == 11
    np.testing.assert_allclose(ends[0], [0, 0, -1.1], atol=1e-12)
    assert abs(res[0, 0] - 1.1) < 1e-12 and abs(res[0, 1]) < 1e-12
    res, steps = topo_lines(np.zeros((3, 3)), [0, 1, 3], x, q, 0.1, [1.0, 1.0, 1.0], precision="fp32c",
                            return_steps=True)
    np.testing.assert_array_equal(steps, [0, 1, 3])
    np.testing.assert_allclose(res[:, 0], [0.0, 0.1, 0.3], atol=1e-6)
    assert topo_lines(np.zeros((0, 3)), [], x, q, 0.1, [1, 1, 1]).shape == (0, 2)


def test_device_path(gpu_lib):
    import torch
    from pycpet_gb300 import synchronize, topo_lines

    x, q, starts, caps, dims, step = _case(1500, 500, 81)
    host = topo_lines(starts, caps, x, q, step, dims, precision="fp32c")
    dev = topo_lines(torch.from_numpy(starts).cuda(), torch.from_numpy(caps).cuda(), torch.from_numpy(x).cuda(),
                     torch.from_numpy(q).cuda(), step, dims, precision="fp32c")
    synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


def test_batch_of_frames_equals_single_frames(gpu_lib):
    """Frames of different sizes (resident and streamed charges, uneven line
    counts, different boxes and steps) in one launch give exactly the
    per-frame results."""
    from pycpet_gb300 import TopoBatch, topo_lines

    specs = [(2000, 300, 1.5, 0.01), (15000, 60, 1.0, 0.02), (700, 1000, 0.5, 0.01), (9000, 1, 1.5, 0.01),
             (3000, 0, 1.5, 0.01)]
    frames = []
    for i, (n, L, half, step) in enumerate(specs):
        x, q, starts, caps, dims, _ = _case(n, max(L, 1), 100 + i, half=half, step=step)
        frames.append({"x": x, "q": q, "starts": starts[:L], "n_iter": caps[:L], "step": step,
                       "half_dims": dims})
    for prec in ("fp32c", "fp64"):
        tb = TopoBatch(frames, precision=prec)
        res, steps = tb.run(return_steps=True)
        for fr, r, s in zip(frames, tb.split(res), tb.split(steps)):
            if len(fr["starts"]) == 0:
                assert len(r) == 0
                continue
            single, ss = topo_lines(fr["starts"], fr["n_iter"], fr["x"], fr["q"], fr["step"], fr["half_dims"],
                                    precision=prec, return_steps=True)
            np.testing.assert_array_equal(s, ss)
            np.testing.assert_array_equal(r, single)


def test_graph_plans_replay(gpu_lib):
    """CUDA-graph plans (grid and streamline batches) give the direct results,
    and a replay after the inputs change in place gives the new results."""
    import torch
    from pycpet_gb300 import GridBatch, TopoBatch, synchronize

    frames = []
    for i, (n, L) in enumerate([(1500, 200), (4000, 50), (600, 300)]):
        x, q, starts, caps, dims, step = _case(n, L, 200 + i)
        frames.append({"x": x, "q": q, "starts": starts, "n_iter": caps, "step": step, "half_dims": dims})
    for prec in ("fp32c", "fp64"):
        direct = TopoBatch(frames, precision=prec, device=True).run()
        tb = TopoBatch(frames, precision=prec, device=True, graph=True)
        r1 = tb.run().clone()
        synchronize()
        np.testing.assert_array_equal(r1.cpu().numpy(), direct.cpu().numpy())
        tb.q.mul_(-1.0)                       # reversed charges: new field lines, replay the same graph
        r2 = tb.run()
        synchronize()
        flipped = [dict(fr, q=-fr["q"]) for fr in frames]
        np.testing.assert_array_equal(r2.cpu().numpy(), TopoBatch(flipped, precision=prec).run())
    gframes = [(np.random.default_rng(i).uniform(-1, 1, (n, 3)), fr["x"], fr["q"])
               for i, (n, fr) in enumerate(zip([700, 1331, 64], frames))]
    for kind in ("field", "esp"):
        direct = GridBatch(gframes, kind=kind, device=True).run().clone()
        gb = GridBatch(gframes, kind=kind, device=True, graph=True)
        out = gb.run()
        synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), direct.cpu().numpy())
        gb.points.add_(0.25)
        out = gb.run()
        synchronize()
        moved = [(p + 0.25, x, q) for p, x, q in gframes]
        np.testing.assert_array_equal(out.cpu().numpy(), GridBatch(moved, kind=kind).run())


def test_tuned_variants_agree(gpu_lib, oracle):
    """Every tile-shape variant the autotuner may pick gives parity results:
    streamline slot counts are bit-identical, grid shapes stay within the
    FP32C tolerance of the FP64 oracle."""
    from pycpet_gb300 import _lib, autotune, field_grid, topo_lines

    x, q, starts, caps, dims, step = _case(3000, 600, 300)
    k = autotune.key(autotune.OP_TOPO, "fp32c", 1, len(starts))
    out = []
    for v in range(2):
        autotune.set_variant(k, v)
        out.append(topo_lines(starts, caps, x, q, step, dims, precision="fp32c"))
    autotune.set_variant(k, -1)
    np.testing.assert_array_equal(out[0], out[1])
    pts = np.random.default_rng(1).uniform(-1, 1, (3000, 3))
    ref = oracle.field_grid_f64(pts, x, q)
    k = autotune.key(autotune.OP_GRID, "fp32c", _lib.FIELD, len(pts) * len(q))
    for v in range(_lib.lib().cpetgb_tune_variants(autotune.OP_GRID)):
        autotune.set_variant(k, v)
        E = field_grid(pts, x, q, precision="fp32c")
        err = np.linalg.norm(E - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err.max() <= 1e-5, (v, err.max())
    autotune.set_variant(k, -1)
