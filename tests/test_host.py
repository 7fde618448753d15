"""Host-side logic (no GPU): synthetic frames, the box/grid/start-point
restatements, the frame descriptor table and the histogram binning rules."""
import os

import numpy as np
import pytest

from conftest import ROOT


def test_synthetic_frame_properties():
    from scipy.spatial import cKDTree
    from pycpet_gb300.synth import cube_edge, make_frame

    fr = make_frame(5000, seed=3)
    x, q = fr["x"], fr["q"]
    assert x.shape == (5000, 3) and q.shape == (5000,)
    d, _ = cKDTree(x).query(x, k=2)
    assert d[:, 1].min() >= 1.0 - 1e-12                 # min separation
    assert np.linalg.norm(x, axis=1).min() >= 2.0 - 1e-12  # nothing within 2 A of the centre
    assert abs(q.sum() - round(q.sum())) < 1e-9          # integer net charge
    assert np.abs(q).max() <= 1.0 + 1e-3
    assert np.linalg.norm(x, axis=1).max() <= cube_edge(5000) * np.sqrt(3) / 2 + 1e-9
    T = fr["T"]
    np.testing.assert_allclose(T @ T.T, np.eye(3), atol=1e-12)
    # determinism
    fr2 = make_frame(5000, seed=3)
    np.testing.assert_array_equal(fr2["x"], x)
    assert cube_edge(40000) == pytest.approx(100.0)


def test_grid_counts_and_mesh():
    from pycpet_gb300.calculator import initialize_box_points_uniform, volume_grid_counts

    assert volume_grid_counts([1.0, 1.0, 1.0], 0.1) == [20, 20, 20]   # -> 21^3 points
    assert volume_grid_counts([0.5, 0.5, 0.5], 0.1) == [10, 10, 10]
    mesh, T = initialize_box_points_uniform(np.zeros(3), np.array([1.0, 0, 0]), np.array([0, 1.0, 0]),
                                            [20, 20, 20], [1.0, 1.0, 1.0])
    assert mesh.shape == (21, 21, 21, 3) and mesh.dtype == np.float32
    np.testing.assert_array_equal(mesh[0, 0, 0], [-1, -1, -1])
    np.testing.assert_array_equal(mesh[-1, 0, 0], [1, -1, -1])      # ij indexing
    np.testing.assert_array_equal(T, np.eye(3))
    starts, caps, _ = initialize_box_points_uniform(np.zeros(3), np.array([1.0, 0, 0]), np.array([0, 1.0, 0]),
                                                    [4, 4, 4], [1.0, 1.0, 1.0], max_steps=50, ret_rand_max=True,
                                                    inclusive=False, seed=42)
    assert starts.shape == (4, 4, 4, 3) and caps.min() >= 1 and caps.max() < 50
    assert np.abs(starts).max() < 1.0                               # faces excluded


def test_restatements_match_reference_functions():
    ref = os.environ.get("CPETGB_REF", "/root/reference")
    if not os.path.isdir(ref) or not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "math_module.so")):
        pytest.skip(f"reference checkout or its library not present (CPETGB_REF={ref})")
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import import_reference
    from pycpet_gb300 import calculator as mine

    ucalc, _ = import_reference(ref)
    c, xp, yp = np.array([0.3, -0.2, 0.1]), np.array([1.3, 0.4, 0.2]), np.array([0.1, 1.5, -0.3])
    for incl in (True, False):
        np.random.seed(1)
        a = ucalc.initialize_box_points_uniform(c, xp, yp, [7, 8, 9], [1.0, 1.2, 1.5], max_steps=40,
                                                ret_rand_max=True, inclusive=incl)
        np.random.seed(1)
        b = mine.initialize_box_points_uniform(c, xp, yp, [7, 8, 9], [1.0, 1.2, 1.5], max_steps=40,
                                               ret_rand_max=True, inclusive=incl)
        for u, v in zip(a, b):
            np.testing.assert_array_equal(u, v)
    np.random.seed(2)
    a = ucalc.initialize_box_points_random(c, xp, yp, [1.0, 1.2, 1.5], 100, max_steps=40)
    np.random.seed(2)
    b = mine.initialize_box_points_random(c, xp, yp, [1.0, 1.2, 1.5], 100, max_steps=40)
    for u, v in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(u, v)


def test_frame_descriptor_table():
    from pycpet_gb300.core import GridBatch

    rng = np.random.default_rng(0)
    frames = [(rng.normal(size=(p, 3)), rng.normal(size=(n, 3)), rng.normal(size=n))
              for p, n in [(5, 3), (0, 4), (7, 0), (2, 2)]]
    gb = GridBatch(frames, kind="esp", precision="fp64")
    np.testing.assert_array_equal(gb.desc, [[0, 3, 0, 5], [3, 4, 5, 0], [7, 0, 5, 7], [7, 2, 12, 2]])
    assert gb.points.shape == (14, 3) and gb.x.shape == (9, 3) and gb.q.shape == (9,)
    assert gb.pair_evals == 5 * 3 + 2 * 2
    parts = gb.split(np.arange(14))
    assert [len(p) for p in parts] == [5, 0, 7, 2]


def test_make_histograms_binning_rules(golden):
    """Freedman-Diaconis bins and ranges of make_histograms
    (CPET/utils/calculator.py:664-707) with numpy's histogram2d as binner
    reproduce the reference's normalised histograms of example 3A."""
    from pycpet_gb300.calculator import histogram_bins

    g = golden("examples_topology.npz")
    tops = [g["top0"], g["top1"]]
    allv = np.concatenate(tops)
    bins, rng = histogram_bins(allv[:, 0], allv[:, 1], len(tops[0]))
    hists = []
    for t in tops:
        h, _, _ = np.histogram2d(t[:, 0], t[:, 1], bins=list(bins), range=list(rng))
        hists.append((h / h.sum()).flatten())
    np.testing.assert_array_equal(np.array(hists), g["hist"])
