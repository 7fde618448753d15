"""GPU histogram (K4) bit-exact against numpy.histogram2d (the reference's
binner, CPET/utils/calculator.py:702-707), and the PyCPET drop-ins
(Math_ops, calculator functions, calculator methods) against the reference's
outputs."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_hist_bit_exact_random(gpu_lib):
    from pycpet_gb300 import topo_hist2d

    rng = np.random.default_rng(3)
    vals = np.column_stack([rng.uniform(-0.2, 5.5, 100000), rng.exponential(0.4, 100000)])
    for bins, rg in [((20, 20), ((0.0, 5.2), (0.0, None))), ((7, 33), ((0.1, 4.0), (0.05, 2.0))),
                     ((20, 20), ((None, None), (None, None)))]:
        counts, e0, e1 = topo_hist2d(vals, bins=bins, range=rg, return_edges=True)
        lo0 = vals[:, 0].min() if rg[0][0] is None else rg[0][0]
        hi0 = vals[:, 0].max() if rg[0][1] is None else rg[0][1]
        lo1 = vals[:, 1].min() if rg[1][0] is None else rg[1][0]
        hi1 = vals[:, 1].max() if rg[1][1] is None else rg[1][1]
        ref, r0, r1 = np.histogram2d(vals[:, 0], vals[:, 1], bins=list(bins), range=[[lo0, hi0], [lo1, hi1]])
        np.testing.assert_array_equal(e0, r0)
        np.testing.assert_array_equal(e1, r1)
        np.testing.assert_array_equal(counts, ref.astype(np.int64))


def test_hist_edge_values(gpu_lib):
    """Values on every edge, on the last edge, outside the range, NaN, and a
    degenerate range."""
    from pycpet_gb300 import topo_hist2d

    e = np.linspace(0.0, 5.2, 21)
    d = np.concatenate([e, e, [-1e-300, 5.2 + 1e-15, np.nan, 2.0]])
    c = np.concatenate([np.linspace(0, 1.7, 21), np.full(21, 1.7), [0.5, 0.5, 0.5, np.nan]])
    vals = np.column_stack([d, c])
    counts = topo_hist2d(vals, bins=(20, 20), range=((0.0, 5.2), (0.0, 1.7)))
    ref, _, _ = np.histogram2d(d, c, bins=[20, 20], range=[[0.0, 5.2], [0.0, 1.7]])
    np.testing.assert_array_equal(counts, ref.astype(np.int64))
    v = np.column_stack([np.full(10, 2.5), np.linspace(0, 1, 10)])
    counts = topo_hist2d(v, bins=(4, 5), range=((2.5, 2.5), (0.0, 1.0)))
    ref, _, _ = np.histogram2d(v[:, 0], v[:, 1], bins=[4, 5], range=[[2.5, 2.5], [0.0, 1.0]])
    np.testing.assert_array_equal(counts, ref.astype(np.int64))


def test_hist_range_errors(gpu_lib):
    from pycpet_gb300 import CpetgbError, topo_hist2d

    v = np.column_stack([np.linspace(0, 1, 10), np.array([0.1] * 9 + [np.nan])])
    with pytest.raises(CpetgbError) as e:
        topo_hist2d(v, bins=(4, 4), range=((0.0, 1.0), (0.0, None)))   # max of a column with NaN
    assert e.value.code == -6
    with pytest.raises(CpetgbError):
        topo_hist2d(v[:9], bins=(4, 4), range=((1.0, 0.0), (0.0, 1.0)))  # inverted
    # the library stays usable after a reported error
    ok = topo_hist2d(v[:9], bins=(4, 4), range=((0.0, 1.0), (0.0, 1.0)))
    assert ok.sum() == 9


def test_make_histograms_golden(gpu_lib, golden, tmp_path):
    """make_histograms over example 3A's shipped .top files equals the
    reference's make_histograms output."""
    from pycpet_gb300.calculator import make_histograms

    g = golden("examples_topology.npz")
    files = []
    for i in range(2):
        f = os.path.join(tmp_path, f"frame{i}.top")
        np.savetxt(f, g[f"top{i}"], fmt="%.18e")
        files.append(f)
    np.testing.assert_array_equal(make_histograms(files), g["hist"])


def test_math_ops_drop_in(gpu_lib, golden):
    """pycpet_gb300.c_ops.Math_ops against the reference's Math_ops outputs."""
    from pycpet_gb300.c_ops import Math_ops

    M = Math_ops()
    g = golden("ref_grid.npz")
    pts = g["mesh"].reshape(-1, 3)
    E = M.compute_looped_field(pts, g["x"], g["Q"].reshape(-1, 1))
    assert E.dtype == np.float32 and E.shape == pts.shape
    ref = g["field"][:, 3:]
    assert np.abs(E - ref).max() <= 1e-5 * np.abs(ref).max()
    esp = M.calc_esp_base(np.ascontiguousarray(pts[5]), g["x"], g["Q"])
    assert esp.shape == (1,) and abs(esp[0] - g["esp"][5]) <= 1e-5 * np.abs(g["esp"]).max()
    pf = M.calc_field(np.zeros(3, np.float32), g["x"], g["Q"])
    np.testing.assert_allclose(pf, g["point_field"], rtol=0, atol=1e-5 * np.abs(pf).max())
    t = golden("ref_topo.npz")
    r = M.thread_operation(np.ascontiguousarray(t["starts"][0]), int(t["caps"][0]), t["x"], t["Q"],
                           float(t["step"]), t["dims"])
    assert r.dtype == np.float32 and abs(r[0] - t["result"][0, 0]) < 1e-5
    rb = M.thread_operation_batch(t["starts"], t["caps"], t["x"], t["Q"], float(t["step"]), t["dims"])
    assert rb.shape == (len(t["starts"]), 2) and np.abs(rb[:, 0] - t["result"][:, 0]).max() < 1e-5
    # the reference's ndpointer checks: float64 arrays are refused like in c_ops.py:85-95
    import ctypes
    with pytest.raises(ctypes.ArgumentError):
        M.thread_operation(t["starts"][0].astype(np.float64), 10, t["x"], t["Q"], 0.01, t["dims"])


def test_calculator_functions_and_methods(gpu_lib, golden):
    from pycpet_gb300 import calculator as C
    from pycpet_gb300.drop_in import Calculator

    g = golden("ref_grid.npz")
    field = C.compute_field_on_grid(g["mesh"], g["x"], g["Q"].reshape(-1, 1))
    assert field.shape == g["field"].shape and field.dtype == np.float32
    assert np.abs(field - g["field"]).max() <= 1e-5 * np.abs(g["field"][:, 3:]).max()
    esp = C.compute_ESP_on_grid(g["mesh"], g["x"], g["Q"].reshape(-1, 1))
    assert esp.dtype == np.float16 and esp.shape == g["esp_half"].shape
    # float16 output: equal up to one half-precision ulp
    assert np.abs(esp.astype(np.float64) - g["esp_half"].astype(np.float64)).max() <= \
        2 * np.spacing(np.abs(g["esp_half"]).max().astype(np.float16))
    d = golden("examples_point_field.npz")
    rng = np.random.default_rng(0)
    opts = {"CPET_method": "point_field", "center": [0.0, 0.0, 0.0], "x": [1.0, 0.0, 0.0],
            "y": [0.0, 1.0, 0.0]}
    calc = Calculator(opts, d["1A_1_alcdehydro_run1_x"], d["1A_1_alcdehydro_run1_Q"])
    np.testing.assert_allclose(calc.compute_point_field(), d["1A_1_alcdehydro_run1_E_shipped"], rtol=0,
                               atol=1e-5)
    opts = {"CPET_method": "topo", "center": [0.0, 0.0, 0.0], "x": [1.0, 0.0, 0.0], "y": [0.0, 1.0, 0.0],
            "dimensions": [0.5, 0.5, 0.5], "step_size": 0.1, "n_samples": 64, "max_streamline_init": "fixed_rand"}
    x = rng.uniform(-8, 8, (400, 3))
    x = x[np.linalg.norm(x, axis=1) > 2]
    calc = Calculator(opts, x, rng.normal(0, 0.4, len(x)))
    assert calc.compute_topo_complete_c_shared().shape == (64, 2)


def _reference_state(**attrs):
    """An object holding the attributes the reference calculator's methods
    read, built as tests/golden/make_golden.py builds the reference's own
    (calculator.__new__ + attributes), with this package's methods bound."""
    import types

    from pycpet_gb300 import drop_in

    s = types.SimpleNamespace(**attrs)
    for name in drop_in.HOT_METHODS:
        setattr(s, name, getattr(drop_in, name).__get__(s))
    return s


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_calculator_methods_match_reference_methods(gpu_lib, golden, precision):
    """compute_topo_complete_c_shared / compute_topo_GPU_batch_filter on the
    state of ref_topo.npz equal the reference's compute_topo_complete_c_shared
    (CPET/source/calculator.py:675-712), and compute_box / compute_box_ESP on
    the state of ref_grid.npz its compute_field_on_grid / compute_ESP_on_grid
    outputs (calculator.py:489-528)."""
    t = golden("ref_topo.npz")
    s = _reference_state(x=t["x"], Q=t["Q"].reshape(-1, 1), random_start_points=t["starts"],
                         random_max_samples=t["caps"], step_size=float(t["step"]), dimensions=t["dims"],
                         n_samples=len(t["starts"]), precision=precision)
    for res in (s.compute_topo_complete_c_shared(), s.compute_topo_GPU_batch_filter()):
        assert res.shape == t["result"].shape and res.dtype == np.float32
        d = np.abs(res[:, 0] - t["result"][:, 0])
        assert np.mean(d < 1e-5) >= 0.97 and np.median(d) < 1e-6
        np.testing.assert_allclose(np.sort(res, axis=0), np.sort(t["result"], axis=0), rtol=1e-2, atol=1e-2)
    g = golden("ref_grid.npz")
    s = _reference_state(x=g["x"], Q=g["Q"].reshape(-1, 1), mesh=g["mesh"], precision=precision)
    box, shape = s.compute_box()
    assert shape == g["mesh"].shape and box.dtype == np.float32 and box.shape == g["field"].shape
    np.testing.assert_array_equal(box[:, :3], g["field"][:, :3])
    assert np.abs(box[:, 3:] - g["field"][:, 3:]).max() <= 1e-5 * np.abs(g["field"][:, 3:]).max()
    esp, shape = s.compute_box_ESP()
    assert esp.dtype == np.float16 and esp.shape == g["esp_half"].shape
    assert np.abs(esp.astype(np.float64) - g["esp_half"].astype(np.float64)).max() <= \
        2 * np.spacing(np.abs(g["esp_half"]).max().astype(np.float16))
