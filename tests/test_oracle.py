"""Pins the CPU oracle to the reference before the GPU tests rely on it.

Golden fixtures (tests/golden, made by make_golden.py from the reference's own
code and its C library compiled from source):
  * examples 1A/1B point fields as shipped in the reference's example outputs;
  * compute_looped_field / calc_esp_base / calc_field on a synthetic grid;
  * compute_topo_complete_c_shared streamlines on a synthetic frame.
The FP64 oracle must agree with the FP32 reference to FP32 rounding; the FP32
restatement must agree with the reference library more tightly still.
"""

import numpy as np
import pytest


def _example_keys(d):
    return sorted({k[: -len("_x")] for k in d.files if k.endswith("_x")})


def test_point_field_matches_shipped_examples(golden, oracle):
    d = golden("examples_point_field.npz")
    keys = _example_keys(d)
    assert len(keys) == 4
    for k in keys:
        x, Q, shipped = d[k + "_x"], d[k + "_Q"], d[k + "_E_shipped"]
        E64 = oracle.field_grid_f64(np.zeros((1, 3)), x, Q, clamp=False)[0]
        # the shipped values are FP32 sums of ~7,900 terms printed to 8 digits
        np.testing.assert_allclose(E64, shipped, rtol=0, atol=5e-6 * np.abs(shipped).max())
        E32 = oracle.point_field_f32(np.zeros((1, 3)), x, Q)[0]
        np.testing.assert_allclose(E32, d[k + "_E_ref"], rtol=0, atol=2e-6 * np.abs(shipped).max())


def test_grid_field_and_esp_match_reference(golden, oracle):
    g = golden("ref_grid.npz")
    pts = g["mesh"].reshape(-1, 3)
    E_ref = g["field"][:, 3:]
    np.testing.assert_array_equal(g["field"][:, :3], pts)
    E64 = oracle.field_grid_f64(pts, g["x"], g["Q"], clamp=True)
    scale = np.abs(E_ref).max()
    assert np.abs(E64 - E_ref).max() <= 1e-5 * scale
    E32 = oracle.field_grid_f32(pts, g["x"], g["Q"])
    assert np.abs(E32 - E_ref).max() <= 2e-6 * scale
    phi64 = oracle.esp_grid_f64(pts, g["x"], g["Q"])
    assert np.abs(phi64 - g["esp"]).max() <= 1e-5 * np.abs(g["esp"]).max()
    # compute_ESP_on_grid casts to float16
    np.testing.assert_array_equal(np.concatenate([pts, g["esp"].reshape(-1, 1)], axis=1).astype(np.half),
                                  g["esp_half"])
    pf = oracle.field_grid_f64(np.zeros((1, 3)), g["x"], g["Q"], clamp=False)[0]
    np.testing.assert_allclose(pf, g["point_field"], rtol=0, atol=1e-5 * np.abs(pf).max())


def test_topology_matches_reference(golden, oracle):
    t = golden("ref_topo.npz")
    r64, ends, steps = oracle.topo_lines_f64(t["starts"], t["caps"], t["x"], t["Q"], float(t["step"]), t["dims"])
    R = t["result"]
    assert np.abs(r64[:, 0] - R[:, 0]).max() < 5e-6          # distance (A)
    rel = np.abs(r64[:, 1] - R[:, 1]) / np.abs(R[:, 1])
    # FP32 curvature is a second difference of float positions: noisy
    assert np.median(rel) < 5e-3 and rel.max() < 5e-2
    assert steps.min() >= 1 and np.all(steps <= t["caps"])
    r32, _, _ = oracle.topo_lines_f32(t["starts"], t["caps"], t["x"], t["Q"], float(t["step"]), t["dims"])
    assert np.abs(r32[:, 0] - R[:, 0]).max() < 5e-6


def test_topology_semantics(oracle):
    """Hand-checkable cases of thread_operation (math_module.c:523-591)."""
    x = np.array([[0.0, 0.0, 10.0]])
    q = np.array([1.0])
    # a single positive charge on +z: field lines point straight down (-z)
    res, ends, steps = oracle.topo_lines_f64(np.array([[0.0, 0.0, 0.0]]), [1000], x, q, 0.1, [1.0, 1.0, 1.0])
    assert steps[0] == 11                                     # first point strictly beyond -1.0
    np.testing.assert_allclose(ends[0], [0, 0, -1.1], atol=1e-12)
    np.testing.assert_allclose(res[0, 0], 1.1, atol=1e-12)
    assert abs(res[0, 1]) < 1e-12                             # straight line: zero curvature
    # cap reached before the box edge
    res, ends, steps = oracle.topo_lines_f64(np.array([[0.0, 0.0, 0.0]]), [3], x, q, 0.1, [1.0, 1.0, 1.0])
    assert steps[0] == 3 and abs(res[0, 0] - 0.3) < 1e-12
    # n_iter = 0: end point = start point
    res, ends, steps = oracle.topo_lines_f64(np.array([[0.2, 0.0, 0.0]]), [0], x, q, 0.1, [1.0, 1.0, 1.0])
    assert steps[0] == 0 and res[0, 0] == 0.0


def test_reference_library_cross_check(oracle):
    """Live comparison with the reference library built from source (only
    where the reference checkout exists)."""
    ref = oracle.load_reference()
    if ref is None:
        pytest.skip("reference library not built here")
    rng = np.random.default_rng(5)
    x = rng.uniform(-10, 10, (500, 3)).astype(np.float32)
    x = x[np.linalg.norm(x, axis=1) > 2.0]
    q = rng.normal(0, 0.4, len(x)).astype(np.float32)
    pts = rng.uniform(-1, 1, (64, 3)).astype(np.float32)
    E = np.zeros_like(pts)
    ref.compute_looped_field(len(pts), len(q), pts, x, q, E)
    E32 = oracle.field_grid_f32(pts, x, q)
    assert np.abs(E32 - E).max() <= 2e-6 * np.abs(E).max()
    ret = np.zeros(2, np.float32)
    dims = np.array([1.0, 1.0, 1.0], np.float32)
    ref.thread_operation(len(q), 200, np.float32(0.01), pts[0].copy(), dims, x, q, ret)
    r64, _, _ = oracle.topo_lines_f64(pts[:1], [200], x, q, 0.01, dims)
    assert abs(r64[0, 0] - ret[0]) < 5e-6


def test_cluster_oracle_matches_reference(golden, oracle):
    """construct_distance_matrix / construct_distance_matrix_volume: the C
    restatement against the reference's own outputs; make_histograms' binning
    rule (Freedman-Diaconis bin counts, global range, numpy histogram2d,
    division by each file's total) restated on the host reproduces the
    reference's histograms bit for bit."""
    from pycpet_gb300.calculator import histogram_bins

    c = golden("ref_cluster.npz")
    np.testing.assert_allclose(oracle.chi2_matrix_f64(c["hists"]), c["dmat"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(oracle.field_matrix_f64(c["fields"]), c["vmat"], rtol=1e-13, atol=0)
    v, off = c["values"], c["offsets"]
    bins, rng = histogram_bins(v[:, 0], v[:, 1], off[1] - off[0])
    rows = []
    for f in range(len(off) - 1):
        h = oracle.histogram2d(v[off[f]:off[f + 1], 0], v[off[f]:off[f + 1], 1], bins, rng)
        rows.append((h / np.sum(h)).flatten())
    np.testing.assert_array_equal(np.array(rows), c["hists"])


def test_dipole_topology_matches_reference(golden, oracle):
    """thread_operation_dipole through the reference's own
    compute_topo_complete_c_shared_dipole (tests/golden/ref_topo_dipole.npz)."""
    t = golden("ref_topo_dipole.npz")
    R = t["result"]
    r64, _, steps = oracle.topo_lines_dipole(t["starts"], t["caps"], t["x"], t["mu"], float(t["step"]), t["dims"])
    assert np.abs(r64[:, 0] - R[:, 0]).max() < 5e-6
    rel = np.abs(r64[:, 1] - R[:, 1]) / np.abs(R[:, 1])
    assert np.median(rel) < 5e-3 and rel.max() < 5e-2
    assert steps.min() >= 1 and np.all(steps <= t["caps"])
    r32, _, _ = oracle.topo_lines_dipole(t["starts"], t["caps"], t["x"], t["mu"], t["step"], t["dims"], f32=True)
    assert np.abs(r32[:, 0] - R[:, 0]).max() < 2e-6


def test_dipole_semantics(oracle):
    """A single dipole along +x at (10, 0, 0): on that axis R = (R_x, 0, 0), the
    reference's term gives E_x = r^-5 (3 mu_x R_x^2 - mu_x r^2) = 2 mu_x / r^3 and
    E_y = E_z = 0, so a line from the origin runs straight along +x and stops at
    the first step strictly beyond 1.0."""
    x = np.array([[10.0, 0.0, 0.0]])
    mu = np.array([[1.0, 0.0, 0.0]])
    res, ends, steps = oracle.topo_lines_dipole(np.zeros((1, 3)), [1000], x, mu, 0.1, [1.0, 1.0, 1.0])
    assert steps[0] == 11
    np.testing.assert_allclose(ends[0], [1.1, 0.0, 0.0], atol=1e-12)
    np.testing.assert_allclose(res[0, 0], 1.1, atol=1e-12)
    assert abs(res[0, 1]) < 1e-12


def test_frame_preparation_fixture_consistent(golden):
    """The reference's frame preparation (tests/golden/ref_prep.npz) restated
    with numpy on the host: residue runs, radius rule, rotation, box rule with
    the second recentring, shift.  Pins the rules the GPU kernels follow."""
    d = golden("ref_prep.npz")
    x, q, c = d["x"], d["q"], d["center"]
    resid, resnum = d["resid"], d["resnum"]
    start = np.ones(len(x), bool)
    start[1:] = (resid[1:] != resid[:-1]) | (resnum[1:] != resnum[:-1])
    run = np.cumsum(start) - 1
    near = np.linalg.norm(x - c, axis=1) < float(d["radius"])
    keep_run = np.zeros(run.max() + 1, bool)
    keep_run[run[near]] = True
    k1 = keep_run[run]
    assert k1.sum() == int(d["n_after_radius"])
    xr = (x[k1] - c) @ np.linalg.inv(d["T"])
    inside = np.all((xr - c > -d["dims"]) & (xr - c < d["dims"]), axis=1)
    np.testing.assert_allclose(xr[~inside] - d["shift"], d["x_ref"], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(q[k1][~inside], d["q_ref"])
