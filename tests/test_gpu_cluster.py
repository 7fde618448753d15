"""Clustering front end on the GPU: histogram sets and distance matrices,
checked against the reference's own outputs (tests/golden/ref_cluster.npz,
made by make_golden.py from make_histograms, construct_distance_matrix and
construct_distance_matrix_volume) and against the FP64 oracle on ragged sizes.

Tolerances: histograms bit-exact (numpy's binning and division reproduced);
FP64 matrices rtol 1e-12 (only the order of the final sum differs from numpy);
FP32C matrices rtol 1e-5 of the largest entry (FP32 terms, compensated sums).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bins(c):
    from pycpet_gb300.calculator import histogram_bins

    v, off = c["values"], c["offsets"]
    return histogram_bins(v[:, 0], v[:, 1], off[1] - off[0])


def test_hist_sets_reproduce_make_histograms(gpu_lib, golden, oracle):
    from pycpet_gb300 import topo_hist2d_sets

    c = golden("ref_cluster.npz")
    bins, rng = _bins(c)
    h = topo_hist2d_sets(c["values"], c["offsets"], bins, rng, normalize=True)
    np.testing.assert_array_equal(h, c["hists"])
    counts = topo_hist2d_sets(c["values"], c["offsets"], bins, rng, normalize=False)
    off = c["offsets"]
    for f in range(len(off) - 1):
        ref = oracle.histogram2d(c["values"][off[f]:off[f + 1], 0], c["values"][off[f]:off[f + 1], 1], bins, rng)
        np.testing.assert_array_equal(counts[f], ref.astype(np.int64).ravel())


def test_hist_sets_ragged_and_empty(gpu_lib, oracle):
    """Uneven set sizes, an empty set (NaN row, as numpy's 0/0), values on the
    edges and outside the range."""
    from pycpet_gb300 import topo_hist2d_sets

    rng = np.random.default_rng(3)
    sizes = [0, 1, 17, 5000, 33]
    vals = rng.uniform(-0.5, 5.5, (sum(sizes), 2))
    vals[5, 0] = 5.2
    vals[6, 1] = 0.0
    off = np.concatenate([[0], np.cumsum(sizes)])
    rg = ((0.0, 5.2), (0.0, 5.0))
    counts = topo_hist2d_sets(vals, off, (13, 7), rg, normalize=False)
    h = topo_hist2d_sets(vals, off, (13, 7), rg, normalize=True)
    for f in range(len(sizes)):
        ref = oracle.histogram2d(vals[off[f]:off[f + 1], 0], vals[off[f]:off[f + 1], 1], (13, 7), rg).ravel()
        np.testing.assert_array_equal(counts[f], ref.astype(np.int64))
        if ref.sum() == 0:
            assert np.all(np.isnan(h[f]))
        else:
            np.testing.assert_array_equal(h[f], ref / np.sum(ref))


def test_chi2_matrix_matches_reference(gpu_lib, golden):
    from pycpet_gb300 import chi2_distance_matrix

    c = golden("ref_cluster.npz")
    d64 = chi2_distance_matrix(c["hists"], precision="fp64")
    np.testing.assert_allclose(d64, c["dmat"], rtol=1e-12, atol=0)
    d32 = chi2_distance_matrix(c["hists"], precision="fp32c")
    np.testing.assert_allclose(d32, c["dmat"], rtol=0, atol=1e-5 * c["dmat"].max())
    for d in (d64, d32):
        np.testing.assert_array_equal(d, d.T)
        assert np.all(np.diag(d) == 0)


def test_field_matrix_matches_reference(gpu_lib, golden):
    from pycpet_gb300 import field_distance_matrix

    c = golden("ref_cluster.npz")
    d64 = field_distance_matrix(c["fields"], precision="fp64")
    np.testing.assert_allclose(d64, c["vmat"], rtol=1e-12, atol=0)
    d32 = field_distance_matrix(c["fields"], precision="fp32c")
    np.testing.assert_allclose(d32, c["vmat"], rtol=0, atol=1e-5 * c["vmat"].max())
    np.testing.assert_array_equal(d32, d32.T)


@pytest.mark.parametrize("n,bins", [(1, 5), (63, 31), (130, 77), (200, 400)])
def test_chi2_matrix_ragged_vs_oracle(gpu_lib, oracle, n, bins):
    """Sizes that are not multiples of the 64-row tile or the 32-bin chunk;
    sparse histograms with bins empty in both rows (skipped terms) and one
    all-zero row."""
    from pycpet_gb300 import chi2_distance_matrix

    rng = np.random.default_rng(n + bins)
    h = rng.random((n, bins)) * (rng.random((n, bins)) < 0.3)
    h[n // 2] = 0.0
    s = h.sum(axis=1, keepdims=True)
    h = np.divide(h, s, out=np.zeros_like(h), where=s > 0)
    ref = oracle.chi2_matrix_f64(h)
    np.testing.assert_allclose(chi2_distance_matrix(h, "fp64"), ref, rtol=1e-12, atol=1e-300)
    scale = max(ref.max(), 1e-300)
    np.testing.assert_allclose(chi2_distance_matrix(h, "fp32c"), ref, rtol=0, atol=1e-5 * scale)


@pytest.mark.parametrize("n,points", [(2, 1), (65, 343), (129, 1331)])
def test_field_matrix_ragged_vs_oracle(gpu_lib, oracle, n, points):
    from pycpet_gb300 import field_distance_matrix

    rng = np.random.default_rng(n * 7 + points)
    f = rng.normal(0.0, 2.0, (n, points, 3))
    f[1] = f[0]  # identical fields: zero distance, zero-length differences
    ref = oracle.field_matrix_f64(f)
    np.testing.assert_allclose(field_distance_matrix(f, "fp64"), ref, rtol=1e-12, atol=0)
    d32 = field_distance_matrix(f, "fp32c")
    np.testing.assert_allclose(d32, ref, rtol=0, atol=1e-5 * ref.max())
    assert d32[0, 1] == 0.0


def test_device_buffers_and_empty(gpu_lib, golden):
    import torch
    from pycpet_gb300 import chi2_distance_matrix, field_distance_matrix, topo_hist2d_sets

    c = golden("ref_cluster.npz")
    bins, rng = _bins(c)
    dv = torch.from_numpy(c["values"]).cuda()
    h = topo_hist2d_sets(dv, c["offsets"], bins, rng)
    assert h.is_cuda
    d = chi2_distance_matrix(h, "fp64")
    torch.cuda.synchronize()
    np.testing.assert_allclose(d.cpu().numpy(), c["dmat"], rtol=1e-12, atol=0)
    fv = field_distance_matrix(torch.from_numpy(c["fields"]).cuda(), "fp32c")
    np.testing.assert_allclose(fv.cpu().numpy(), c["vmat"], rtol=0, atol=1e-5 * c["vmat"].max())
    assert chi2_distance_matrix(np.zeros((0, 4)), "fp64").shape == (0, 0)


def test_calculator_drop_ins(gpu_lib, golden, tmp_path):
    """make_histograms -> construct_distance_matrix through the reference's
    function names, from .top files, as the clustering front end calls them
    (CPET/source/cluster.py:126-128)."""
    from pycpet_gb300 import calculator

    c = golden("ref_cluster.npz")
    v, off = c["values"], c["offsets"]
    files = []
    for f in range(len(off) - 1):
        p = tmp_path / f"frame_{f:02d}.top"
        np.savetxt(p, v[off[f]:off[f + 1]])
        files.append(str(p))
    hists = calculator.make_histograms(files)
    np.testing.assert_array_equal(hists, c["hists"])
    np.testing.assert_allclose(calculator.construct_distance_matrix(hists, "fp64"), c["dmat"], rtol=1e-12)
    np.testing.assert_allclose(calculator.construct_distance_matrix_volume(list(c["fields"]), "fp64"), c["vmat"],
                               rtol=1e-12)
    assert calculator.distance_numpy(hists[0], hists[1]) == pytest.approx(c["dmat"][0, 1], rel=1e-14)
