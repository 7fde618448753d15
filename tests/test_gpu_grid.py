"""GPU parity of the grid kernels (K1 field, K2 potential) against the FP64
oracle and the reference's own outputs.

Tolerances (stated here, checked per point):
  FP64 form   |dE| <= 1e-11 * max|E_oracle| (same arithmetic, other summation order)
  FP32C field |dE| / |E_oracle| <= 1e-5 at every point whose |E_oracle| is at
              least 1e-6 of the frame's median (smaller ones are flagged, not
              scored), and |dE| <= 1e-5 * median|E_oracle| everywhere
  FP32C potential: the same with points below 1e-3 of the median |phi|
              flagged (the relative error of a potential is unbounded where
              phi crosses zero)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32C_REL = 1e-5


def _frame(n, seed):
    from pycpet_gb300.synth import make_frame

    fr = make_frame(n, seed)
    return fr["x"], fr["q"]


def _grid(half, step):
    from pycpet_gb300.calculator import initialize_box_points_uniform, volume_grid_counts

    mesh, _ = initialize_box_points_uniform(np.zeros(3), np.array([1.0, 0, 0]), np.array([0, 1.0, 0]),
                                            volume_grid_counts([half] * 3, step), [half] * 3, dtype="float64")
    return mesh.reshape(-1, 3)


def _fp32c_ok(E, ref):
    n_ref = np.linalg.norm(ref, axis=-1) if ref.ndim == 2 else np.abs(ref)
    err = np.linalg.norm(E - ref, axis=-1) if ref.ndim == 2 else np.abs(E - ref)
    med = np.median(n_ref)
    mask = n_ref >= (1e-6 if ref.ndim == 2 else 1e-3) * med
    rel = err[mask] / n_ref[mask]
    return rel.max(), err.max() / med


@pytest.mark.parametrize("n_charges,seed", [(5000, 1), (1234, 2)])
def test_field_volume_config0(gpu_lib, oracle, n_charges, seed):
    """Plain 'volume' field: 21^3 grid, FP64 and FP32C against the FP64 oracle."""
    from pycpet_gb300 import field_grid

    x, q = _frame(n_charges, seed)
    pts = _grid(1.0, 0.1)
    assert len(pts) == 21 ** 3
    ref = oracle.field_grid_f64(pts, x, q, clamp=True)
    E64 = field_grid(pts, x, q, precision="fp64")
    assert np.abs(E64 - ref).max() <= 1e-11 * np.abs(ref).max()
    E32 = field_grid(pts, x, q, precision="fp32c")
    rel, absn = _fp32c_ok(E32, ref)
    assert rel <= FP32C_REL and absn <= FP32C_REL, (rel, absn)


def test_esp_volume(gpu_lib, oracle):
    from pycpet_gb300 import esp_grid

    x, q = _frame(3000, 4)
    pts = _grid(1.0, 0.1)
    ref = oracle.esp_grid_f64(pts, x, q)
    p64 = esp_grid(pts, x, q, precision="fp64")
    assert np.abs(p64 - ref).max() <= 1e-11 * np.abs(ref).max()
    p32 = esp_grid(pts, x, q, precision="fp32c")
    rel, absn = _fp32c_ok(p32, ref)
    assert rel <= FP32C_REL and absn <= FP32C_REL, (rel, absn)


def test_reference_grid_golden(gpu_lib, golden):
    """The reference's compute_looped_field / calc_esp_base / calc_field
    outputs (FP32 C) on the same inputs, to FP32 rounding."""
    from pycpet_gb300 import esp_grid, field_grid, point_field

    g = golden("ref_grid.npz")
    pts = g["mesh"].reshape(-1, 3)
    for prec in ("fp64", "fp32c"):
        E = field_grid(pts, g["x"], g["Q"], precision=prec)
        ref = g["field"][:, 3:]
        assert np.abs(E - ref).max() <= 1e-5 * np.abs(ref).max()
        phi = esp_grid(pts, g["x"], g["Q"], precision=prec)
        assert np.abs(phi - g["esp"]).max() <= 1e-5 * np.abs(g["esp"]).max()
        pf = point_field(np.zeros(3), g["x"], g["Q"], precision=prec)[0]
        np.testing.assert_allclose(pf, g["point_field"], rtol=0, atol=1e-5 * np.abs(pf).max())


def test_examples_point_field(gpu_lib, golden):
    """Examples 1A/1B: point field at the active-site centre vs the values the
    reference ships in its example outputs."""
    from pycpet_gb300 import point_field

    d = golden("examples_point_field.npz")
    keys = sorted({k[:-2] for k in d.files if k.endswith("_x")})
    for k in keys:
        for prec in ("fp64", "fp32c"):
            E = point_field(np.zeros(3), d[k + "_x"], d[k + "_Q"], precision=prec)[0]
            shipped = d[k + "_E_shipped"]
            np.testing.assert_allclose(E, shipped, rtol=0, atol=5e-6 * np.abs(shipped).max())


def test_clamp_and_edge_cases(gpu_lib, oracle):
    """A grid point on a charge (r^2 clamp), an empty charge set, ragged point
    counts, a single point, and charges not a multiple of a stage."""
    from pycpet_gb300 import field_grid, esp_grid

    rng = np.random.default_rng(9)
    x = rng.uniform(-5, 5, (777, 3))
    q = rng.normal(0, 0.4, 777)
    pts = np.concatenate([x[:3], rng.uniform(-1, 1, (1030, 3))])   # first 3 points sit on charges
    ref = oracle.field_grid_f64(pts, x, q, clamp=True)
    for prec in ("fp64", "fp32c"):
        E = field_grid(pts, x, q, precision=prec)
        assert np.all(np.isfinite(E))
        tol = 1e-11 if prec == "fp64" else 2e-5
        assert np.abs(E - ref).max() <= tol * np.abs(ref).max()
    # no charges: zero field
    assert np.all(field_grid(pts[:10], np.zeros((0, 3)), np.zeros(0)) == 0.0)
    # no points: empty result
    assert field_grid(np.zeros((0, 3)), x, q).shape == (0, 3)
    # single point, single charge: Coulomb's law
    E = field_grid(np.array([[1.0, 0, 0]]), np.array([[0.0, 0, 0]]), np.array([1.0]), precision="fp64")
    np.testing.assert_allclose(E[0], [14.3996451, 0, 0], rtol=1e-15)
    phi = esp_grid(np.array([[2.0, 0, 0]]), np.array([[0.0, 0, 0]]), np.array([-1.0]), precision="fp64")
    np.testing.assert_allclose(phi, [-14.3996451 / 2], rtol=1e-15)


def test_batch_equals_single(gpu_lib):
    """Frames through one descriptor-table launch give exactly the single-frame
    results (same work split per frame is not required: compare to 1 ulp-ish)."""
    from pycpet_gb300 import GridBatch, esp_grid, field_grid

    frames = []
    for i, (n, half) in enumerate([(3000, 0.5), (9000, 1.0), (4000, 1.5), (100, 0.5)]):
        x, q = _frame(n, 20 + i)
        frames.append((_grid(half, 0.1), x, q))
    for kind, fn in (("field", field_grid), ("esp", esp_grid)):
        for prec in ("fp64", "fp32c"):
            gb = GridBatch(frames, kind=kind, precision=prec)
            outs = gb.split(gb.run())
            for (p, x, q), o in zip(frames, outs):
                single = fn(p, x, q, precision=prec).reshape(len(p), -1)
                tol = 1e-12 if prec == "fp64" else 2e-6
                assert np.abs(o - single).max() <= tol * np.abs(single).max()


def test_device_path_matches_host_path(gpu_lib):
    import torch
    from pycpet_gb300 import esp_grid, field_grid, synchronize

    x, q = _frame(2500, 31)
    pts = _grid(1.0, 0.1)
    for prec in ("fp64", "fp32c"):
        host = field_grid(pts, x, q, precision=prec)
        dev = field_grid(torch.from_numpy(pts).cuda(), torch.from_numpy(x).cuda(), torch.from_numpy(q).cuda(),
                         precision=prec)
        synchronize()
        np.testing.assert_array_equal(dev.cpu().numpy(), host)
        hp = esp_grid(pts, x, q, precision=prec)
        dp = esp_grid(torch.from_numpy(pts).cuda(), torch.from_numpy(x).cuda(), torch.from_numpy(q).cuda(),
                      precision=prec)
        synchronize()
        np.testing.assert_array_equal(dp.cpu().numpy(), hp)
