"""Frame preparation on the GPU (cpetgb_prepare_frame) against the
reference's own filter_radius_whole_residue / rotation / filter_in_box /
box shift (tests/golden/ref_prep.npz).  Kept atoms and their order and
charges exact; box-frame coordinates within 1e-12 A (the 3x3 rotation's
summation order may differ from numpy's by the last bit)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_prepare_frame_matches_reference(gpu_lib, golden):
    from pycpet_gb300.core import prepare_frame

    d = golden("ref_prep.npz")
    x, q = prepare_frame(d["x"], d["q"], d["center"], inv_basis=np.linalg.inv(d["T"]), radius=float(d["radius"]),
                         resid=d["resid"], resnum=d["resnum"], box_half=d["dims"], box_shift=d["shift"])
    assert len(q) == len(d["q_ref"])
    np.testing.assert_array_equal(q, d["q_ref"])
    np.testing.assert_allclose(x, d["x_ref"], rtol=0, atol=1e-12)


def test_prepare_frame_device_and_options(gpu_lib, golden):
    import torch
    from pycpet_gb300.core import prepare_frame

    d = golden("ref_prep.npz")
    inv = np.linalg.inv(d["T"])
    xd, qd = prepare_frame(torch.from_numpy(d["x"]).cuda(), torch.from_numpy(d["q"]).cuda(), d["center"],
                           inv_basis=inv, radius=float(d["radius"]), resid=d["resid"], resnum=d["resnum"],
                           box_half=d["dims"], box_shift=d["shift"])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(qd.cpu().numpy(), d["q_ref"])
    np.testing.assert_allclose(xd.cpu().numpy(), d["x_ref"], rtol=0, atol=1e-12)
    # rotation only, then no rotation at all
    x, q = prepare_frame(d["x"], d["q"], d["center"], inv_basis=inv)
    np.testing.assert_allclose(x, (d["x"] - d["center"]) @ inv, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(q, d["q"])
    x, q = prepare_frame(d["x"], d["q"], d["center"])
    np.testing.assert_array_equal(x, d["x"] - d["center"])
    # everything filtered out; empty input
    x, q = prepare_frame(d["x"], d["q"], d["center"], radius=1e-6, resid=d["resid"], resnum=d["resnum"])
    assert x.shape == (0, 3) and q.shape == (0,)
    x, q = prepare_frame(np.zeros((0, 3)), np.zeros(0), d["center"])
    assert x.shape == (0, 3)


def test_calculator_uses_device_preparation(gpu_lib, golden):
    """drop_in.Calculator with the reference's filter options gives the
    reference's prepared charges."""
    from pycpet_gb300.drop_in import Calculator

    d = golden("ref_prep.npz")
    T = d["T"]
    # axis points that rebuild the fixture's basis: centre + first two basis rows
    opts = {"CPET_method": "point_field", "center": list(d["center"]), "x": list(d["center"] + T[0]),
            "y": list(d["center"] + T[1]), "dimensions": list(d["dims"]), "filter_radius": float(d["radius"]),
            "filter_in_box": True, "box_shift": list(d["shift"]), "dtype": "float64"}
    calc = Calculator(opts, d["x"], d["q"], resid=d["resid"], resnum=d["resnum"])
    np.testing.assert_allclose(calc.transformation_matrix, T, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(calc.Q, d["q_ref"])
    np.testing.assert_allclose(calc.x, d["x_ref"], rtol=0, atol=1e-9)


def test_drop_in_calculator_state(gpu_lib):
    """Calculator state for volume and topo runs (the frame is prepared on the GPU)."""
    from pycpet_gb300.drop_in import Calculator

    rng = np.random.default_rng(1)
    x = rng.uniform(-10, 10, (50, 3))
    Q = rng.normal(size=50)
    opts = {"CPET_method": "volume", "dimensions": [1.0, 1.0, 1.0], "step_size": 0.1,
            "center": [0.5, 0.0, 0.0], "x": [1.5, 0.0, 0.0], "y": [0.5, 1.0, 0.0]}
    c = Calculator(opts, x, Q)
    assert c.mesh.shape == (21, 21, 21, 3)
    np.testing.assert_allclose(c.x, (x - [0.5, 0, 0]).astype(np.float32), atol=1e-6)
    opts.update({"CPET_method": "topo", "n_samples": 100, "max_streamline_init": "fixed_rand"})
    c = Calculator(opts, x, Q)
    assert c.n_samples == 125 and c.random_start_points.shape == (125, 3)      # 5^3 interior grid
    assert c.max_steps == round(2 * np.sqrt(3) / 0.1)
    assert c.random_max_samples.min() >= 1 and c.random_max_samples.max() < c.max_steps
