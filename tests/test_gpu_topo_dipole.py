"""GPU parity of the dipole streamline path (thread_operation_dipole,
CPET/utils/math_module.c:593-659) against the FP64 oracle and the reference's
own compute_topo_complete_c_shared_dipole output (tests/golden/ref_topo_dipole.npz).

Tolerances (as for the charge path):
  FP64 form   same step count on >= 99% of lines; on those |d end|, |d dist|
              <= 1e-9 A and |d curv| <= 1e-6 |curv| + 1e-9
  FP32C form  |d dist| <= 1e-4 A on 99% of lines; curvature relative error
              <= 1e-2 on 99% of lines
  reference   |d dist| < 1e-5 A; curvature (FP32 noise on the reference side)
              median relative < 5e-3, max < 5e-2
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dipoles(n, seed, box=12.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-box, box, (3 * n, 3))
    x = x[np.linalg.norm(x, axis=1) > 2.5][:n]
    mu = rng.normal(0.0, 0.3, (len(x), 3))
    return x, mu


def _case(n, n_lines, seed, half=1.5, step=0.01):
    from pycpet_gb300.synth import random_start_points

    x, mu = _dipoles(n, seed)
    starts = random_start_points(n_lines, [half] * 3, seed + 1)
    max_steps = round(2 * np.linalg.norm([half] * 3) / step)
    caps = np.random.default_rng(seed + 2).integers(1, max_steps, n_lines).astype(np.int32)
    return x, mu, starts, caps, [half] * 3, step


def test_dipole_fp64_matches_oracle(gpu_lib, oracle):
    from pycpet_gb300 import topo_dipole_lines

    x, mu, starts, caps, dims, step = _case(700, 300, 81)
    caps[:4] = [0, 1, 2, 3]
    ref, ref_end, ref_steps = oracle.topo_lines_dipole(starts, caps, x, mu, step, dims)
    res, ends, steps = topo_dipole_lines(starts, caps, x, mu, step, dims, precision="fp64", return_ends=True,
                                         return_steps=True)
    same = steps == ref_steps
    assert same.mean() >= 0.99
    assert np.abs(ends[same] - ref_end[same]).max() <= 1e-9
    assert np.abs(res[same, 0] - ref[same, 0]).max() <= 1e-9
    assert np.all(np.abs(res[same, 1] - ref[same, 1]) <= 1e-6 * np.abs(ref[same, 1]) + 1e-9)
    np.testing.assert_array_equal(steps[:4], [0, 1, 2, 3])


@pytest.mark.parametrize("n", [2000, 12000])   # charges resident in shared memory / streamed from L2
def test_dipole_fp32c_matches_oracle(gpu_lib, oracle, n):
    from pycpet_gb300 import topo_dipole_lines

    x, mu, starts, caps, dims, step = _case(n, 200, 91 + n, step=0.02)
    ref, _, ref_steps = oracle.topo_lines_dipole(starts, caps, x, mu, step, dims)
    res, steps = topo_dipole_lines(starts, caps, x, mu, step, dims, precision="fp32c", return_steps=True)
    assert np.quantile(np.abs(res[:, 0] - ref[:, 0]), 0.99) <= 1e-4
    rel = np.abs(res[:, 1] - ref[:, 1]) / np.maximum(np.abs(ref[:, 1]), 1e-12)
    assert np.quantile(rel, 0.99) <= 1e-2
    assert (steps == ref_steps).mean() >= 0.97


def test_dipole_reference_golden(gpu_lib, golden):
    from pycpet_gb300 import topo_dipole_lines

    t = golden("ref_topo_dipole.npz")
    R = t["result"]
    for prec in ("fp64", "fp32c"):
        res = topo_dipole_lines(t["starts"], t["caps"], t["x"], t["mu"], float(t["step"]), t["dims"],
                                precision=prec)
        assert np.abs(res[:, 0] - R[:, 0]).max() < 1e-5
        rel = np.abs(res[:, 1] - R[:, 1]) / np.abs(R[:, 1])
        assert np.median(rel) < 5e-3 and rel.max() < 5e-2


def test_dipole_axis_line_and_slot_variants(gpu_lib):
    """A dipole along +x at (10, 0, 0): the line from the origin runs straight
    along +x in steps of 0.125 and stops at the first position beyond the
    half-width 1.05 (1.125, step 9; the half-width sits between two steps so
    a last-bit difference in the step vector cannot move the exit); results
    do not depend on the line-slot variant."""
    from pycpet_gb300 import autotune, topo_dipole_lines

    x, mu = np.array([[10.0, 0.0, 0.0]]), np.array([[1.0, 0.0, 0.0]])
    for prec in ("fp64", "fp32c"):
        res, ends, steps = topo_dipole_lines(np.zeros((1, 3)), [1000], x, mu, 0.125, [1.05] * 3, precision=prec,
                                             return_ends=True, return_steps=True)
        assert steps[0] == 9
        np.testing.assert_allclose(ends[0], [1.125, 0.0, 0.0], atol=1e-6)
        assert abs(res[0, 1]) < 1e-6
    x, mu, starts, caps, dims, step = _case(1500, 500, 97, step=0.02)
    k = autotune.key(autotune.OP_TOPO, "fp32c", 1, len(starts))
    out = []
    for v in range(2):
        autotune.set_variant(k, v)
        out.append(topo_dipole_lines(starts, caps, x, mu, step, dims, precision="fp32c"))
    autotune.set_variant(k, -1)
    np.testing.assert_array_equal(out[0], out[1])


def test_dipole_drop_ins(gpu_lib, golden):
    """c_ops.Math_ops.thread_operation_dipole, calculator.calculate_thread_c_shared_dipole
    and the calculator method compute_topo_complete_c_shared_dipole."""
    import torch
    from pycpet_gb300 import calculator, topo_dipole_lines
    from pycpet_gb300.c_ops import Math_ops
    from pycpet_gb300.drop_in import Calculator

    t = golden("ref_topo_dipole.npz")
    x, mu, starts, caps = t["x"], t["mu"], t["starts"], t["caps"]
    m = Math_ops(precision="fp64")
    one = m.thread_operation_dipole(starts[0], caps[0], x, mu, t["step"], t["dims"])
    assert abs(one[0] - t["result"][0, 0]) < 1e-5
    two = calculator.calculate_thread_c_shared_dipole(starts[1], caps[1], x, mu, t["step"], t["dims"])
    assert abs(two[0] - t["result"][1, 0]) < 1e-5
    calc = Calculator.__new__(Calculator)
    calc.x, calc.mu, calc.precision = x, mu, "fp32c"
    calc.random_start_points, calc.random_max_samples = starts, caps
    calc.step_size, calc.dimensions = float(t["step"]), t["dims"]
    hist = calc.compute_topo_complete_c_shared_dipole()
    assert hist.dtype == np.float32 and hist.shape == (len(starts), 2)
    assert np.abs(hist[:, 0] - t["result"][:, 0]).max() < 1e-5
    d = topo_dipole_lines(torch.from_numpy(starts.astype(np.float64)).cuda(), torch.from_numpy(caps).cuda(),
                          torch.from_numpy(x.astype(np.float64)).cuda(), torch.from_numpy(mu.astype(np.float64)).cuda(),
                          float(t["step"]), t["dims"], precision="fp32c")
    np.testing.assert_array_equal(d.cpu().numpy().astype(np.float32), hist)
