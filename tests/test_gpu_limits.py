"""Size limits and refusals of the streamline path on the GPU: frames exactly
at and just above the shared-memory residency limit (charges and dipoles take
different kernels there, with the same results within the FP32C tolerance),
negative and oversized step caps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frame(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-60.0, 60.0, (3 * n, 3))
    x = x[np.linalg.norm(x, axis=1) > 3.0][:n]
    return x, rng.normal(0.0, 0.4, n), rng.normal(0.0, 0.3, (n, 3))


@pytest.mark.parametrize("dipoles", [False, True])
def test_residency_boundary(gpu_lib, oracle, dipoles):
    from pycpet_gb300 import _lib, topo_dipole_lines, topo_lines
    from pycpet_gb300.synth import random_start_points

    limit = _lib.lib().cpetgb_topo_resident_limit(_lib.FP32C, int(dipoles))
    assert limit > 0
    starts = random_start_points(24, [1.5] * 3, 5)
    caps = np.full(24, 60, np.int32)
    for n in (limit, limit + 1):
        x, q, mu = _frame(n, n)
        if dipoles:
            res, steps = topo_dipole_lines(starts, caps, x, mu, 0.02, [1.5] * 3, precision="fp32c",
                                           return_steps=True)
            ref, _, ref_steps = oracle.topo_lines_dipole(starts, caps, x, mu, 0.02, [1.5] * 3)
        else:
            res, steps = topo_lines(starts, caps, x, q, 0.02, [1.5] * 3, precision="fp32c", return_steps=True)
            ref, _, ref_steps = oracle.topo_lines_f64(starts, caps, x, q, 0.02, [1.5] * 3)
        assert (steps == ref_steps).mean() >= 0.95
        assert np.quantile(np.abs(res[:, 0] - ref[:, 0]), 0.9) <= 1e-4


def test_step_caps(gpu_lib):
    """Negative caps run no step (the end point is the start point); a cap
    above 2^24 is refused with an error instead of a multi-hour kernel."""
    from pycpet_gb300 import CpetgbError, topo_lines

    x, q, _ = _frame(500, 3)
    starts = np.zeros((2, 3))
    res, steps = topo_lines(starts, [-5, 0], x, q, 0.01, [1.0] * 3, precision="fp32c", return_steps=True)
    np.testing.assert_array_equal(steps, [0, 0])
    assert np.all(res[:, 0] == 0.0)
    with pytest.raises(CpetgbError) as e:
        topo_lines(starts, [10, (1 << 24) + 1], x, q, 0.01, [1.0] * 3, precision="fp32c")
    assert "step cap exceeds" in str(e.value)
    # the library stays usable after the refusal
    res = topo_lines(starts, [10, 10], x, q, 0.01, [1.0] * 3, precision="fp32c")
    assert np.all(np.isfinite(res))
