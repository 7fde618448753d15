"""The headline streamline workload at full shape against the CPU FP64 oracle
of thread_operation (CPET/utils/math_module.c:523-591): one frame of 8,000
charges, step 0.001 A, cap 6,000 steps, on a strided sample of the 100,000
seeded start points, and the topology histogram of make_histograms
(CPET/utils/calculator.py:702-707: numpy.histogram2d, 20 x 20 bins over
distance [0, 5.2] and curvature [0, max]).

Tolerances of the FP32C form (stated here): end point p99 <= 1e-6 A, mean
curvature relative error p99 <= 1e-2, histogram L1 (normalised) <= 1e-3.
FP64 form: end points within 1e-9 A on lines with the oracle's step count.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STRIDE = 12          # 8,334 of the 100,000 lines


def test_fp32c_full_shape_against_oracle(gpu_lib, oracle):
    from pycpet_gb300 import topo_lines
    from pycpet_gb300.synth import TOPO_HALF, TOPO_STEP, topo_workload

    x, q, starts, caps = topo_workload()
    assert len(q) == 8000 and len(starts) == 100_000 and caps.max() == 6000
    idx = np.arange(0, len(starts), STRIDE)
    s, c = starts[idx], caps[idx]
    dims = [TOPO_HALF] * 3
    ref, ref_end, ref_steps = oracle.topo_lines_f64(s, c, x, q, TOPO_STEP, dims)
    res, ends, steps = topo_lines(s, c, x, q, TOPO_STEP, dims, precision="fp32c", return_ends=True,
                                  return_steps=True)
    end_err = np.linalg.norm(ends - ref_end, axis=1)
    assert np.quantile(end_err, 0.99) <= 1e-6, np.quantile(end_err, 0.99)
    curv_rel = np.abs(res[:, 1] - ref[:, 1]) / np.abs(ref[:, 1])
    assert np.quantile(curv_rel, 0.99) <= 1e-2, np.quantile(curv_rel, 0.99)
    rng = [[0.0, 5.2], [0.0, float(ref[:, 1].max())]]
    h_ref, _, _ = np.histogram2d(ref[:, 0], ref[:, 1], bins=[20, 20], range=rng)
    h, _, _ = np.histogram2d(res[:, 0], res[:, 1], bins=[20, 20], range=rng)
    l1 = np.abs(h / h.sum() - h_ref / h_ref.sum()).sum()
    assert l1 <= 1e-3, (l1, int((steps != ref_steps).sum()))


def test_fp64_full_shape_against_oracle(gpu_lib, oracle):
    from pycpet_gb300 import topo_lines
    from pycpet_gb300.synth import TOPO_HALF, TOPO_STEP, topo_workload

    x, q, starts, caps = topo_workload()
    idx = np.arange(0, len(starts), 391)[:256]
    s, c = starts[idx], caps[idx]
    dims = [TOPO_HALF] * 3
    ref, ref_end, ref_steps = oracle.topo_lines_f64(s, c, x, q, TOPO_STEP, dims)
    res, ends, steps = topo_lines(s, c, x, q, TOPO_STEP, dims, precision="fp64", return_ends=True,
                                  return_steps=True)
    same = steps == ref_steps
    assert same.mean() >= 0.99
    assert np.abs(ends[same] - ref_end[same]).max() <= 1e-9
