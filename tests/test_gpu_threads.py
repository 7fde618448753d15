"""Math_ops objects of different precisions used from two threads at once:
each call carries its own precision (the *_p entry points), so every result
equals the one the same object gives when it runs alone."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_math_ops_precisions_from_two_threads(gpu_lib, golden):
    from pycpet_gb300.c_ops import Math_ops

    g = dict(golden("ref_grid.npz"))      # arrays read once: the archive is not thread-safe
    t = dict(golden("ref_topo.npz"))
    pts = g["mesh"].reshape(-1, 3)
    objs = {"fp64": Math_ops(precision="fp64"), "fp32c": Math_ops(precision="fp32c")}

    def work(M):
        return (M.compute_looped_field(pts, g["x"], g["Q"].reshape(-1, 1)),
                M.thread_operation_batch(t["starts"][:64], t["caps"][:64], t["x"], t["Q"], float(t["step"]),
                                         t["dims"]),
                M.calc_field(np.zeros(3, np.float32), g["x"], g["Q"]))

    alone = {k: work(M) for k, M in objs.items()}
    # the two forms differ, so a call run in the other object's precision would show
    assert not np.array_equal(alone["fp64"][0], alone["fp32c"][0])
    errors, results = [], {k: [] for k in objs}

    def loop(key):
        try:
            for _ in range(12):
                results[key].append(work(objs[key]))
        except Exception as e:  # reported below
            errors.append(e)

    th = [threading.Thread(target=loop, args=(k,)) for k in objs for _ in range(2)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors, errors
    for key, runs in results.items():
        assert len(runs) == 24
        for r in runs:
            for a, b in zip(r, alone[key]):
                np.testing.assert_array_equal(a, b)
