"""Failure handling without a GPU fault: a device-side wait that runs out is
reported as CPETGB_ETIMEOUT and leaves the device usable; the serving loop
refuses requests that can never run and cancels requests pending past their
deadline, while valid ones complete."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_device_stays_usable(gpu_lib):
    from pycpet_gb300 import _lib, field_grid

    L = _lib.lib()
    t0 = time.perf_counter()
    assert L.cpetgb_check_wait_limit(0.05) == _lib.ETIMEOUT
    assert time.perf_counter() - t0 < 1.5              # the 50 ms limit, not the kernels' 2 s
    assert "wait exceeded" in _lib.last_error()
    assert L.cpetgb_synchronize(None) == _lib.OK       # the status word was cleared
    for bad in (0.0, -1.0, 3.0, float("nan")):
        assert L.cpetgb_check_wait_limit(bad) == _lib.EINVAL
    E = field_grid(np.array([[1.0, 0, 0]]), np.zeros((1, 3)), np.array([1.0]), precision="fp64")
    np.testing.assert_allclose(E[0], [14.3996451, 0, 0], rtol=1e-15)


def test_server_refusals_watchdog_and_completion(gpu_lib):
    from pycpet_gb300.serving import Request, Server
    from pycpet_gb300.synth import make_frame

    srv = Server(line_capacity=20_000, charge_capacity=50_000, max_frames=4, max_requests=64,
                 pending_deadline_s=0.5)
    try:
        fr = make_frame(3000, seed=3)
        srv.add_frame(0, fr["x"], fr["q"])
        for x, q in ((np.zeros((0, 3)), np.zeros(0)), (np.array([[np.nan, 0, 0]]), np.ones(1))):
            with pytest.raises(ValueError):
                srv.add_frame(1, x, q)
        srv.budget = srv.resident_bytes + (1 << 20)       # 1 MiB beside the resident frame
        g = np.linspace(-0.5, 0.5, 11)
        small = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        big = np.zeros((30_000, 3))                        # 1.4 MB: more than the budget leaves
        now = time.perf_counter()
        ok = Request("volume", 0, now, points=small)
        reqs = [ok,
                Request("volume", 0, now, points=big),
                Request("topo", 0, now, starts=np.array([[0.1, np.nan, 0.0]]), n_iter=100),
                Request("volume", 5, now, points=small)]
        accepted = [srv.submit(r) for r in reqs]
        assert accepted == [True, False, False, False]
        assert [r.status for r in reqs[1:]] == ["rejected"] * 3
        assert "budget" in reqs[1].error and "finite" in reqs[2].error and "not resident" in reqs[3].error
        srv.step()                                         # admits and launches `ok`
        assert ok.status in ("running", "done")
        # two requests still waiting for admission 1 s after arriving are cancelled
        late = [Request("point_field", 0, now, points=small[:4]) for _ in range(2)]
        srv.pending.extend(late)
        for r in late:
            r.status = "pending"
        srv.step(now + 1.0)
        assert [r.status for r in late] == ["expired", "expired"]
        t_end = time.perf_counter() + 30
        while srv.busy() and time.perf_counter() < t_end:
            srv.step()
        assert ok.status == "done" and ok.result.shape == (len(small), 3)
        assert not srv.busy()
    finally:
        srv.close()
