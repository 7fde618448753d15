"""Serving loop: each request's result is the same alone and in a mix of
concurrent requests (streamlines bit-identical; grid sums within the FP32C
tolerance, since batching changes how the charge sums are split), requests
overlap on the device, and admission retries when the engine is full."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frames():
    from pycpet_gb300.synth import make_frame

    return {i: make_frame(n, 500 + i) for i, n in enumerate([2000, 8000, 20000])}


def _requests(seed=0):
    from pycpet_gb300.serving import Request

    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(4):
        L = int(rng.integers(300, 1500))
        reqs.append(Request("topo", i % 3, 0.0, starts=rng.uniform(-1.5, 1.5, (L, 3)),
                            n_iter=rng.integers(0, 400, L).astype(np.int32), step=0.01))
    for i in range(3):
        g = np.linspace(-1.0, 1.0, 11 + 10 * i)
        pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        reqs.append(Request("volume", i % 3, 0.0, points=pts))
        reqs.append(Request("volume_esp", (i + 1) % 3, 0.0, points=pts))
    for i in range(4):
        reqs.append(Request("point_field", i % 3, 0.0, points=rng.uniform(-1, 1, (int(rng.integers(1, 65)), 3))))
    return reqs


def _clone(r):
    from dataclasses import replace

    return replace(r, result=None, t_start=None, t_done=None, _rid=-1)


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_same_alone_and_in_mix(gpu_lib, precision):
    from pycpet_gb300 import esp_grid, field_grid, topo_lines
    from pycpet_gb300.serving import Server

    frames = _frames()
    srv = Server(precision=precision, line_capacity=200_000, charge_capacity=200_000, max_requests=64)
    for fid, fr in frames.items():
        srv.add_frame(fid, fr["x"], fr["q"])
    base = _requests()
    alone = []
    for r in base:
        a = _clone(r)
        srv.run([a])
        alone.append(a)
    mix = [_clone(r) for r in base]
    srv.run(mix)
    assert srv.max_topo_inflight >= 2          # streamline requests overlapped in the engine
    for a, m in zip(alone, mix):
        fr = frames[a.frame]
        if a.kind == "topo":
            np.testing.assert_array_equal(m.result, a.result)
            direct = topo_lines(a.starts, a.n_iter, fr["x"], fr["q"], a.step, a.half_dims, precision=precision)
            np.testing.assert_array_equal(a.result, direct)
        else:
            if a.kind == "volume_esp":
                direct = esp_grid(a.points, fr["x"], fr["q"], precision=precision)
            else:
                direct = field_grid(a.points, fr["x"], fr["q"], precision=precision, clamp=(a.kind == "volume"))
            np.testing.assert_array_equal(a.result, direct)
            tol = 1e-12 if precision == "fp64" else 2e-6
            assert np.abs(m.result - a.result).max() <= tol * np.abs(a.result).max()
    srv.close()


def test_engine_on_whole_sms(gpu_lib):
    """Two engine CTAs per SM (whole SMs for streamlines): results identical
    to cpetgb_topo_lines; a third value is refused."""
    from pycpet_gb300 import _lib, topo_lines
    from pycpet_gb300.serving import Request, Server

    frames = _frames()
    srv = Server(line_capacity=100_000, charge_capacity=100_000, max_requests=64, engine_ctas_per_sm=2)
    for fid, fr in frames.items():
        srv.add_frame(fid, fr["x"], fr["q"])
    rng = np.random.default_rng(11)
    reqs = []
    for i in range(6):
        L = int(rng.integers(50, 3000))
        reqs.append(Request("topo", i % 3, 0.0, starts=rng.uniform(-1.5, 1.5, (L, 3)),
                            n_iter=rng.integers(0, 300, L).astype(np.int32), step=0.01))
    srv.run(reqs)
    for r in reqs:
        fr = frames[r.frame]
        np.testing.assert_array_equal(r.result, topo_lines(r.starts, r.n_iter, fr["x"], fr["q"], r.step, r.half_dims))
    assert _lib.lib().cpetgb_engine_set_ctas_per_sm(srv.engine, 3) == _lib.EINVAL
    srv.close()


@pytest.mark.parametrize("ctas_per_sm", [1, 2])
def test_burst_right_after_a_run_uses_every_warp(gpu_lib, ctas_per_sm):
    """A burst submitted while the previous engine launch is still alive (its
    warps idle after a small request) is served by all of that launch's warps:
    it takes about as long as the same burst on an engine that had ended
    (a launch whose idle warps had left served such a burst with its few busy
    warps, several times slower), with identical results."""
    import time

    from pycpet_gb300 import _lib, topo_lines
    from pycpet_gb300.serving import Request, Server

    fr = _frames()[1]
    srv = Server(line_capacity=200_000, charge_capacity=100_000, max_requests=256, engine_ctas_per_sm=ctas_per_sm)
    srv.add_frame(0, fr["x"], fr["q"])
    rng = np.random.default_rng(3)
    base = [Request("topo", 0, 0.0, starts=rng.uniform(-1.5, 1.5, (600, 3)), n_iter=2000, step=0.001)
            for _ in range(40)]
    # a few long lines (about 20,000 steps of 1e-4 A): the launch outlives the
    # 50 ms idle period of its other warps
    small = Request("topo", 0, 0.0, starts=rng.uniform(-0.2, 0.2, (8, 3)), n_iter=20000, step=0.0001)

    def timed(reqs):
        t0 = time.perf_counter()
        srv.run(reqs)
        return time.perf_counter() - t0

    timed([_clone(r) for r in base])                      # warm-up
    _lib.check(_lib.lib().cpetgb_engine_drain(srv.engine))
    cold = [_clone(r) for r in base]
    t_cold = timed(cold)                                  # on an engine that had ended
    _lib.check(_lib.lib().cpetgb_engine_drain(srv.engine))
    srv.run([_clone(small)])
    hot = [_clone(r) for r in base]
    t_hot = timed(hot)                                    # right after a small run
    srv.close()
    for a, b in zip(cold, hot):
        np.testing.assert_array_equal(a.result, b.result)
    r0 = base[0]
    np.testing.assert_array_equal(hot[0].result, topo_lines(r0.starts, r0.n_iter, fr["x"], fr["q"], r0.step,
                                                            r0.half_dims))
    assert t_hot < 2.0 * t_cold + 0.1, (t_hot, t_cold)


def test_admission_retries_when_full(gpu_lib):
    """A line store smaller than the queued work: requests wait for capacity
    and all finish with the right results."""
    from pycpet_gb300 import topo_lines
    from pycpet_gb300.serving import Request, Server

    frames = _frames()
    srv = Server(line_capacity=2500, charge_capacity=100_000, max_requests=64)
    srv.add_frame(0, frames[0]["x"], frames[0]["q"])
    rng = np.random.default_rng(7)
    reqs = [Request("topo", 0, 0.001 * i, starts=rng.uniform(-1.5, 1.5, (1000, 3)), n_iter=300, step=0.01)
            for i in range(6)]
    srv.run(reqs)
    for r in reqs:
        np.testing.assert_array_equal(
            r.result, topo_lines(r.starts, r.n_iter, frames[0]["x"], frames[0]["q"], r.step, r.half_dims))
    srv.close()


def test_grid_requests_run_beside_the_streamline_engine(gpu_lib):
    """With the engine at one CTA per SM busy on a long streamline request,
    volume (refined FP32C field), potential and point requests submitted after
    it finish while the streamline request is still running: every kernel of
    the grid path fits in the half of each SM the engine leaves free."""
    import time

    from pycpet_gb300.serving import Request, Server
    from pycpet_gb300.synth import make_frame

    srv = Server(precision="fp32c", line_capacity=100_000, charge_capacity=50_000, max_requests=64,
                 engine_ctas_per_sm=1)
    try:
        fr = make_frame(20000, seed=71)
        srv.add_frame(0, fr["x"], fr["q"])
        rng = np.random.default_rng(72)
        topo = Request("topo", 0, 0.0, starts=rng.uniform(-1.5, 1.5, (40_000, 3)), n_iter=6000, step=0.001)
        g = np.linspace(-1.0, 1.0, 21)
        pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        grid = [Request(k, 0, 0.0, points=pts) for k in ("volume", "volume_esp")]
        grid.append(Request("point_field", 0, 0.0, points=pts[:20]))
        now = time.perf_counter()
        for r in [topo] + grid:
            r.arrival = now
            assert srv.submit(r)
        t_end = time.perf_counter() + 60
        while any(r.status != "done" for r in grid) and time.perf_counter() < t_end:
            srv.step()
        assert all(r.status == "done" for r in grid)
        assert topo.status == "running", "the grid requests waited for the streamline request"
        while srv.busy() and time.perf_counter() < t_end:
            srv.step()
        assert topo.status == "done"
    finally:
        srv.close()
