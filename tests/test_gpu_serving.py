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
