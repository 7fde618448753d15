"""The allocation-free streamline entry point, called through the C ABI.

Callers whose device memory is reserved up front by their own allocator, or who
forbid allocation after start-up, use cpetgb_topo_lines_noalloc: its scratch is
a fixed array inside the library instead of memory allocated per call.  This
checks it against the allocating entry point (cpetgb_topo_lines on device
buffers) on the same inputs, twice in a row so that leftovers of the first call
in the shared array cannot go unnoticed, in both precision forms, and that a
frame larger than the fixed array is refused with a clear error.

This file is collected last on purpose; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(n_charges, n_lines, seed):
    from pycpet_gb300.synth import make_frame, random_start_points

    fr = make_frame(n_charges, seed)
    starts = random_start_points(n_lines, [1.5] * 3, seed + 1)
    caps = np.random.default_rng(seed + 2).integers(0, 400, n_lines).astype(np.int32)
    return fr["x"], fr["q"], starts, caps


def _noalloc(lib, prec, d_starts, d_caps, d_x, d_q, step, half, stream):
    import torch

    L = d_starts.shape[0]
    res = torch.full((L, 2), float("nan"), dtype=torch.float64, device=d_starts.device)
    ends = torch.full((L, 3), float("nan"), dtype=torch.float64, device=d_starts.device)
    steps = torch.full((L,), -7, dtype=torch.int32, device=d_starts.device)
    rc = lib.cpetgb_topo_lines_noalloc(prec, L, d_q.numel(), d_starts.data_ptr(), d_caps.data_ptr(), step,
                                       half.ctypes.data, d_x.data_ptr(), d_q.data_ptr(), res.data_ptr(),
                                       ends.data_ptr(), steps.data_ptr(), stream)
    return rc, res, ends, steps


@pytest.mark.parametrize("n_charges", [3000, 16000])
def test_noalloc_matches_allocating_entry_point(gpu_lib, n_charges):
    import torch
    from pycpet_gb300 import _lib, topo_lines

    x, q, starts, caps = _inputs(n_charges, 1500, 90 + n_charges)
    dev = torch.device("cuda", 0)
    d_x, d_q = torch.from_numpy(x).to(dev), torch.from_numpy(q).to(dev)
    d_starts, d_caps = torch.from_numpy(starts).to(dev), torch.from_numpy(caps).to(dev)
    half = np.array([1.5, 1.5, 1.5])
    stream = torch.cuda.current_stream(dev).cuda_stream
    for prec_name, prec in (("fp32c", _lib.FP32C), ("fp64", _lib.FP64)):
        ref_res, ref_ends, ref_steps = topo_lines(d_starts, d_caps, d_x, d_q, 0.01, half, precision=prec_name,
                                                  return_ends=True, return_steps=True)
        torch.cuda.synchronize()
        for _ in range(2):
            rc, res, ends, steps = _noalloc(gpu_lib, prec, d_starts, d_caps, d_x, d_q, 0.01, half, stream)
            assert rc == 0, _lib.last_error()
            np.testing.assert_array_equal(steps.cpu().numpy(), ref_steps.cpu().numpy())
            # same kernels on the same inputs: equal within the FP64 parity tolerance of the other tests
            np.testing.assert_allclose(res.cpu().numpy(), ref_res.cpu().numpy(), rtol=1e-12, atol=1e-12)
            np.testing.assert_allclose(ends.cpu().numpy(), ref_ends.cpu().numpy(), rtol=0, atol=1e-12)


def test_noalloc_refuses_frames_beyond_its_array(gpu_lib):
    import torch
    from pycpet_gb300 import _lib

    dev = torch.device("cuda", 0)
    n = 16385
    d_x = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    d_q = torch.zeros((n,), dtype=torch.float64, device=dev)
    d_starts = torch.zeros((4, 3), dtype=torch.float64, device=dev)
    d_caps = torch.ones((4,), dtype=torch.int32, device=dev)
    rc, res, _, _ = _noalloc(gpu_lib, _lib.FP32C, d_starts, d_caps, d_x, d_q, 0.01, np.ones(3),
                             torch.cuda.current_stream(dev).cuda_stream)
    assert rc == _lib.EINVAL
    assert "16384" in _lib.last_error()
    assert torch.isnan(res).all()          # nothing was written
