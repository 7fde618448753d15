"""The calculator methods of pycpet_gb300.drop_in on the GPU, given the state
the reference's calculator held for one frame of example 1A (charges after
parsing, filtering and rotation; mesh; start points and caps), write through
the dispatcher's output steps the same files as the reference's own
CPET(options).run() (tests/golden/ref_dispatch.npz; comparison rules in
dispatch_outputs.py)."""
import types

import pytest

import dispatch_outputs as D

pytestmark = pytest.mark.gpu


def _state(g, method, precision):
    s = types.SimpleNamespace(precision=precision)
    pre = method + "/"
    for k in g.files:
        if k.startswith(pre) and "/file/" not in k:
            setattr(s, k[len(pre):], g[k])
    s.Q = s.Q.reshape(-1, 1)
    if method == "topo":
        s.random_start_points, s.random_max_samples = s.starts, s.caps
        s.n_samples = len(s.starts)
    if hasattr(s, "step_size"):
        s.step_size = float(s.step_size)
    return s


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_dispatcher_outputs_from_gpu_methods(gpu_lib, golden, tmp_path, precision):
    from pycpet_gb300 import drop_in

    g = golden("ref_dispatch.npz")
    for m in D.METHODS:
        calc = _state(g, m, precision)
        for name in drop_in.HOT_METHODS:           # what patch_pycpet() installs on the class
            setattr(calc, name, getattr(drop_in, name).__get__(calc))
        files = D.write_outputs(m, calc, str(tmp_path / precision / m))
        D.compare(m, files, D.fixture_files(g, m))
        if m == "topo":   # the .top writer on the GPU: numpy's bytes
            gpu = D.write_outputs(m, calc, str(tmp_path / precision / "gpu_top"), gpu_savetxt=True)
            assert gpu == files
