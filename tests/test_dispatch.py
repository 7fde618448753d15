"""The reference's own dispatcher, CPET(options).run(), with this package's
calculator methods installed by patch_pycpet(): every output file it writes
must match the files of the unpatched reference (tests/golden/ref_dispatch.npz).

This is host-side glue: the calculator state the methods read (self.x,
self.Q, self.mesh, self.random_start_points, ...), the return shapes and
dtypes the dispatcher's writers expect.  It runs where the reference checkout
is present (CPETGB_REF, default /root/reference) and needs no GPU: the three
device calls the methods make are replaced here by the FP64 test oracle.
It runs twice: with the dispatcher's own writers, and with
patch_pycpet(gpu_writers=True) installing this package's save_numpy_as_dat and
savetxt (their GPU text formatting replaced by numpy's here).  The same outputs
from the GPU are checked in test_gpu_dispatch.py.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
import dispatch_outputs as D

REF = os.environ.get("CPETGB_REF", "/root/reference")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "math_module.so")


def test_reference_dispatcher_with_drop_in_methods(oracle, golden, monkeypatch, tmp_path):
    if not os.path.isdir(os.path.join(REF, "CPET")) or not os.path.exists(REF_SO):
        pytest.skip(f"reference checkout or its library not present (CPETGB_REF={REF})")
    sys.path.insert(0, GOLDEN)
    import make_golden as mg
    from pycpet_gb300 import drop_in

    _, scalc = mg.import_reference(REF)

    def field_grid(points, x, q, precision=None, clamp=True):
        return oracle.field_grid_f64(points, x, q, clamp=clamp)

    def esp_grid(points, x, q, precision=None):
        return oracle.esp_grid_f64(points, x, q)

    def topo_lines(starts, caps, x, q, step, half, precision=None):
        return oracle.topo_lines_f64(starts, caps, x, q, step, half)[0]

    monkeypatch.setattr(drop_in, "field_grid", field_grid)
    monkeypatch.setattr(drop_in, "esp_grid", esp_grid)
    monkeypatch.setattr(drop_in, "topo_lines", topo_lines)
    # the text writers' GPU formatting, replaced by numpy's own (the bytes the
    # GPU writers must produce) so the writer glue runs here too
    import io

    from pycpet_gb300 import calculator as C

    def text(fmt):
        def f(values):
            sink = io.BytesIO()
            np.savetxt(sink, np.asarray(values).reshape(len(values), -1), fmt=fmt)
            return sink.getvalue()
        return f

    monkeypatch.setattr(C, "format_fixed3", text("%.3f"))
    monkeypatch.setattr(C, "format_sci18", text("%.18e"))
    from CPET.source import CPET as dispatcher

    cls = scalc.calculator
    saved = {n: cls.__dict__[n] for n in drop_in.HOT_METHODS if n in cls.__dict__}
    saved_writers = (dispatcher.np, dispatcher.save_numpy_as_dat)
    try:
        g = golden("ref_dispatch.npz")
        for writers in (False, True):
            assert drop_in.patch_pycpet("fp64", gpu_writers=writers) is cls
            assert (dispatcher.save_numpy_as_dat is C.save_numpy_as_dat) == writers
            for m in D.METHODS:
                files = mg.run_dispatcher(m, os.path.join(REF, mg.DISPATCH_PDB), str(tmp_path / f"{m}{writers}"))
                D.compare(m, files, D.fixture_files(g, m))
    finally:
        dispatcher.np, dispatcher.save_numpy_as_dat = saved_writers
        for n in drop_in.HOT_METHODS:
            if n in saved:
                setattr(cls, n, saved[n])
            elif n in cls.__dict__:
                delattr(cls, n)
        if "precision" in cls.__dict__:
            delattr(cls, "precision")
