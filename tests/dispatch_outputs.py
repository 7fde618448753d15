"""Output files of PyCPET's dispatcher (CPET/source/CPET.py) written from the
calculator methods of this package, and their comparison with the files the
reference's own dispatcher wrote (tests/golden/ref_dispatch.npz, made by
tests/golden/make_golden.py:ref_dispatch).

The writers follow the dispatcher's steps:
  point_field  "{protein}:{E}\\n" per frame              CPET.py:172-189
  volume       save_numpy_as_dat(compute_box() ...)     CPET.py:148-166
  volume_ESP   save_numpy_as_dat(compute_box_ESP() ...) CPET.py:207-225
  topo         np.savetxt(protein.top, hist)            CPET.py:119-123
"""
import io
import os

import numpy as np

METHODS = ("point_field", "volume", "volume_ESP", "topo")
PROTEIN = "1_alcdehydro_run1"


def fixture_files(g, method):
    pre = f"{method}/file/"
    return {k[len(pre):]: bytes(g[k]) for k in g.files if k.startswith(pre)}


def write_outputs(method, calc, outdir, gpu_savetxt=False):
    """The dispatcher's output step for one frame, from `calc`'s methods
    (.top files with numpy.savetxt, or with the GPU savetxt drop-in)."""
    from pycpet_gb300.calculator import save_numpy_as_dat, savetxt

    os.makedirs(outdir, exist_ok=True)
    if method == "point_field":
        with open(os.path.join(outdir, "point_field.dat"), "w") as f:
            f.write("{}:{}\n".format(PROTEIN, calc.compute_point_field()))
    elif method in ("volume", "volume_ESP"):
        box, shape = calc.compute_box() if method == "volume" else calc.compute_box_ESP()
        meta = {"dimensions": calc.dimensions, "step_size": [calc.step_size] * 3,
                "num_steps": [shape[0], shape[1], shape[2]],
                "transformation_matrix": calc.transformation_matrix, "center": calc.center}
        suffix = "_efield.dat" if method == "volume" else "_esp.dat"
        save_numpy_as_dat(name=os.path.join(outdir, PROTEIN + suffix), volume=box, meta_data=meta)
    else:
        (savetxt if gpu_savetxt else np.savetxt)(os.path.join(outdir, PROTEIN + ".top"),
                                                 calc.compute_topo_complete_c_shared())
    files = {}
    for f in sorted(os.listdir(outdir)):
        with open(os.path.join(outdir, f), "rb") as fh:
            files[f] = fh.read()
    return files


def _rows(data, skip=0):
    return np.loadtxt(io.BytesIO(data), skiprows=skip, ndmin=2)


def compare(method, mine, ref):
    """Asserts that `mine` holds the same files as `ref` with the same values:
    headers byte for byte; numbers within the rounding of the reference's
    float32 arithmetic and of the files' text formats."""
    assert sorted(mine) == sorted(ref), (sorted(mine), sorted(ref))
    for name, data in ref.items():
        got = mine[name]
        if method == "point_field":
            a = [line.split(":", 1) for line in got.decode().splitlines()]
            b = [line.split(":", 1) for line in data.decode().splitlines()]
            assert [k for k, _ in a] == [k for k, _ in b]
            for (_, va), (_, vb) in zip(a, b):
                va = np.array(va.strip("[] ").split(), float)
                vb = np.array(vb.strip("[] ").split(), float)
                np.testing.assert_allclose(va, vb, rtol=0, atol=1e-5 * np.abs(vb).max())
        elif method in ("volume", "volume_ESP"):
            assert got.split(b"\n")[:7] == data.split(b"\n")[:7]      # the seven header lines
            a, b = _rows(got, 7), _rows(data, 7)
            assert a.shape == b.shape
            np.testing.assert_array_equal(a[:, :3], b[:, :3])          # grid coordinates
            # 3-decimal text of float32 (field) or float16 (potential) values
            ulp = 0.0 if method == "volume" else np.spacing(np.abs(b[:, 3:]).astype(np.float16)).astype(float)
            assert np.all(np.abs(a[:, 3:] - b[:, 3:]) <= 1.0001e-3 + 1e-5 * np.abs(b[:, 3:]) + ulp)
        else:
            a, b = _rows(got), _rows(data)
            assert a.shape == b.shape
            close = np.abs(a[:, 0] - b[:, 0]) <= 1e-4
            assert close.mean() >= 0.95, close.mean()     # same lines, same step counts
            # sorted (distance, curvature) pairs, the reference's own test convention
            # (CPET tests/test_topology.py: rtol = atol = 1e-2)
            np.testing.assert_allclose(np.sort(a, axis=0), np.sort(b, axis=0), rtol=1e-2, atol=1e-2)
