"""GPU text formatting of volume outputs (cpetgb_format_fixed3 and the
save_numpy_as_dat drop-in) against numpy.savetxt(fmt="%.3f") — the function
the reference's writer calls (CPET/utils/io.py:50-109) — and against the
reference writer's own files (tests/golden/ref_dat.npz).  Bit-exact bytes."""
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _savetxt(a):
    sink = io.BytesIO()
    np.savetxt(sink, a, fmt="%.3f")
    return sink.getvalue()


def test_save_numpy_as_dat_matches_reference_files(gpu_lib, golden, tmp_path):
    from pycpet_gb300.calculator import save_numpy_as_dat

    d, g = golden("ref_dat.npz"), golden("ref_grid.npz")
    meta = {"dimensions": d["dimensions"], "num_steps": list(d["num_steps"]), "transformation_matrix": d["T"],
            "center": d["center"]}
    for key, vol in (("field", g["field"]), ("esp", g["esp_half"])):
        path = tmp_path / f"{key}.dat"
        save_numpy_as_dat(meta, vol, str(path))
        assert path.read_bytes() == bytes(d[f"{key}_dat"])


def test_fixed3_adversarial_values(gpu_lib):
    """Exact decimal ties (round half to even), negative values that round to
    zero, signed zeros, the 2^24 boundary, huge integers, NaN and infinities."""
    from pycpet_gb300.core import format_fixed3

    f = np.float32
    special = np.array([0.0625, 0.1875, 2.5e-4, 0.0005, 1.0005, -0.0004, -0.0, 0.0, 0.9995, -0.0625,
                        16777215.0, 16777216.0, 16777218.0, 3.4028235e38, -3.4028235e38, 1.1754944e-38,
                        1e-45, 123456.789, -99999.9995, np.nan, np.inf, -np.inf, 1e9, -2.5e15], dtype=f)
    rng = np.random.default_rng(1)
    mags = 10.0 ** rng.uniform(-9, 12, 20000)
    rnd = (mags * rng.choice([-1.0, 1.0], 20000)).astype(f)
    ties = (rng.integers(-200000, 200000, 20000) / 16.0).astype(f)  # k/16: many exact x.xxx5 ties
    for a in (special.reshape(-1, 4), rnd.reshape(-1, 5), ties.reshape(-1, 1), special):
        assert format_fixed3(a) == _savetxt(a), a[:4]
    h = rng.normal(0, 30, (300, 4)).astype(np.float16)
    assert format_fixed3(h) == _savetxt(h)


def test_fixed3_volume_sized(gpu_lib):
    """A 51^3-point field volume (the largest serving volume): same bytes."""
    from pycpet_gb300.core import format_fixed3

    rng = np.random.default_rng(2)
    g = np.linspace(-2.5, 2.5, 51, dtype=np.float32)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    vol = np.concatenate([pts, rng.normal(0, 5, (len(pts), 3)).astype(np.float32)], axis=1)
    assert format_fixed3(vol) == _savetxt(vol)
    assert format_fixed3(np.zeros((0, 6), np.float32)) == b""
