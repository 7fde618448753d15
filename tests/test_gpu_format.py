"""GPU text formatting of volume and topology outputs, bit-exact bytes:
cpetgb_format_fixed3 and the save_numpy_as_dat drop-in against
numpy.savetxt(fmt="%.3f") -- the function the reference's writer calls
(CPET/utils/io.py:50-109) -- and the reference writer's own files
(tests/golden/ref_dat.npz); cpetgb_format_sci18 and the savetxt drop-in
against numpy.savetxt's default "%.18e" (the .top files,
CPET/source/CPET.py:123) and example 3A's shipped .top files."""
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


def _savetxt_default(a):
    sink = io.BytesIO()
    np.savetxt(sink, a)
    return sink.getvalue()


def test_sci18_random_bit_patterns(gpu_lib):
    """numpy.savetxt's default "%.18e" on 200,000 float32 values drawn as raw
    bit patterns (every exponent, subnormals, NaNs of both signs, infinities)."""
    from pycpet_gb300.core import format_sci18

    rng = np.random.default_rng(5)
    a = rng.integers(0, 2 ** 32, 200_000, dtype=np.uint64).astype(np.uint32).view(np.float32).reshape(-1, 2)
    assert format_sci18(a) == _savetxt_default(a)


def test_sci18_adversarial_values(gpu_lib):
    """Exact decimal ties at the 19th digit (every float32 in [32, 64) with an
    odd significand is one; round half to even), values next to powers of ten,
    the extremes, signed zeros, subnormals, NaN and infinities."""
    from pycpet_gb300.core import format_sci18

    f = np.float32
    rng = np.random.default_rng(6)
    ties = rng.uniform(16.0, 64.0, 20_000).astype(f)
    near = []
    for n in range(-45, 39):
        v = f(10.0 ** n)
        for k in range(-2, 3):
            w = v
            for _ in range(abs(k)):
                w = np.nextafter(w, f(np.inf) if k > 0 else f(0.0))
            near.append(w)
    near = np.array(near, dtype=f)
    special = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 0.1, 1e10, 1e-10, 3.4028235e38, -3.4028235e38,
                        1.1754944e-38, 1e-45, -1e-45, 2 ** -149, 9.999999e18, 1e19, 1.0000001e19,
                        np.nan, -np.nan, np.inf, -np.inf, 16777216.0, 8388607.5, 123456.789], dtype=f)
    for a in (ties.reshape(-1, 2), near.reshape(-1, 1), special.reshape(-1, 2), special):
        assert format_sci18(a) == _savetxt_default(a), a[:4]


def test_top_writer_reproduces_example_files(gpu_lib, golden, tmp_path):
    """The .top files example 3A ships (np.savetxt of float32 (distance,
    curvature) rows, CPET/source/CPET.py:123), byte for byte, through the
    savetxt drop-in; other dtypes and arguments go to numpy itself."""
    from pycpet_gb300.calculator import savetxt

    g = golden("examples_topology.npz")
    for i in range(2):
        rows = g[f"top{i}"].astype(np.float32)      # the files' values, exact in float32
        path = tmp_path / f"frame{i}.top"
        savetxt(str(path), rows)
        assert path.read_bytes() == bytes(g[f"top{i}_bytes"])
    rows64 = g["top0"][:50]
    sink = io.BytesIO()
    savetxt(sink, rows64)
    assert sink.getvalue() == _savetxt_default(rows64)
    sink = io.BytesIO()
    savetxt(sink, rows, fmt="%.4f")
    ref = io.BytesIO()
    np.savetxt(ref, rows, fmt="%.4f")
    assert sink.getvalue() == ref.getvalue()
