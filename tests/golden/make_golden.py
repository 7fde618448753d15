"""Generates the golden fixtures of tests/golden from the reference itself.

Needs a checkout of pujanajmera/pycpet (``--ref``, default: the CPETGB_REF
environment variable, else /root/reference) and
its C library compiled from source by ``make -C oracle`` (into
oracle/_ref/math_module.so; the prebuilt binaries shipped in the checkout are
never loaded).  Third-party modules the reference imports but this path does
not use (numba, matplotlib, kneed, tensorly, pandas, seaborn) are stubbed.

    make -C oracle && python tests/golden/make_golden.py

Fixtures written (all small, compressed .npz):
  examples_point_field.npz  examples 1A/1B: the charges of each frame after
                            the reference's parse/filter/rotate pipeline, the
                            reference's point field recomputed here and the
                            values in the shipped outputs point_field.dat
  ref_grid.npz              a 2,000-charge synthetic frame on an 11^3 grid:
                            compute_field_on_grid, calc_esp_base per point,
                            compute_ESP_on_grid (float16) and calc_field
  ref_topo.npz              192 streamlines of a 1,500-charge synthetic frame
                            through the reference's compute_topo_complete_c_shared
  examples_topology.npz     the (distance, curvature) rows of example 3A's
                            shipped .top files, the files' bytes, and the
                            reference's make_histograms of them
  ref_topo_dipole.npz       160 streamlines of 600 synthetic point dipoles
                            through the reference's
                            compute_topo_complete_c_shared_dipole
  ref_dat.npz               the field and potential volumes of ref_grid.npz
                            written by the reference's save_numpy_as_dat (the
                            .dat files' bytes) with their meta data
  ref_prep.npz              a 3,000-atom synthetic frame with residue ids
                            through the reference's filter_radius_whole_residue,
                            rotation, filter_in_box and box shift
  ref_cluster.npz           ten synthetic .top files (900 rows each) through
                            the reference's make_histograms and
                            construct_distance_matrix, and eight synthetic
                            vector fields (343 points) through its
                            construct_distance_matrix_volume
  ref_dispatch.npz          one frame of example 1A through the reference's
                            own dispatcher, CPET(options).run(), for
                            point_field, volume, volume_ESP and topo: the
                            calculator state each method reads (charges after
                            parsing, filtering and rotation; mesh; start
                            points and caps) and the bytes of every output
                            file the dispatcher wrote
"""
from __future__ import annotations

import argparse
import glob
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_SO = os.path.join(REPO, "oracle", "_ref", "math_module.so")
REF_ROOT = os.environ.get("CPETGB_REF", "/root/reference")


def _stub_modules():
    def mod(name, **attrs):
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
        return m

    def njit(*a, **k):
        if a and callable(a[0]) and not k:
            return a[0]
        return lambda f: f

    mod("numba", njit=njit, jit=njit, prange=range)
    mpl = mod("matplotlib")
    mpl.pyplot = mod("matplotlib.pyplot")
    mod("mpl_toolkits")
    mod("mpl_toolkits.mplot3d", Axes3D=object)
    mod("kneed", KneeLocator=object)
    tl = mod("tensorly")
    tl.decomposition = mod("tensorly.decomposition", parafac=None)
    mod("pandas", DataFrame=type("DataFrame", (), {}), Series=type("Series", (), {}))  # sklearn type checks
    mod("seaborn")


def import_reference(ref_root):
    if not os.path.exists(REF_SO):
        raise SystemExit(f"{REF_SO} missing: run `make -C oracle` first")
    _stub_modules()
    orig = importlib.util.find_spec

    def find_spec(name, *a, **k):  # point the reference at the library built from source
        if name == "CPET.utils.math_module":
            return types.SimpleNamespace(origin=REF_SO)
        return orig(name, *a, **k)

    importlib.util.find_spec = find_spec
    sys.path.insert(0, ref_root)
    import CPET.utils.calculator as ucalc
    import CPET.source.calculator as scalc
    import CPET.source.CPET  # noqa: F401  (the dispatcher, for ref_dispatch)

    return ucalc, scalc


def examples_point_field(ref_root, scalc, out):
    rec = {}
    for ex in ("1A_point-field", "1B_point-field-oriented"):
        with open(os.path.join(ref_root, "examples", ex, "options", "options.json")) as fh:
            opts = json.load(fh)
        shipped = {}
        with open(os.path.join(ref_root, "examples", ex, "outdir", "point_field.dat")) as fh:
            for line in fh:
                name, vec = line.strip().split(":", 1)
                shipped[name] = np.array(vec.strip("[] \n").split(), dtype=np.float64)
        for pdb in sorted(glob.glob(os.path.join(ref_root, "examples", "1A_point-field", "pdb", "*.pdb"))):
            name = os.path.basename(pdb).split(".")[0]
            calc = scalc.calculator(dict(opts), path_to_pdb=pdb)
            E = calc.compute_point_field()
            key = f"{ex[:2]}_{name}"
            rec[f"{key}_x"] = np.asarray(calc.x, np.float32)
            rec[f"{key}_Q"] = np.asarray(calc.Q, np.float32).reshape(-1)
            rec[f"{key}_E_ref"] = np.asarray(E, np.float32)
            rec[f"{key}_E_shipped"] = shipped[name]
    np.savez_compressed(out, **rec)
    return rec


def ref_grid(ucalc, out):
    sys.path.insert(0, REPO)
    from pycpet_gb300.synth import make_frame

    fr = make_frame(2000, seed=11)
    x = fr["x"].astype(np.float32)
    Q = fr["q"].astype(np.float32).reshape(-1, 1)
    mesh, _ = ucalc.initialize_box_points_uniform(center=np.zeros(3), x=np.array([1.0, 0, 0]),
                                                  y=np.array([0, 1.0, 0]), N_cr=[10, 10, 10],
                                                  dimensions=[1.0, 1.0, 1.0], dtype="float32", inclusive=True)
    field = ucalc.compute_field_on_grid(mesh, x, Q)
    pts = mesh.reshape(-1, 3)
    esp = np.array([ucalc.calculate_esp_c_shared_full(p, x, Q)[0] for p in pts], dtype=np.float32)
    esp_half = ucalc.compute_ESP_on_grid(mesh, x, Q)
    pf = ucalc.calculate_electric_field_c_shared_full_alt(np.array([0.0, 0.0, 0.0]), x, Q)
    np.savez_compressed(out, x=x, Q=Q.reshape(-1), mesh=mesh, field=field, esp=esp, esp_half=esp_half,
                        point_field=np.asarray(pf, np.float32))


def ref_topo(scalc, out):
    from pycpet_gb300.synth import make_frame, random_start_points

    fr = make_frame(1500, seed=12)
    dims = np.array([1.5, 1.5, 1.5], dtype=np.float32)
    step = 0.01
    starts = random_start_points(192, dims, seed=13).astype(np.float32)
    max_steps = round(2 * np.linalg.norm(dims) / step)
    caps = np.random.default_rng(14).integers(1, max_steps, 192)
    calc = scalc.calculator.__new__(scalc.calculator)
    calc.x = fr["x"].astype(np.float32)
    calc.Q = fr["q"].astype(np.float32).reshape(-1, 1)
    calc.random_start_points = starts
    calc.random_max_samples = caps
    calc.step_size = step
    calc.dimensions = dims
    calc.n_samples = len(starts)
    calc.concur_slip = 4
    calc.transformation_matrix = np.eye(3)
    calc.center = np.zeros(3, np.float32)
    calc.log = scalc.log
    hist = calc.compute_topo_complete_c_shared()
    np.savez_compressed(out, x=calc.x, Q=calc.Q.reshape(-1), starts=starts, caps=caps.astype(np.int32),
                        dims=dims, step=np.float32(step), result=np.asarray(hist, np.float32))


def ref_topo_dipole(scalc, out):
    from pycpet_gb300.synth import random_start_points

    rng = np.random.default_rng(31)
    x = rng.uniform(-12.0, 12.0, (900, 3))
    x = x[np.linalg.norm(x, axis=1) > 2.5][:600].astype(np.float32)
    mu = rng.normal(0.0, 0.3, (len(x), 3)).astype(np.float32)
    dims = np.array([1.5, 1.5, 1.5], dtype=np.float32)
    step = 0.01
    starts = random_start_points(160, dims, seed=32).astype(np.float32)
    caps = np.random.default_rng(33).integers(1, round(2 * np.linalg.norm(dims) / step), 160)
    calc = scalc.calculator.__new__(scalc.calculator)
    calc.x, calc.mu = x, mu
    calc.random_start_points, calc.random_max_samples = starts, caps
    calc.step_size, calc.dimensions, calc.n_samples = step, dims, len(starts)
    calc.concur_slip = 4
    calc.transformation_matrix = np.eye(3)
    calc.center = np.zeros(3, np.float32)
    calc.log = scalc.log
    hist = calc.compute_topo_complete_c_shared_dipole()
    np.savez_compressed(out, x=x, mu=mu, starts=starts, caps=caps.astype(np.int32), dims=dims,
                        step=np.float32(step), result=np.asarray(hist, np.float32))


def examples_topology(ref_root, ucalc, out):
    files = sorted(glob.glob(os.path.join(ref_root, "examples", "3A_field-topology", "outdir", "*.top")))
    rec = {}
    for i, f in enumerate(files):
        rec[f"top{i}"] = np.loadtxt(f)
        with open(f, "rb") as fh:
            rec[f"top{i}_bytes"] = np.frombuffer(fh.read(), dtype=np.uint8)
    rec["hist"] = ucalc.make_histograms(files)
    np.savez_compressed(out, **rec)


def ref_dat(ref_root, out):
    import tempfile

    import CPET.utils.io as rio

    g = np.load(os.path.join(HERE, "ref_grid.npz"))
    T = np.array([[0.8, 0.6, 0.0], [-0.6, 0.8, 0.0], [0.0, 0.0, 1.0]], dtype=np.float32)
    meta = {"dimensions": np.array([1.0, 1.0, 1.0], np.float32), "num_steps": [11, 11, 11],
            "transformation_matrix": T, "center": np.array([1.25, -3.5, 0.125], np.float32)}
    rec = {"T": T, "dimensions": meta["dimensions"], "center": meta["center"], "num_steps": np.array([11, 11, 11])}
    with tempfile.TemporaryDirectory() as tmp:
        for key, vol in (("field", g["field"]), ("esp", g["esp_half"])):
            path = os.path.join(tmp, f"{key}.dat")
            rio.save_numpy_as_dat(meta, vol, path)
            with open(path, "rb") as fh:
                rec[f"{key}_dat"] = np.frombuffer(fh.read(), dtype=np.uint8)
    np.savez_compressed(out, **rec)


def ref_prep(ucalc, out):
    import CPET.utils.io as rio

    rng = np.random.default_rng(41)
    n = 3000
    x = rng.uniform(-20.0, 20.0, (n, 3)) + np.array([3.0, -1.0, 2.0])
    q = rng.normal(0.0, 0.4, n)
    sizes = rng.integers(5, 20, n)
    resnum, names, i, r = [], [], 0, 0
    while len(resnum) < n:  # runs of 5-19 atoms; some neighbouring residues share a number
        k = int(sizes[r])
        resnum += [r // 2 + 1] * k
        names += [["ALA", "GLY", "HIS", "LYS"][r % 4]] * k
        r += 1
    resnum, names = np.array(resnum[:n]), np.array(names[:n])
    ID = [(j + 1, "CA", names[j], int(resnum[j]), "A") for j in range(n)]
    center = np.array([3.0, -1.0, 2.0])
    xa, ya = x[10], x[20]
    T = ucalc.initialize_box_points_uniform(center=center, x=xa, y=ya, N_cr=[4, 4, 4],
                                            dimensions=[1.5, 1.5, 1.5], inclusive=True)[1]
    dims = np.array([3.0, 2.5, 4.0])
    shift = np.array([0.25, -0.5, 0.125])
    xf, qf, idf = rio.filter_radius_whole_residue(x=x, Q=q, ID=ID, center=center, radius=10.0)
    xr = (xf - center) @ np.linalg.inv(T)
    xb, qb, idb = rio.filter_in_box(x=xr, Q=qf, ID=np.array(idf, dtype=object), center=center, dimensions=dims)
    xs = xb - shift
    np.savez_compressed(out, x=x, q=q, resid=names, resnum=resnum, center=center, T=T, radius=10.0,
                        dims=dims, shift=shift, x_ref=xs, q_ref=qb, n_after_radius=len(qf))


def ref_cluster(ucalc, out):
    import tempfile

    rng = np.random.default_rng(21)
    sets = []
    for f in range(10):  # (distance, curvature) rows shaped like streamline output
        d = np.clip(rng.gamma(2.0 + 0.2 * f, 0.6, 900), 0.0, 5.2)
        c = rng.lognormal(0.3 + 0.05 * f, 0.8, 900)
        sets.append(np.column_stack([d, c]))
    with tempfile.TemporaryDirectory() as tmp:
        files = []
        for f, v in enumerate(sets):
            path = os.path.join(tmp, f"frame_{f:02d}.top")
            np.savetxt(path, v)
            files.append(path)
        hists = ucalc.make_histograms(files)
    dmat = ucalc.construct_distance_matrix(hists)
    fields = [rng.normal(0.0, 1.0 + 0.1 * f, (343, 3)) for f in range(8)]
    vmat = ucalc.construct_distance_matrix_volume(fields)
    np.savez_compressed(out, values=np.concatenate(sets), offsets=np.arange(11) * 900, hists=hists,
                        dmat=dmat, fields=np.stack(fields), vmat=vmat)


DISPATCH_OPTIONS = {
    "inputfiletype": "pdb",
    "center": {"method": "mean", "atoms": [{"C7": 378}, {"O9": 378}]},
    "x": {"method": "first", "atoms": [{"O9": 378}]},
    "y": {"method": "first", "atoms": [{"N8": 378}]},
    "filter_intersect": True,
    "filter": {"resid": ["CF1"], "resnum": [378]},
    "filter_radius": 40,
    "dimensions": [0.5, 0.5, 0.5],
    "step_size": 0.1,
    "n_samples": 64,
    "max_streamline_init": "fixed_rand",
    "concur_slip": 2,
}
DISPATCH_METHODS = ("point_field", "volume", "volume_ESP", "topo")
DISPATCH_PDB = os.path.join("examples", "1A_point-field", "pdb", "1_alcdehydro_run1.pdb")


def dispatch_options(method, inputpath, outputpath):
    """Options of one dispatcher run (the example 3A box on example 1A's first frame)."""
    return dict(DISPATCH_OPTIONS, CPET_method=method, inputpath=inputpath, outputpath=outputpath)


def run_dispatcher(method, pdb, workdir):
    """CPET(options).run() of the imported reference on a directory holding
    `pdb`; returns {output file name: bytes}."""
    import shutil

    from CPET.source.CPET import CPET

    inp, outp = os.path.join(workdir, "in"), os.path.join(workdir, "out")
    os.makedirs(inp, exist_ok=True)
    shutil.copy(pdb, inp)
    CPET(dispatch_options(method, inp, outp)).run()
    files = {}
    for f in sorted(os.listdir(outp)):
        with open(os.path.join(outp, f), "rb") as fh:
            files[f] = fh.read()
    return files


def ref_dispatch(ref_root, scalc, out):
    import tempfile

    pdb = os.path.join(ref_root, DISPATCH_PDB)
    rec = {}
    for m in DISPATCH_METHODS:
        calc = scalc.calculator(dispatch_options(m, "", ""), path_to_pdb=pdb)
        rec[f"{m}/x"] = np.asarray(calc.x)
        rec[f"{m}/Q"] = np.asarray(calc.Q).reshape(-1)
        rec[f"{m}/center"] = np.asarray(calc.center)
        rec[f"{m}/transformation_matrix"] = np.asarray(calc.transformation_matrix)
        if m in ("volume", "volume_ESP"):
            rec[f"{m}/mesh"] = np.asarray(calc.mesh)
            rec[f"{m}/dimensions"] = np.asarray(calc.dimensions)
            rec[f"{m}/step_size"] = np.float64(calc.step_size)
        if m == "topo":
            rec[f"{m}/starts"] = np.asarray(calc.random_start_points)
            rec[f"{m}/caps"] = np.asarray(calc.random_max_samples).reshape(-1)
            rec[f"{m}/dimensions"] = np.asarray(calc.dimensions)
            rec[f"{m}/step_size"] = np.float64(calc.step_size)
        with tempfile.TemporaryDirectory() as tmp:
            for name, data in run_dispatcher(m, pdb, tmp).items():
                rec[f"{m}/file/{name}"] = np.frombuffer(data, dtype=np.uint8)
    np.savez_compressed(out, **rec)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=REF_ROOT)
    a = ap.parse_args()
    ucalc, scalc = import_reference(a.ref)
    examples_point_field(a.ref, scalc, os.path.join(HERE, "examples_point_field.npz"))
    ref_grid(ucalc, os.path.join(HERE, "ref_grid.npz"))
    ref_topo(scalc, os.path.join(HERE, "ref_topo.npz"))
    examples_topology(a.ref, ucalc, os.path.join(HERE, "examples_topology.npz"))
    ref_cluster(ucalc, os.path.join(HERE, "ref_cluster.npz"))
    ref_dat(a.ref, os.path.join(HERE, "ref_dat.npz"))
    ref_prep(ucalc, os.path.join(HERE, "ref_prep.npz"))
    ref_topo_dipole(scalc, os.path.join(HERE, "ref_topo_dipole.npz"))
    ref_dispatch(a.ref, scalc, os.path.join(HERE, "ref_dispatch.npz"))
    for f in sorted(glob.glob(os.path.join(HERE, "*.npz"))):
        print(f, os.path.getsize(f))


if __name__ == "__main__":
    main()
