"""Generates the golden fixtures in tests/golden/ from the reference psim built from its own
sources (oracle/_ref/ref_driver, see oracle/ref_recipe/Makefile).  Run it where the
reference tree is available:

    python tests/golden/make_golden.py --reference /path/to/reference [--skip-runs]
        [--only geom,tables,invert,runs,topology,seeded,demos,headline,headline_tables,headline_topology,rates,
                exports]
        [--demo <demo>[,<demo>]]

The demo runs dominate: each of the 16 runs of kinked_demo_120_35_spec (6174 cells, a 2e7
phonon budget, 6.2e9 phonon-steps) took about an hour of one host thread.

Outputs (all small):
  models/*.json          the model files the fixtures were made from (psim_gb300.modelgen)
  geom.npz               Line::getIntersection / Line::contains(Point) / Triangle::contains /
                         Triangle normals, area and getRandPoint on random and degenerate cases
  tables_<model>.npz     material tables after Model::initializeMaterialTables
  invert_<model>.npz     SensorInterpreter results for given tallies
  rates.npz              Material::relaxRates of two materials on a (T, frequency, polarization) grid
  export_<model>.npz     a seeded run's per-run statistics and the ss_ table the reference wrote for it
  topology_<model>.npz   the assembled model (cells, sensors, edge sub-surfaces) of every model
                         file here, demos included
  runs_<model>.npz       per-sensor results of 16 seeded reference runs (statistical parity)
  models/<demo>.json.gz  the reference's own demo models (psim_python/json/), gzipped, and
  runs_<demo>.npz        16 seeded runs of each by the reference built from its sources, with
                         the result table the reference commits for it (psim_python/json/results/)
  seeded_<demo>.npz      one seeded run of the largest demo at a reduced phonon budget
"""
from __future__ import annotations

import argparse
import gzip
import json
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from psim_gb300 import modelgen as mg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.golden.tables_io import read_tables  # noqa: E402

MODELS = os.path.join(HERE, "models")
SEEDS = list(range(1, 17))


def model_specs():
    """Small models of the benchmark shapes (same geometry family, reduced sizes)."""
    return {
        "bar_ss": mg.bar(num_phonons=100000, num_measurements=1000, sim_time=5.0),
        "bar_full": mg.bar(num_phonons=50000, num_measurements=1000, sim_time=5.0, t_eq=0.0, t_left=60.0,
                           t_right=40.0, t_init=50.0),
        "bar_periodic": mg.bar(num_phonons=50000, num_measurements=500, sim_time=2.5, sim_type=1, step_interval=25,
                               spec=0.3),
        "kinked_small": mg.kinked(num_phonons=60000, num_measurements=400, sim_time=2.0, n_len=10, step_interval=20),
        "plate_small": mg.plate(length=1000.0, width=250.0, nx=16, ny=4, strip=(100.0, 150.0), num_phonons=60000,
                                num_measurements=400, sim_time=0.4, pulse=0.02, step_interval=20),
        "bar_runs": mg.bar(num_phonons=30000, num_measurements=400, sim_time=2.0, num_runs=3, spec=0.5),
        "bar_phasor": mg.bar(num_phonons=20000, num_measurements=400, sim_time=2.0, sim_type=1, step_interval=20,
                             phasor_sim=True),
    }


def headline_specs():
    """The benchmark configurations as they are stated: geometry, mode, step length and number
    of steps of each, at its own phonon budget where the reference runs 16 seeds in minutes,
    else at a reduced one (the per-sensor means of a deviational run do not depend on the
    budget; only their noise does).

    cfg0_bar_ss     1 um x 100 nm bar, 10 cells, 310/290 K, deviational steady state, 2000
                    steps of 5 ps, 2e5 phonons per step (budget 3.09e6 at a mean lifetime
                    of 129.5 steps)
    cfg2b_bar_full  the same bar in full mode at 60/40 K (budget 2.04e6, lifetime 196 steps)
    cfg1_kinked     the 400-sensor kinked structure, periodic, 5000 steps of 2 ps, output
                    every 50 steps; budget 6e6 instead of the 1.2e8 of 1e7 per step
    cfg2a_plate     the 4 x 1 um plate, 64 x 16 cells, transient 20 ps pulse, 3000 steps of
                    1 ps; budget 5e5 instead of 2e7
    si_ge_bar       the bar with five silicon and five germanium cells: one interface between
                    two materials (germanium from psim_python/psim/pre_builts.py:25-29)
    """
    return {
        "cfg0_bar_ss": mg.bar(num_phonons=3090000, num_measurements=2000, sim_time=10.0),
        "cfg2b_bar_full": mg.bar(num_phonons=2040000, num_measurements=2000, sim_time=10.0, t_eq=0.0, t_left=60.0,
                                 t_right=40.0, t_init=50.0),
        "cfg1_kinked": mg.kinked(seed=0, num_measurements=5000, sim_time=10.0, step_interval=50, num_phonons=6000000),
        "cfg2a_plate": mg.plate(num_phonons=500000),
        "si_ge_bar": mg.two_material_bar(num_phonons=300000, num_measurements=1000, sim_time=5.0),
    }


GZIPPED = {"cfg1_kinked", "cfg2a_plate"}  # larger model files are kept gzipped


def write_models():
    os.makedirs(MODELS, exist_ok=True)
    paths = {}
    for name, m in model_specs().items():
        p = os.path.join(MODELS, name + ".json")
        mg.write(m, p)
        paths[name] = p
    td = tempfile.mkdtemp(prefix="psim_headline_")
    for name, m in headline_specs().items():
        if name in GZIPPED:
            p = mg.write(m, os.path.join(td, name + ".json"))
            with open(p, "rb") as f, gzip.GzipFile(os.path.join(MODELS, name + ".json.gz"), "wb", mtime=0) as g:
                g.write(f.read())
        else:
            p = mg.write(m, os.path.join(MODELS, name + ".json"))
        paths[name] = p
    return paths


def driver(*args, env=None):
    out = subprocess.run([O.REF_DRIVER, *args], capture_output=True, text=True, env=env)
    if out.returncode != 0:
        raise RuntimeError(f"ref_driver {args} failed: {out.stderr}")
    return out.stdout


# ---------------------------------------------------------------- geometry
def geometry_cases(rng: np.random.Generator):
    lines = []
    # random segments, half on a coarse grid to create collinear/parallel/touching cases
    for i in range(4000):
        if i % 2:
            a = rng.integers(-3, 4, size=4).astype(float) * 25.0
            b = rng.integers(-3, 4, size=4).astype(float) * 25.0
        else:
            a = rng.uniform(-100, 100, size=4)
            b = rng.uniform(-100, 100, size=4)
        if i % 7 == 0:
            b[2] = b[0]  # vertical
        if i % 11 == 0:
            a[3] = a[1]  # horizontal
        if i % 13 == 0:
            b[:2] = a[2:]  # touching at an end point
        if i % 17 == 0:
            a[2:] = a[:2]  # degenerate (identical end points)
        lines.append("I " + " ".join(repr(float(v)) for v in np.concatenate([a, b])))
    intersect = [list(map(float, l.split()[1:])) for l in lines]
    # point on line: points on, near and off random lines (including the end points)
    on = []
    for i in range(3000):
        l = rng.uniform(-50, 50, size=4)
        if i % 5 == 0:
            l[2] = l[0]
        t = rng.uniform(-0.5, 1.5)
        p = l[:2] + t * (l[2:] - l[:2])
        if i % 3 == 1:
            p = p + rng.normal(scale=1e-9, size=2)
        elif i % 3 == 2:
            p = p + rng.normal(scale=1.0, size=2)
        on.append(np.concatenate([l, p]))
    # triangles: random and grid-snapped, points inside/outside/on edges/at vertices
    tri = []
    for i in range(3000):
        t = rng.uniform(-50, 50, size=6) if i % 2 else rng.integers(-2, 3, size=6).astype(float) * 10.0
        w = rng.dirichlet([1, 1, 1])
        if i % 4 == 1:
            w[rng.integers(0, 3)] = 0.0
            w = w / w.sum()
        p = w[0] * t[0:2] + w[1] * t[2:4] + w[2] * t[4:6]
        if i % 4 == 2:
            p = p + rng.normal(scale=5.0, size=2)
        if i % 4 == 3:
            p = t[2 * (i % 3): 2 * (i % 3) + 2].copy()
        tri.append(np.concatenate([t, p]))
    rand_pts = []
    for i in range(500):
        t = rng.uniform(-50, 50, size=6)
        r = rng.uniform(0, 1, size=2)
        rand_pts.append(np.concatenate([t, r]))
    return np.array(intersect), np.array(on), np.array(tri), np.array(rand_pts)


def make_geom():
    rng = np.random.default_rng(20261203)
    inter, on, tri, rnd = geometry_cases(rng)
    with tempfile.TemporaryDirectory() as td:
        cases = os.path.join(td, "cases.txt")
        out = os.path.join(td, "out.txt")
        with open(cases, "w") as f:
            for r in inter:
                f.write("I " + " ".join(repr(float(v)) for v in r) + "\n")
            for r in on:
                f.write("L " + " ".join(repr(float(v)) for v in r) + "\n")
            for r in tri:
                f.write("C " + " ".join(repr(float(v)) for v in r) + "\n")
            for r in tri:
                f.write("N " + " ".join(repr(float(v)) for v in r[:6]) + "\n")
            for r in rnd:
                f.write("R " + " ".join(repr(float(v)) for v in r) + "\n")
        driver("geom", cases, out)
        rows = open(out).read().splitlines()
    k = 0
    has = np.zeros(len(inter), dtype=np.int32)
    poi = np.zeros((len(inter), 2))
    for i in range(len(inter)):
        parts = rows[k].split()
        k += 1
        if parts[0] == "X":
            has[i] = -1
        elif parts[0] == "1":
            has[i] = 1
            poi[i] = [float(parts[1]), float(parts[2])]
    on_out = np.array([int(rows[k + i]) if rows[k + i] != "X" else -1 for i in range(len(on))], dtype=np.int32)
    k += len(on)
    tri_out = np.array([int(rows[k + i]) if rows[k + i] not in ("X", "E") else -2 for i in range(len(tri))], dtype=np.int32)
    k += len(tri)
    normals = np.full((len(tri), 8), np.nan)
    for i in range(len(tri)):
        parts = rows[k + i].split()
        if parts[0] != "X":
            normals[i] = [float(v) for v in parts]
    k += len(tri)
    rnd_out = np.array([[float(v) for v in rows[k + i].split()] for i in range(len(rnd))])
    np.savez_compressed(os.path.join(HERE, "geom.npz"), intersect_a=inter[:, :4], intersect_b=inter[:, 4:],
                        intersect_has=has, intersect_poi=poi, online_lines=on[:, :4], online_pts=on[:, 4:],
                        online_out=on_out, tri=tri[:, :6], tri_pts=tri[:, 6:], tri_out=tri_out, tri_normals=normals,
                        rand_tri=rnd[:, :6], rand_r=rnd[:, 6:], rand_out=rnd_out)
    print("geom.npz:", len(inter), "intersections,", int((has == 1).sum()), "hits")


# ---------------------------------------------------------------- tables
def make_tables_two_materials(paths, name="si_ge_bar"):
    """tables_<name>.npz for a model of two materials: each material's frequency grid,
    velocities, densities of states and every temperature's sums, with full tables at three
    temperatures (prefix m0_ / m1_ in the model's material order)."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "t.bin")
        driver("tables", paths[name], out)
        mats, bounds = read_tables(out, n_materials=2)
    arrays = {"bounds": bounds}
    for i, m in enumerate(mats):
        nt = len(m["temps"])
        keep = sorted(set([0, nt // 2, nt - 1] + [int(np.searchsorted(m["temps"], t)) for t in (300.0, 310.0, 290.0)
                                                  if m["temps"][0] <= t <= m["temps"][-1]]))
        for k in ("temps", "freq", "vel_la", "vel_ta", "dens_la", "dens_ta", "base_sum", "emit_sum", "scatter_sum"):
            arrays[f"m{i}_{k}"] = m[k]
        arrays[f"m{i}_keep"] = np.array(keep)
        for k in ("base", "emit", "scatter"):
            arrays[f"m{i}_{k}"] = m[k][keep]
    np.savez_compressed(os.path.join(HERE, f"tables_{name}.npz"), **arrays)
    print(f"tables_{name}.npz: {[len(m['temps']) for m in mats]} temperatures")


def make_tables(paths):
    for name in ("bar_ss", "bar_full", "kinked_small"):
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "t.bin")
            driver("tables", paths[name], out)
            mats, bounds = read_tables(out)
        m = mats[0]
        nt = len(m["temps"])
        keep = sorted(set([0, nt // 2, nt - 1] + [int(np.searchsorted(m["temps"], t)) for t in (300.0, 310.0, 290.0, 50.0, 60.0, 40.0, 320.0, 280.0) if m["temps"][0] <= t <= m["temps"][-1]]))
        np.savez_compressed(os.path.join(HERE, f"tables_{name}.npz"), temps=m["temps"], freq=m["freq"],
                            vel_la=m["vel_la"], vel_ta=m["vel_ta"], dens_la=m["dens_la"], dens_ta=m["dens_ta"],
                            base_sum=m["base_sum"], emit_sum=m["emit_sum"], scatter_sum=m["scatter_sum"],
                            keep=np.array(keep), base=m["base"][keep], emit=m["emit"][keep], scatter=m["scatter"][keep],
                            bounds=bounds)
        print(f"tables_{name}.npz: {nt} temperatures, kept {keep}")


# ---------------------------------------------------------------- the steady-state writer
EXPORTS = (("bar_runs", 5), ("bar_ss", 6), ("si_ge_bar", 7))  # model, seed


def make_exports(paths):
    """export_<model>.npz: one seeded reference run's per-run statistics (as the run dump prints
    them, 17 significant digits) and the ss_ table OutputManager::exportResults wrote for that run
    (psim/src/outputManager.cpp:13-38,40-78): its header line and its body bytes."""
    for name, seed in EXPORTS:
        with tempfile.TemporaryDirectory() as td:
            model = os.path.join(td, name + ".json")
            with open(paths[name], "rb") as f, open(model, "wb") as g:
                g.write(f.read())
            dump = os.path.join(td, "d.json")
            driver("run", model, dump, model, env=dict(os.environ, PSIM_SEED=str(seed)))
            d = json.load(open(dump))
            text = open(os.path.join(td, f"ss_{name}.txt"), "rb").read()
        stats = np.array([[m["stats"] for m in run] for run in d["runs"]])
        header, body = text.split(b"\n", 1)
        np.savez_compressed(os.path.join(HERE, f"export_{name}.npz"), stats=stats, header=np.frombuffer(header, np.uint8),
                            body=np.frombuffer(body, np.uint8))
        print(f"export_{name}.npz: {stats.shape[0]} runs, {len(body)} body bytes")


# ---------------------------------------------------------------- scattering rates
def rate_cases():
    """(T, frequency, polarization) known-answer grid for Material::relaxRates: temperatures from
    2 K to 1000 K; frequencies on each material's bin centres (every 7th of the 1000) and both
    sides of the TA cut-off w; both polarizations."""
    temps = np.array([2.0, 5.0, 10.0, 20.0, 40.0, 50.0, 77.0, 150.0, 250.0, 280.0, 290.0, 300.0, 310.0, 320.0, 400.0,
                      600.0, 1000.0])
    return temps


def make_rates(paths, name="si_ge_bar"):
    """rates.npz: Material::relaxRates of the silicon and germanium of si_ge_bar on rate_cases(),
    the cases of each material on its own frequency grid."""
    model = json.load(open(paths[name]))
    arrays = {}
    with tempfile.TemporaryDirectory() as td:
        for i, mat in enumerate(model["materials"]):
            w_cut = mat["r_data"]["w"]
            w_max = max(mat["d_data"]["max_freq_la"], mat["d_data"]["max_freq_ta"])
            centres = (np.arange(1, 2000, 2) * (w_max / 1000.0) / 2.0)[::7]
            freqs = np.concatenate([centres, [np.nextafter(w_cut, 0.0), w_cut, np.nextafter(w_cut, np.inf)]])
            T, F, P = np.meshgrid(rate_cases(), freqs, [0.0, 1.0], indexing="ij")
            cases = np.stack([T.ravel(), F.ravel(), P.ravel()], axis=1)
            cp = os.path.join(td, "cases.bin")
            op = os.path.join(td, "out.bin")
            cases.astype("<f8").tofile(cp)
            driver("rates", paths[name], cp, op)
            out = np.fromfile(op, dtype="<f8").reshape(len(model["materials"]), len(cases), 3)
            arrays[f"m{i}_cases"] = cases
            arrays[f"m{i}_rates"] = out[i]
    np.savez_compressed(os.path.join(HERE, "rates.npz"), **arrays)
    print("rates.npz:", {k: v.shape for k, v in arrays.items()})


# ---------------------------------------------------------------- model assembly
def read_topology(path):
    """The reference's assembled model as written by `ref_driver topology`: per cell its sensor,
    vertices and edge specularities; per edge sub-surface its cell, edge, kind (0 transition,
    1 emitting), target (neighbour cell, or the emitting surface's owning cell), line and, for
    emitting surfaces, (temperature, duration, start time)."""
    cells, subs = [], []
    for line in open(path):
        f = line.split()
        if f[0] == "c":
            cells.append([float(v) for v in f[1:]])
        elif f[0] == "t":
            subs.append([int(f[1]), int(f[2]), 0, int(f[3])] + [float(v) for v in f[4:8]] + [np.nan] * 3)
        elif f[0] == "e":
            vals = [float(v) for v in f[4:]]
            subs.append([int(f[1]), int(f[2]), 1, int(f[3])] + vals[3:7] + vals[0:3])
    c = np.array(cells, dtype=np.float64)
    s = np.array(subs, dtype=np.float64).reshape(-1, 11)
    return dict(cell_sensor=c[:, 0].astype(np.int64), cell_vertices=c[:, 1:7], cell_spec=c[:, 7:10],
                sub_cell=s[:, 0].astype(np.int64), sub_edge=s[:, 1].astype(np.int64), sub_kind=s[:, 2].astype(np.int64),
                sub_target=s[:, 3].astype(np.int64), sub_line=s[:, 4:8], sub_emit=s[:, 8:11])


def make_topology(paths):
    """topology_<model>.npz: the reference's model assembly (Model::addCell's neighbour search,
    Model::setEmitSurface) for every model file the fixtures use."""
    for name, path in paths.items():
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "t.txt")
            driver("topology", path, out)
            topo = read_topology(out)
        np.savez_compressed(os.path.join(HERE, f"topology_{name}.npz"), **topo)
        print(f"topology_{name}.npz: {len(topo['cell_sensor'])} cells, {int((topo['sub_kind'] == 0).sum())} transition "
              f"and {int((topo['sub_kind'] == 1).sum())} emitting sub-surfaces")


# ---------------------------------------------------------------- inversion
def make_invert(paths):
    rng = np.random.default_rng(7)
    for name in ("bar_ss", "bar_full", "kinked_small"):
        shape = O.shape(paths[name])
        S, K = shape[0], shape[1]
        scale = 40 if name != "bar_full" else 4000
        counts = rng.integers(-scale, scale, size=(S, K))
        if name == "bar_full":
            counts = np.abs(counts) + rng.integers(0, 20000, size=(S, K))
        with tempfile.TemporaryDirectory() as td:
            cp = os.path.join(td, "c.txt")
            op = os.path.join(td, "o.txt")
            with open(cp, "w") as f:
                for s in range(S):
                    f.write(f"{s} {K} " + " ".join(str(int(v)) for v in counts[s]) + "\n")
            driver("invert", paths[name], cp, op)
            rows = open(op).read().splitlines()
        eff = float(rows[0].split()[1])
        stats = np.zeros((S, 6))
        temps = np.zeros((S, K))
        for r in rows[1:]:
            v = r.split()
            s = int(v[0])
            stats[s] = [float(x) for x in v[1:7]]
            temps[s] = [float(x) for x in v[7:]]
        np.savez_compressed(os.path.join(HERE, f"invert_{name}.npz"), counts=counts, flux_x_factor=1000.5,
                            flux_y_factor=-250.25, eff=eff, stats=stats, temps=temps)
        print(f"invert_{name}.npz: eff {eff:.6e}")


# ---------------------------------------------------------------- statistical references
def ref_run(path, seed):
    with tempfile.TemporaryDirectory() as td:
        dump = os.path.join(td, "d.json")
        env = dict(os.environ, PSIM_SEED=str(seed))
        driver("run", path, dump, env=env)
        d = json.load(open(dump))
    runs = [np.array([m["stats"] for m in run]) for run in d["runs"]]
    acc = np.zeros_like(runs[0])
    for r in runs:
        acc = acc + r
    return acc / len(runs), d["total_phonons_last_run"]


def make_runs(paths, names, single=False):
    """runs_<name>.npz: 16 seeded reference runs per model.  ``single`` stores float32 (larger
    tables; the seed-to-seed spreads lie far above its resolution)."""
    for name in names:
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
            res = list(pool.map(lambda s: ref_run(paths[name], s), SEEDS))
        stats = np.stack([r[0] for r in res])
        phonons = np.array([r[1] for r in res])
        if single:
            stats = stats.astype(np.float32)
        np.savez_compressed(os.path.join(HERE, f"runs_{name}.npz"), seeds=np.array(SEEDS), stats=stats, phonons=phonons)
        print(f"runs_{name}.npz: {stats.shape}, mean T {stats[:, :, 0].mean(axis=0)[:4]}", flush=True)


# ---------------------------------------------------------------- the reference's own demo models
DEMOS = ["linear_demo", "linear_sides_demo_ss", "kinked_demo_120_35_spec"]


def copy_demos(reference):
    """The demo model files the reference ships, gzipped into models/; returns plain copies in a
    temporary directory for the reference driver."""
    td = tempfile.mkdtemp(prefix="psim_demos_")
    paths = {}
    for name in DEMOS:
        src = os.path.join(reference, "psim_python", "json", name + ".json")
        data = open(src, "rb").read()
        with gzip.GzipFile(os.path.join(MODELS, name + ".json.gz"), "wb", mtime=0) as f:
            f.write(data)
        paths[name] = os.path.join(td, name + ".json")
        with open(paths[name], "wb") as f:
            f.write(data)
    return paths


def make_demo_runs(reference, paths, names=DEMOS):
    """16 seeded reference runs of each demo, next to the steady-state table the reference
    commits for it (a single unseeded run: T, SE, flux x, SE, flux y, SE per sensor)."""
    for name in names:
        committed = np.loadtxt(os.path.join(reference, "psim_python", "json", "results", f"ss_{name}.txt"), skiprows=1)
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
            res = list(pool.map(lambda s: ref_run(paths[name], s), SEEDS))
        stats = np.stack([r[0] for r in res])
        phonons = np.array([r[1] for r in res])
        # float32 keeps these larger tables small; seed-to-seed spreads are far above its resolution
        np.savez_compressed(os.path.join(HERE, f"runs_{name}.npz"), seeds=np.array(SEEDS), stats=stats.astype(np.float32),
                            phonons=phonons, committed=committed.astype(np.float32))
        print(f"runs_{name}.npz: {stats.shape}, mean T {stats[:, :, 0].mean(axis=0)[:4]}, committed {committed[:4, 0]}")


SEEDED_DEMO = ("kinked_demo_120_35_spec", 20000, 1)  # demo, reduced phonon budget, seed


def reduced_budget(src, dst, num_phonons):
    """The model file src with its phonon budget set to num_phonons (everything else as is)."""
    d = json.load(open(src))
    d["settings"]["num_phonons"] = num_phonons
    with open(dst, "w") as f:
        json.dump(d, f)
    return dst


def make_demo_seeded(paths):
    """seeded_<demo>.npz: one seeded reference run of the largest demo at a reduced phonon
    budget, in full precision, for a bit-exact check of the oracle on that geometry."""
    name, budget, seed = SEEDED_DEMO
    with tempfile.TemporaryDirectory() as td:
        p = reduced_budget(paths[name], os.path.join(td, name + ".json"), budget)
        stats, phonons = ref_run(p, seed)
    np.savez_compressed(os.path.join(HERE, f"seeded_{name}.npz"), seed=seed, num_phonons=budget, stats=stats,
                        phonons=phonons)
    print(f"seeded_{name}.npz: budget {budget}, seed {seed}, {phonons} phonons")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the reference checkout (the psim project)")
    ap.add_argument("--skip-runs", action="store_true")
    ap.add_argument("--only", default="")
    ap.add_argument("--demo", default="", help="comma-separated demo models for the demo runs (default: all three)")
    args = ap.parse_args()
    if not O.build_reference(args.reference):
        sys.exit("the reference sources are not available")
    O.build()
    paths = write_models()
    only = set(args.only.split(",")) if args.only else None
    if only is None or "geom" in only:
        make_geom()
    if only is None or "tables" in only:
        make_tables(paths)
    if only is None or "invert" in only:
        make_invert(paths)
    if not args.skip_runs and (only is None or "runs" in only):
        make_runs(paths, list(model_specs()))
    if only is None or "headline_tables" in only:
        make_tables_two_materials(paths)
    if only is None or "rates" in only:
        make_rates(paths)
    if only is None or "exports" in only:
        make_exports(paths)
    if only is None or "headline_topology" in only:
        make_topology({k: paths[k] for k in headline_specs()})
    if not args.skip_runs and (only is None or "headline" in only):
        # quickest first, so that the fixtures arrive as they are done
        make_runs(paths, ["si_ge_bar", "cfg2b_bar_full", "cfg0_bar_ss"])
        make_runs(paths, ["cfg2a_plate", "cfg1_kinked"], single=True)
    demo_paths = copy_demos(args.reference) if only is None or {"demos", "topology", "seeded"} & only else {}
    if only is None or "seeded" in only:
        make_demo_seeded(demo_paths)
    if only is None or "topology" in only:
        make_topology({**paths, **demo_paths})
    if only is None or "demos" in only:
        make_demo_runs(args.reference, demo_paths, args.demo.split(",") if args.demo else DEMOS)


if __name__ == "__main__":
    main()
