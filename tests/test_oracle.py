"""The CPU oracle against the golden vectors made by the reference itself (tests/golden/).

The oracle (oracle/psim_oracle.cpp) restates the reference and draws the same random stream
as the reference built with the seeding shim, so its results must equal the reference's
bit for bit: geometry answers, material tables, and whole seeded runs.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, model_path


@pytest.fixture(scope="module")
def O(built):
    from oracle import oracle
    return oracle


def test_geometry_intersections(O):
    g = np.load(os.path.join(GOLDEN, "geom.npz"))
    has, poi = O.intersect(g["intersect_a"], g["intersect_b"])
    assert np.array_equal(has, g["intersect_has"])
    hit = has == 1
    assert np.array_equal(poi[hit], g["intersect_poi"][hit])


def test_geometry_point_on_line(O):
    g = np.load(os.path.join(GOLDEN, "geom.npz"))
    assert np.array_equal(O.on_line(g["online_lines"], g["online_pts"]), g["online_out"])


def test_geometry_triangle_contains(O):
    g = np.load(os.path.join(GOLDEN, "geom.npz"))
    ok = g["tri_out"] >= 0
    out = O.tri_contains(g["tri"][ok], g["tri_pts"][ok])
    assert np.array_equal(out, g["tri_out"][ok])


def _read_tables(path):
    from tests.golden.tables_io import read_tables
    return read_tables(path)


@pytest.mark.parametrize("name", ["bar_ss", "bar_full", "kinked_small"])
def test_material_tables(O, name):
    gold = np.load(os.path.join(GOLDEN, f"tables_{name}.npz"))
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "t.bin")
        O.tables(model_path(name), out)
        mats, bounds = _read_tables(out)
    m = mats[0]
    exact = os.uname().machine == "x86_64"
    cmp = (lambda a, b: np.array_equal(a, b)) if exact else (lambda a, b: np.allclose(a, b, rtol=1e-12, atol=0, equal_nan=True))
    assert np.array_equal(m["temps"], gold["temps"])
    for key in ("freq", "vel_la", "vel_ta", "dens_la", "dens_ta", "base_sum", "emit_sum", "scatter_sum"):
        assert cmp(m[key], gold[key]), key
    keep = gold["keep"]
    for key in ("base", "emit", "scatter"):
        assert cmp(np.nan_to_num(m[key][keep], nan=-1.0), np.nan_to_num(gold[key], nan=-1.0)), key
    assert np.array_equal(bounds, gold["bounds"])


@pytest.mark.parametrize("name,seeds", [("bar_ss", [1, 2]), ("bar_full", [3]), ("bar_periodic", [4]),
                                        ("kinked_small", [5]), ("plate_small", [6]), ("bar_runs", [7]),
                                        ("bar_phasor", [8])])
def test_seeded_runs_match_reference(O, name, seeds):
    """Whole runs: with the reference's seed, the oracle reproduces its per-sensor results."""
    gold = np.load(os.path.join(GOLDEN, f"runs_{name}.npz"))
    exact = os.uname().machine == "x86_64"
    for seed in seeds:
        r = O.run(model_path(name), seed, threads=1)
        ref = gold["stats"][list(gold["seeds"]).index(seed)]
        if exact:
            assert np.array_equal(r.stats, ref), (name, seed)
        else:
            # libm may round differently on another architecture; trajectories then diverge
            # after a while, so only the bulk agreement is checked there.
            assert np.allclose(r.stats[:, 0], ref[:, 0], rtol=5e-3), (name, seed)


def test_seeded_run_of_a_reference_demo_matches(O, tmp_path):
    """The reference's own linear_demo model with the reference's seed 1: the oracle reproduces
    its per-sensor results.  The demo fixtures keep float32, so the oracle's results are rounded
    to float32 and must then be equal."""
    from conftest import demo_model_path
    gold = np.load(os.path.join(GOLDEN, "runs_linear_demo.npz"))
    r = O.run(demo_model_path("linear_demo", str(tmp_path)), 1, threads=1)
    ref = gold["stats"][list(gold["seeds"]).index(1)]
    if os.uname().machine == "x86_64":
        assert np.array_equal(r.stats.astype(np.float32), ref)
    else:
        assert np.allclose(r.stats[:, 0], ref[:, 0], rtol=5e-3)


def test_seeded_run_of_the_largest_reference_demo_matches(O, tmp_path):
    """The reference's kinked demo (6174 cells, 3108 sensors, 42 emitting surfaces) at a reduced
    phonon budget with the reference's seed: the oracle reproduces its per-sensor results."""
    import json
    from conftest import demo_model_path
    gold = np.load(os.path.join(GOLDEN, "seeded_kinked_demo_120_35_spec.npz"))
    d = json.load(open(demo_model_path("kinked_demo_120_35_spec", str(tmp_path))))
    d["settings"]["num_phonons"] = int(gold["num_phonons"])
    path = str(tmp_path / "kinked_demo_reduced.json")
    with open(path, "w") as f:
        json.dump(d, f)
    r = O.run(path, int(gold["seed"]), threads=1)
    assert r.stats.shape == gold["stats"].shape == (3108, 6)
    if os.uname().machine == "x86_64":
        assert np.array_equal(r.stats, gold["stats"])
    else:
        assert np.allclose(r.stats[:, 0], gold["stats"][:, 0], rtol=5e-3)


def test_multithreaded_oracle_is_the_same_process(O):
    """Several threads draw different streams but simulate the same process."""
    gold = np.load(os.path.join(GOLDEN, "runs_bar_ss.npz"))
    r = O.run(model_path("bar_ss"), 11, threads=4)
    t_ref = gold["stats"][:, :, 0]
    mean, se = t_ref.mean(axis=0), t_ref.std(axis=0, ddof=1) / np.sqrt(len(t_ref))
    z = (r.stats[:, 0] - mean) / np.sqrt(se ** 2 * len(t_ref) + 1e-12)
    assert np.all(np.abs(z) < 5.0)
    assert r.phonon_steps > 0
