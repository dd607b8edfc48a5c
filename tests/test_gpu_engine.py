"""GPU engine behaviour through the C ABI: determinism, independence from the launch shape,
the ModelSimulator seam, output files, counters and the step loop's bookkeeping."""
import os
import re
import shutil
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, model_path

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(gpu):
    from psim_gb300 import api
    return api


@pytest.mark.parametrize("precision", [0, 1])
def test_same_seed_same_tallies(api, precision):
    m = api.Model(model_path("kinked_small"))
    m.run(seed=5, precision=precision)
    e1, f1 = m.tallies()
    s1 = m.measurements()
    m.run(seed=5, precision=precision)
    e2, f2 = m.tallies()
    assert np.array_equal(e1, e2) and np.array_equal(f1, f2)
    assert np.array_equal(s1, m.measurements())
    m.run(seed=6, precision=precision)
    e3, _ = m.tallies()
    assert not np.array_equal(e1, e3)


def test_launch_shape_does_not_change_results(api, monkeypatch):
    """Each phonon's random stream is keyed by its id and step, so the grid size (which
    reorders the buffer) cannot change any tally."""
    m = api.Model(model_path("bar_ss"))
    m.run(seed=9)
    ref = m.tallies()
    for grid in ("7", "301"):
        monkeypatch.setenv("PSIM_GB300_GRID", grid)
        m2 = api.Model(model_path("bar_ss"))
        m2.run(seed=9)
        got = m2.tallies()
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1]), grid
    monkeypatch.delenv("PSIM_GB300_GRID")
    # tables read from global memory instead of the shared-memory copies
    monkeypatch.setenv("PSIM_GB300_STAGE", "0")
    m3 = api.Model(model_path("bar_ss"))
    m3.run(seed=9)
    got = m3.tallies()
    assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])


@pytest.mark.parametrize("name", ["kinked_small", "plate_small", "bar_ss", "plate_2560"])
def test_steps_per_launch_do_not_change_results(api, monkeypatch, tmp_path, name):
    """An FP32 launch covers up to 16 measurement steps and carries phonons across the inner
    boundaries in registers; plain boundaries are crossed in a warp-uniform loop while enough
    lanes cross one.  Tallies, the population history and the phonon-step count equal those of
    one step per launch, with every table in shared memory, with the tables but not the cell
    records there, and with global ones, whatever the coasting threshold, with survivors written
    in two groups by their time to scattering or their velocity, and in a chunked run whose state
    buffers grow between chunks of launches (both groups copied).  plate_2560 has
    more sensors than the shared-memory tally holds (tallies in global memory)."""
    from psim_gb300 import modelgen as mg
    path = (mg.write(mg.plate(nx=64, ny=40, num_phonons=30000, num_measurements=120, sim_time=0.12),
                     os.path.join(str(tmp_path), "plate_2560.json")) if name == "plate_2560" else model_path(name))
    ref = None
    # (staging, steps per launch, coasting lanes, survivor grouping, chunked run with growing buffers,
    # free lanes per fetch, warp work pool, overlapped loop tail)
    for stage, fuse, coast, sort, chunked, fetch, pool, tail in (
            ("1", "1", "0", "0", "0", "1", "0", "0"), ("1", "3", "16", "0", "0", "4", "0", "0"), ("1", "8", "1", "0", "0", "4", "0", "0"),
            ("1", "16", "32", "0", "0", "2", "0", "0"), ("0", "5", "16", "0", "0", "4", "0", "0"), ("2", "7", "16", "0", "0", "4", "0", "0"),
            ("2", "2", "0", "0", "0", "8", "0", "0"), ("1", "8", "0", "1:9", "0", "4", "0", "0"), ("1", "6", "0", "2:5000", "1", "4", "0", "0"),
            ("1", "4", "0", "1:4", "1", "4", "0", "0"), ("1", "9", "0", "0", "1", "4", "32", "1"), ("0", "3", "0", "0", "0", "1", "64", "1")):
        monkeypatch.setenv("PSIM_GB300_STAGE", stage)
        monkeypatch.setenv("PSIM_GB300_FUSE", fuse)
        monkeypatch.setenv("PSIM_GB300_COAST", coast)
        monkeypatch.setenv("PSIM_GB300_SORT", sort)
        monkeypatch.setenv("PSIM_GB300_CHUNKED", chunked)
        monkeypatch.setenv("PSIM_GB300_FETCH", fetch)
        monkeypatch.setenv("PSIM_GB300_POOL", pool)
        monkeypatch.setenv("PSIM_GB300_TAIL", tail)
        m = api.Model(path)
        m.run(seed=11)
        e, f = m.tallies()
        c = m.counters()
        got = (e, f, m.population(), c["phonon_steps"], c["max_population"])
        assert c["steps_per_launch"] == int(fuse)
        assert c["transport_launches"] == -(-m.n_steps // int(fuse))
        if ref is None:
            ref = got
            continue
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1]), (stage, fuse)
        assert np.array_equal(ref[2], got[2]), (stage, fuse)
        assert ref[3:] == got[3:], (stage, fuse)
    monkeypatch.delenv("PSIM_GB300_STAGE")
    monkeypatch.delenv("PSIM_GB300_FUSE")
    monkeypatch.delenv("PSIM_GB300_COAST")
    monkeypatch.delenv("PSIM_GB300_SORT")
    monkeypatch.delenv("PSIM_GB300_CHUNKED")
    for var in ("PSIM_GB300_FETCH", "PSIM_GB300_POOL", "PSIM_GB300_TAIL"):
        monkeypatch.delenv(var)


def test_counters_and_phonon_steps(api):
    m = api.Model(model_path("bar_ss"))
    m.run(seed=3)
    c = m.counters()
    assert c["phonons"] > 90000
    assert c["phonon_steps"] > c["phonons"]
    # 1000 steps: ceil(1000 / steps per launch) transport launches and one population pass
    assert 1 <= c["steps_per_launch"] <= 16
    assert c["transport_launches"] == -(-1000 // c["steps_per_launch"])
    assert c["kernel_launches"] == c["transport_launches"] + 1
    assert c["max_population"] > 0
    assert c["kernel_ms"] > 0
    # SS records the last 10 % of steps: every tallied phonon-step adds its sign; the net
    # count can never exceed the phonon-steps taken
    e, _ = m.tallies()
    assert np.abs(e).sum() <= c["phonon_steps"]


def test_seam_matches_model_statistically(api):
    """psim_sim_* driven directly (the ModelSimulator seam) with the model's own description
    and emitter energies taken from the reference's tables gives the reference's result."""
    gold_r = np.load(os.path.join(GOLDEN, "runs_bar_ss.npz"))["stats"]
    m = api.Model(model_path("bar_ss"))
    d = m.sim_desc()
    sim = api.Simulator(d)
    idesc = m.interp_desc()
    t_eq = idesc.t_eq
    emit = emit_energies_bar_ss(d, t_eq)
    cell = np.zeros(d.n_cells)  # the sensors start at t_eq: no initial phonons
    S = d.n_sensors
    init_t = np.ctypeslib.as_array(idesc.sensor_init_temp, shape=(S,)).copy()
    eff = idesc.eff_energy
    out = []
    for seed in range(1, 17):
        sim.reset()
        n = sim.init_phonon_builders(t_eq, eff, cell, emit, init_t, seed)
        assert n > 0
        sim.run(t_eq)
        energy, flux = sim.tallies()
        _, _, stats = api.interpret(idesc, energy, flux)
        out.append(stats)
    got = np.stack(out)
    # the seam applies no post-run energy rescaling (that is Model's job), so compare the
    # temperature rise profile shape: ordered along the bar like the reference's
    t_got = got[:, :, 0].mean(axis=0)
    t_ref = gold_r[:, :, 0].mean(axis=0)
    assert np.all(np.diff(t_got) < 0) and np.all(np.diff(t_ref) < 0)
    assert np.corrcoef(t_got, t_ref)[0, 1] > 0.99


def test_two_shards_match_one_job(api):
    """A job split over two ranks (run one after the other on this device, tallies summed as
    the all-reduce would) has the unsplit job's expected temperatures and phonon count."""
    from psim_gb300 import shard
    m = api.Model(model_path("bar_ss"))
    d = m.sim_desc()
    idesc = m.interp_desc()
    sim = api.Simulator(d)
    t_eq, eff = idesc.t_eq, idesc.eff_energy
    emit = emit_energies_bar_ss(d, t_eq)
    cell = np.zeros(d.n_cells)
    init_t = np.ctypeslib.as_array(idesc.sensor_init_temp, shape=(d.n_sensors,)).copy()
    one, two, n_one, n_two = [], [], [], []
    for seed in range(1, 9):
        sim.reset()
        n_one.append(sim.init_phonon_builders(t_eq, eff, cell, emit, init_t, seed))
        sim.run(t_eq)
        e, f = sim.tallies()
        one.append(api.interpret(idesc, e, f)[2][:, 0])
        counts = []

        def rank(r):
            sim.reset()
            counts.append(sim.init_phonon_builders(t_eq, shard.rank_eff_energy(eff, 2), cell, emit, init_t,
                                                   shard.rank_seed(100 + seed, r)))
            sim.run(t_eq)
            return sim.tallies()

        e, f = shard.local_world(2, rank)
        n_two.append(sum(counts))
        two.append(api.interpret(idesc, e, f)[2][:, 0])
    one, two = np.array(one), np.array(two)
    assert abs(np.mean(n_two) / np.mean(n_one) - 1) < 0.01
    se = np.sqrt(one.var(axis=0, ddof=1) / len(one) + two.var(axis=0, ddof=1) / len(two))
    z = (one.mean(axis=0) - two.mean(axis=0)) / np.maximum(se, 1e-9)
    assert np.abs(z).max() < 4.5, z


def emit_energies_bar_ss(d, t_eq):
    """Emitter energies from the reference's tables (as the ModelSimulator seam receives them)."""
    gold_t = np.load(os.path.join(GOLDEN, "tables_bar_ss.npz"))
    E = d.n_emitters
    lines = np.ctypeslib.as_array(d.emit_line, shape=(E, 4))
    et = np.ctypeslib.as_array(d.emit_temp, shape=(E,))
    dur = np.ctypeslib.as_array(d.emit_duration, shape=(E,))
    emit = np.zeros(E)
    for e in range(E):
        k = int(np.searchsorted(gold_t["temps"], et[e]))
        length = np.hypot(lines[e, 2] - lines[e, 0], lines[e, 3] - lines[e, 1])
        emit[e] = gold_t["emit_sum"][k] * dur[e] * length / 4.0 * abs(t_eq - et[e])
    return emit


def test_export_writes_reference_format(api):
    with tempfile.TemporaryDirectory() as td:
        for name, prefix, kind in (("bar_ss", "ss_", "Steady State"), ("bar_periodic", "per_", "Periodic"),
                                   ("plate_small", "per_", "Periodic")):
            p = os.path.join(td, name + ".json")
            shutil.copy(model_path(name), p)
            m = api.Model(p)
            m.run(seed=1)
            m.export(p, 1.5)
            text = open(os.path.join(td, prefix + name + ".txt")).read().splitlines()
            assert re.match(rf'^{kind} Results from "{name}\.json" @ \d{{4}}-\d\d-\d\d \d\d:\d\d:\d\d - Time Taken 1\.5\[s\] over 1 runs$', text[0])
            if prefix == "ss_":
                assert len(text) == 1 + m.n_sensors
                vals = np.array([[float(v) for v in line.split()] for line in text[1:]])
                assert vals.shape == (m.n_sensors, 6)
                assert np.allclose(vals, m.measurements(), rtol=1e-5)
            else:
                interval = 25 if name == "bar_periodic" else 20
                blocks = m.n_recorded // interval
                assert len(text) == 1 + blocks * (2 + m.n_sensors)
                assert int(text[1]) == interval // 2 and int(text[2]) == m.n_sensors
                temps, fluxes = m.series(0)
                first = np.array([float(v) for v in text[3].split()])
                assert np.allclose(first, [temps[0, :interval].mean(), fluxes[0, :interval, 0].mean(),
                                           fluxes[0, :interval, 1].mean()], rtol=1e-5)


def test_transient_pulse_spreads_and_conserves(api):
    """Plate with a 20 ps pulse: energy enters only during the pulse, then only moves."""
    m = api.Model(model_path("plate_small"))
    m.run(seed=2)
    temps, _ = m.series(0)
    e, _ = m.tallies()
    total = e.sum(axis=0)
    # after the pulse there are no absorbing surfaces: the net count is constant
    assert np.all(total[30:] == total[30])
    # heat reaches the far side later than the near side
    near = temps[0:4, :].mean(axis=0)
    far = temps[-4:, :].mean(axis=0)
    assert near[:100].max() > far[:100].max()


def test_phasor_mode_runs(api):
    m = api.Model(model_path("bar_phasor"))
    m.run(seed=4)
    c = m.counters()
    assert c["phonon_steps"] > 0
    st = m.measurements()
    assert np.all(np.isfinite(st))
