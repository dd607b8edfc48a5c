"""Host side of libpsim_gb300 without a GPU: the C ABI's exports, model loading and
validation (the reference's InputManager / Model::addCell / setEmitSurface rules), the
material tables it builds (bit-exact with the reference's), and that every GPU entry point
fails loudly when no device is present."""
import json
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, model_path


@pytest.fixture(scope="module")
def api(built):
    from psim_gb300 import api
    return api


def header_symbols():
    text = open(os.path.join(ROOT, "include", "psim_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(psim_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(api):
    declared = header_symbols()
    assert len(declared) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", api.lib_path()], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (psim_[a-z0-9_]+)$", out, flags=re.M))
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    # and the ctypes table covers the same set
    assert sorted(api.SIGNATURES) == declared
    for name in declared:
        assert getattr(api.lib(), name) is not None


def test_model_shape(api):
    m = api.Model(model_path("bar_ss"))
    assert (m.n_sensors, m.n_cells, m.n_steps, m.n_recorded, m.n_runs) == (10, 20, 1000, 100, 1)
    k = api.Model(model_path("kinked_small"))
    assert k.n_sensors == 64 and k.n_cells == 129 and k.n_recorded == 400
    p = api.Model(model_path("plate_small"))
    assert p.n_sensors == 64 and p.n_cells == 128 and p.n_recorded == 400
    d = p.sim_desc()
    assert d.n_emitters == 2 and d.sim_type == 2


def test_topology_of_bar(api):
    """Transition surfaces on every shared edge, emitters on the two ends (cell.cpp:81-98)."""
    m = api.Model(model_path("bar_ss"))
    d = m.sim_desc()  # arrays point into m, which must stay alive
    C = d.n_cells
    begin = np.ctypeslib.as_array(d.edge_sub_begin, shape=(3 * C + 1,))
    kind = np.ctypeslib.as_array(d.sub_kind, shape=(d.n_subs,))
    assert (kind == 0).sum() == 2 * 19  # 10 diagonals + 9 shared rectangle edges, both sides
    assert (kind == 1).sum() == 2
    edge_cell = np.ctypeslib.as_array(d.emit_cell, shape=(2,))
    assert set(edge_cell.tolist()) == {0, 19}
    assert begin[-1] == d.n_subs


@pytest.mark.parametrize("name", ["bar_ss", "bar_full", "kinked_small"])
def test_tables_match_reference(api, name):
    """The cumulative tables handed to the GPU equal the reference's Material tables."""
    gold = np.load(os.path.join(GOLDEN, f"tables_{name}.npz"))
    m = api.Model(model_path(name))
    d = m.sim_desc()
    tabs = m.tables()
    temps = gold["temps"]
    keep = list(gold["keep"])
    S = d.n_sensors
    st = np.ctypeslib.as_array(d.sensor_temp, shape=(S,))
    base_idx = np.ctypeslib.as_array(d.sensor_base_table, shape=(S,))
    scat_idx = np.ctypeslib.as_array(d.sensor_scatter_table, shape=(S,))
    exact = os.uname().machine == "x86_64"

    def same(a, b):
        a = np.nan_to_num(a, nan=-1.0)
        b = np.nan_to_num(b, nan=-1.0)
        return np.array_equal(a, b) if exact else np.allclose(a, b, rtol=1e-12, atol=0)

    checked = 0
    for s in range(S):
        ti = int(np.searchsorted(temps, st[s]))
        if ti in keep:
            k = keep.index(ti)
            assert same(tabs[base_idx[s]], gold["base"][k])
            assert same(tabs[scat_idx[s]], gold["scatter"][k])
            checked += 1
    E = d.n_emitters
    et = np.ctypeslib.as_array(d.emit_temp, shape=(E,))
    ei = np.ctypeslib.as_array(d.emit_table, shape=(E,))
    for e in range(E):
        ti = int(np.searchsorted(temps, et[e]))
        if ti in keep:
            assert same(tabs[ei[e]], gold["emit"][keep.index(ti)])
            checked += 1
    assert checked > 0
    freq = np.ctypeslib.as_array(d.mat_freq, shape=(1000,))
    vel = np.ctypeslib.as_array(d.mat_vel, shape=(2, 1000))
    assert same(freq, gold["freq"]) and same(vel[0], gold["vel_la"]) and same(vel[1], gold["vel_ta"])
    idesc = m.interp_desc()
    n = idesc.mat_temp_begin[1]
    assert np.array_equal(np.ctypeslib.as_array(idesc.temps, shape=(n,)), temps)
    assert same(np.ctypeslib.as_array(idesc.energies, shape=(n,)), gold["base_sum"])
    assert (idesc.lower_bound, idesc.upper_bound) == tuple(gold["bounds"])


def test_tables_of_two_materials_match_reference(api):
    """A model of two materials (silicon and germanium cells): each material's frequency grid,
    velocities and temperature sums, and the cumulative tables each sensor and emitter uses,
    equal the reference's (Material::Material and initializeTables per material,
    psim/src/material.cpp:20-51,101-204; Model::initializeMaterialTables)."""
    gold = np.load(os.path.join(GOLDEN, "tables_si_ge_bar.npz"))
    m = api.Model(model_path("si_ge_bar"))
    d = m.sim_desc()
    assert d.n_materials == 2
    tabs = m.tables()
    exact = os.uname().machine == "x86_64"

    def same(a, b):
        a = np.nan_to_num(a, nan=-1.0)
        b = np.nan_to_num(b, nan=-1.0)
        return np.array_equal(a, b) if exact else np.allclose(a, b, rtol=1e-12, atol=0)

    S = d.n_sensors
    st = np.ctypeslib.as_array(d.sensor_temp, shape=(S,))
    smat = np.ctypeslib.as_array(d.sensor_material, shape=(S,))
    base_idx = np.ctypeslib.as_array(d.sensor_base_table, shape=(S,))
    scat_idx = np.ctypeslib.as_array(d.sensor_scatter_table, shape=(S,))
    freq = np.ctypeslib.as_array(d.mat_freq, shape=(2, 1000))
    vel = np.ctypeslib.as_array(d.mat_vel, shape=(2, 2, 1000))
    idesc = m.interp_desc()
    begin = [idesc.mat_temp_begin[i] for i in range(3)]
    all_temps = np.ctypeslib.as_array(idesc.temps, shape=(begin[2],))
    all_energies = np.ctypeslib.as_array(idesc.energies, shape=(begin[2],))
    checked = 0
    for i in range(2):
        temps = gold[f"m{i}_temps"]
        keep = list(gold[f"m{i}_keep"])
        assert same(freq[i], gold[f"m{i}_freq"])
        assert same(vel[i, 0], gold[f"m{i}_vel_la"]) and same(vel[i, 1], gold[f"m{i}_vel_ta"])
        assert np.array_equal(all_temps[begin[i]:begin[i + 1]], temps)
        assert same(all_energies[begin[i]:begin[i + 1]], gold[f"m{i}_base_sum"])
        for s in np.nonzero(smat == i)[0]:
            ti = int(np.searchsorted(temps, st[s]))
            if ti in keep:
                k = keep.index(ti)
                assert same(tabs[base_idx[s]], gold[f"m{i}_base"][k])
                assert same(tabs[scat_idx[s]], gold[f"m{i}_scatter"][k])
                checked += 1
    # the two materials' grids differ (germanium's branch maxima lie below silicon's)
    assert freq[1, -1] < freq[0, -1]
    assert checked >= 2
    assert (idesc.lower_bound, idesc.upper_bound) == tuple(gold["bounds"])


@pytest.mark.parametrize("name", ["bar_ss", "bar_full", "kinked_small"])
def test_energy_per_phonon_matches_reference(api, name):
    """Model::getTotalInitialEnergy / num_phonons (model.cpp:148-155,196-201)."""
    gold = np.load(os.path.join(GOLDEN, f"invert_{name}.npz"))
    m = api.Model(model_path(name))
    eff = m.interp_desc().eff_energy
    if os.uname().machine == "x86_64":
        assert eff == float(gold["eff"])
    else:
        assert eff == pytest.approx(float(gold["eff"]), rel=1e-12)


def _write(tmp, model):
    p = os.path.join(tmp, "m.json")
    with open(p, "w") as f:
        json.dump(model, f)
    return p


def test_validation_errors(api):
    from psim_gb300 import modelgen as mg
    with tempfile.TemporaryDirectory() as td:
        base = mg.bar(num_cells=3, num_phonons=1000, num_measurements=100, sim_time=1.0)
        # degenerate triangle (TriangleError)
        m = json.loads(json.dumps(base))
        m["cells"][0]["triangle"]["p2"] = dict(m["cells"][0]["triangle"]["p1"])
        with pytest.raises(api.PsimError, match="valid triangle"):
            api.Model(_write(td, m))
        # duplicate cell: found when the copy is checked against itself after the original
        # (model.cpp:102-111); a copy added later first collides with the original's
        # transition surfaces, as in the reference
        m = json.loads(json.dumps(base))
        m["cells"].insert(0, dict(m["cells"][0]))
        with pytest.raises(api.PsimError, match="Duplicate cell"):
            api.Model(_write(td, m))
        m = json.loads(json.dumps(base))
        m["cells"].append(dict(m["cells"][0]))
        with pytest.raises(api.PsimError, match="conflicts"):
            api.Model(_write(td, m))
        # overlapping cell (IntersectError)
        m = json.loads(json.dumps(base))
        m["cells"].append({"triangle": {"p1": {"x": 10.0, "y": 10.0}, "p2": {"x": 10.0, "y": 150.0},
                                        "p3": {"x": 150.0, "y": 10.0}}, "sensorID": 0, "specularity": 0.0})
        with pytest.raises(api.PsimError, match="intersects|contained"):
            api.Model(_write(td, m))
        # emitting surface that lies on no cell edge
        m = json.loads(json.dumps(base))
        m["emit_surfaces"].append({"p1": {"x": 50.0, "y": 20.0}, "p2": {"x": 50.0, "y": 80.0}, "temp": 300.0,
                                   "duration": 1.0, "start_time": 0.0, "length": 1.0})
        with pytest.raises(api.PsimError, match="emitting surface|conflicts"):
            api.Model(_write(td, m))
        # transient emitter in a steady-state model
        m = json.loads(json.dumps(base))
        m["emit_surfaces"][0]["duration"] = 0.5
        with pytest.raises(api.PsimError, match="non transient"):
            api.Model(_write(td, m))
        # unknown sensor
        m = json.loads(json.dumps(base))
        m["cells"][0]["sensorID"] = 99
        with pytest.raises(api.PsimError, match="Sensor does not exist"):
            api.Model(_write(td, m))
        # steady state with a step interval
        m = json.loads(json.dumps(base))
        m["settings"]["step_interval"] = 5
        api.Model(_write(td, m))  # the reference ignores step_interval for sim_type 0 (inputManager.cpp:81-82)
        # transient in full mode
        m = json.loads(json.dumps(base))
        m["settings"]["sim_type"] = 2
        m["settings"]["step_interval"] = 5
        m["settings"]["t_eq"] = 0.0
        with pytest.raises(api.PsimError, match="deviational"):
            api.Model(_write(td, m))
        with pytest.raises(api.PsimError) as e:
            api.Model(os.path.join(td, "missing.json"))
        assert e.value.code == api.PSIM_ERR_IO
        with open(os.path.join(td, "bad.json"), "w") as f:
            f.write("{ not json")
        with pytest.raises(api.PsimError, match="JSON"):
            api.Model(os.path.join(td, "bad.json"))


def test_gpu_entry_points_fail_loudly_without_a_device(api):
    if api.device_count() > 0:
        pytest.skip("a CUDA device is present")
    m = api.Model(model_path("bar_ss"))
    with pytest.raises(api.PsimError) as e:
        m.run(seed=1)
    assert e.value.code == api.PSIM_ERR_CUDA
    with pytest.raises(api.PsimError) as e:
        api.Simulator(m.sim_desc())
    assert e.value.code == api.PSIM_ERR_CUDA
    g = np.load(os.path.join(GOLDEN, "geom.npz"))
    with pytest.raises(api.PsimError):
        api.geom_intersect(g["intersect_a"][:4], g["intersect_b"][:4])


def test_interpreter_rejects_decreasing_material_offsets(api):
    """A second material whose temperature-grid offset decreases would let the first material's
    lookups run past the grid the call copies: refused before any device work."""
    import ctypes
    m = api.Model(model_path("bar_ss"))
    d = m.interp_desc()
    assert d.n_materials == 1
    n = int(np.ctypeslib.as_array(d.mat_temp_begin, shape=(2,))[1])
    bad = np.array([0, n, n // 2], dtype=np.uint64)
    d.n_materials = 2
    d.mat_temp_begin = bad.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    counts = np.zeros((d.n_sensors, d.recorded_steps), dtype=np.int64)
    with pytest.raises(api.PsimError) as e:
        api.final_temps(d, counts, 0)
    assert e.value.code == api.PSIM_ERR_INVALID and "decreases" in str(e.value)


def test_modelgen_workloads_load(api):
    from psim_gb300 import modelgen as mg
    with tempfile.TemporaryDirectory() as td:
        k = api.Model(mg.write(mg.kinked(num_phonons=1000, num_measurements=100, sim_time=1.0), os.path.join(td, "k.json")))
        # (k stays alive while its description is read)
        assert k.n_sensors == 400 and k.n_cells == 801
        d = k.sim_desc()
        assert d.n_emitters == 6
        p = api.Model(mg.write(mg.plate(num_phonons=1000), os.path.join(td, "p.json")))
        assert p.n_sensors == 1024 and p.n_cells == 2048 and p.sim_desc().n_emitters == 4


def test_start_temperatures_are_checked_and_reset(api):
    m = api.Model(model_path("bar_periodic"))
    t0 = m.start_temps()
    assert t0.shape == (m.n_sensors,) and np.all(t0 > 0)
    warm = np.linspace(305.0, 295.0, m.n_sensors)
    m.set_start_temps(warm)
    assert np.array_equal(m.start_temps(), warm)
    m.set_start_temps(None)
    assert np.array_equal(m.start_temps(), t0)
    bad = warm.copy()
    bad[1] = -1.0
    with pytest.raises(api.PsimError) as e:
        m.set_start_temps(bad)
    assert e.value.code == api.PSIM_ERR_INVALID
    full = api.Model(model_path("bar_full"))
    with pytest.raises(api.PsimError) as e:
        full.set_start_temps(np.full(full.n_sensors, 50.0))
    assert e.value.code == api.PSIM_ERR_INVALID


def test_command_line_messages(api, tmp_path):
    """The psim_gb300 command line prints the reference's messages (psim/src/main.cpp:10-31)
    and reports a failed file through its exit status."""
    import subprocess
    from psim_gb300 import build
    cli = build.CLI
    out = subprocess.run([cli], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout == "Need filenames\ndone\n"
    missing = str(tmp_path / "missing.json")
    out = subprocess.run([cli, missing], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and out.stdout.endswith("done\n")
    assert f'There was an error reading the data from the file at "{missing}"' in out.stderr
    if api.device_count() == 0:  # no device: the run fails loudly, nothing is written
        out = subprocess.run([cli, model_path("bar_ss")], capture_output=True, text=True, timeout=60)
        assert out.returncode == 1 and "run failed" in out.stderr and "CUDA" in out.stderr
        assert not os.path.exists(os.path.join(os.path.dirname(model_path("bar_ss")), "ss_bar_ss.txt"))


def test_rate_inputs_are_refused_before_any_device_work(api, tmp_path):
    """A negative relaxation coefficient or a non-positive sensor temperature would make a
    scattering rate negative; the kernels' event loops cannot end a step with a negative
    scattering time, so such inputs are refused on the host, at load and at the simulator seam.
    The seam also refuses a non-positive simulated time and emitting windows outside it."""
    import ctypes
    from psim_gb300 import modelgen as mg
    base = mg.bar(num_cells=3, num_phonons=1000, num_measurements=100, sim_time=1.0)
    m = json.loads(json.dumps(base))
    m["materials"][0]["r_data"]["b_i"] = -1.2e-45
    with pytest.raises(api.PsimError, match="Relaxation coefficients") as e:
        api.Model(_write(str(tmp_path), m))
    assert e.value.code == api.PSIM_ERR_INVALID
    for t in (0.0, -5.0):
        m = json.loads(json.dumps(base))
        m["sensors"][1]["t_init"] = t
        with pytest.raises(api.PsimError, match="Sensor temperature"):
            api.Model(_write(str(tmp_path), m))
    # the tables hold one temperature per 0.1 K between the model's lowest and highest: a span
    # beyond the grid limit is a size error, found before anything is allocated
    m = json.loads(json.dumps(base))
    m["sensors"][1]["t_init"] = 1e12
    with pytest.raises(api.PsimError, match="span more than 5000 K") as e:
        api.Model(_write(str(tmp_path), m))
    assert e.value.code == api.PSIM_ERR_LIMIT
    m = json.loads(json.dumps(base))
    m["emit_surfaces"][0]["temp"] = -5.0
    with pytest.raises(api.PsimError, match="Emitting surface temperature"):
        api.Model(_write(str(tmp_path), m))
    # the simulator seam takes the rate temperatures and coefficients from its caller
    model = api.Model(model_path("bar_ss"))
    d = model.sim_desc()
    temps = np.ctypeslib.as_array(d.sensor_temp, shape=(d.n_sensors,)).copy()
    params = np.ctypeslib.as_array(d.mat_params, shape=(8 * d.n_materials,)).copy()
    for bad in (0.0, -300.0, np.nan, np.inf):
        t = temps.copy()
        t[3] = bad
        d.sensor_temp = t.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        with pytest.raises(api.PsimError, match="sensor temperatures") as e:
            api.Simulator(d)
        assert e.value.code == api.PSIM_ERR_INVALID
    d.sensor_temp = temps.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    for k, bad in ((0, -2e-24), (3, np.nan), (2, np.inf)):
        p = params.copy()
        p[k] = bad
        d.mat_params = p.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        with pytest.raises(api.PsimError, match="relaxation coefficients") as e:
            api.Simulator(d)
        assert e.value.code == api.PSIM_ERR_INVALID
    d.mat_params = params.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    # and the time line: a positive simulated time, emitting windows inside it
    sim_time = d.simulation_time
    for bad in (0.0, -1.0, np.nan):
        d.simulation_time = bad
        with pytest.raises(api.PsimError, match="simulation.time"):
            api.Simulator(d)
    d.simulation_time = sim_time
    start = np.ctypeslib.as_array(d.emit_start, shape=(d.n_emitters,)).copy()
    dur = np.ctypeslib.as_array(d.emit_duration, shape=(d.n_emitters,)).copy()
    for s0, du in ((-0.1, 0.5), (sim_time, 0.0), (0.0, sim_time * 1.01), (0.5 * sim_time, 0.6 * sim_time), (0.0, -1.0)):
        s1, d1 = start.copy(), dur.copy()
        s1[1], d1[1] = s0, du
        d.emit_start = s1.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.emit_duration = d1.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        with pytest.raises(api.PsimError, match="emitter start time or duration") as e:
            api.Simulator(d)
        assert e.value.code == api.PSIM_ERR_INVALID
    model.close()


@pytest.mark.parametrize("name", ["bar_runs", "bar_ss", "si_ge_bar"])
def test_steady_state_table_is_byte_identical_to_reference_writer(api, name, tmp_path):
    """OutputManager::exportResults / calculateAverages / steadyStateExport
    (psim/src/outputManager.cpp:13-38,40-78) against the table the reference itself wrote for
    a seeded run (tests/golden/export_<name>.npz): fed the same per-run statistics, the writer
    gives the same body, byte for byte, and the same header up to its date and time."""
    import re
    gold = np.load(os.path.join(GOLDEN, f"export_{name}.npz"))
    src = model_path(name)
    model_file = os.path.join(str(tmp_path), name + ".json")
    with open(src, "rb") as f, open(model_file, "wb") as g:
        g.write(f.read())
    m = api.Model(model_file)
    m.set_measurements(gold["stats"])
    m.export(model_file, 0.0)
    text = open(os.path.join(str(tmp_path), f"ss_{name}.txt"), "rb").read()
    header, body = text.split(b"\n", 1)
    assert body == gold["body"].tobytes()
    date = rb"\d{4}-\d\d-\d\d \d\d:\d\d:\d\d"
    assert re.sub(date, b"DATE", header) == re.sub(date, b"DATE", gold["header"].tobytes())
    # the averaged statistics behind the table are the reference's calculateAverages
    assert np.allclose(m.measurements(), gold["stats"].mean(axis=0), rtol=1e-15, atol=0)


def test_periodic_export_needs_per_step_series(api, tmp_path):
    """Statistics set from elsewhere carry no per-step series: a periodic table of them is refused."""
    m = api.Model(model_path("bar_periodic"))
    m.set_measurements(np.zeros((1, m.n_sensors, 6)))
    with pytest.raises(Exception, match="per-step series"):
        m.export(os.path.join(str(tmp_path), "p.json"), 0.0)
