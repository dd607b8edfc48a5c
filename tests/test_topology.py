"""Model assembly without a GPU: the flattened model libpsim_gb300 hands to its kernels equals
the reference's assembled Model, bit for bit, on every model file of the fixtures, the
reference's three demo models included (up to 6174 cells).

What is compared, per cell and per edge (psim/src/model.cpp:98-138, psim/src/cell.cpp:13-124,
psim/src/compositeSurface.cpp:20-45):
- the triangle's vertices, its sensor (Model::getSensor by ID) and the clamped specularity of
  its three boundary surfaces;
- the sub-surfaces of each edge in CompositeSurface order: the transition surfaces
  (Cell::findTransitionSurface) with their neighbour cell and line, then the emitting surfaces
  (Model::setEmitSurface) with their owning cell, line, temperature, duration and start time.
The fixtures come from the reference built from its own sources (tests/golden/make_golden.py,
``ref_driver topology``)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, demo_model_path, model_path

NAMES = sorted(os.path.basename(p)[len("topology_"):-len(".npz")] for p in glob.glob(os.path.join(GOLDEN, "topology_*.npz")))
DEMOS = ("linear_demo", "linear_sides_demo_ss", "kinked_demo_120_35_spec")


@pytest.fixture(scope="module")
def api(built):
    from psim_gb300 import api
    return api


def test_every_model_file_has_a_fixture():
    files = {os.path.basename(p).split(".")[0] for p in glob.glob(os.path.join(GOLDEN, "models", "*.json*"))}
    assert files == set(NAMES), sorted(files ^ set(NAMES))
    assert set(DEMOS) <= set(NAMES)


def arr(ptr, shape, dtype=None):
    n = int(np.prod(shape))
    if n == 0:
        return np.zeros(shape, dtype=dtype or np.float64)
    return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(shape).copy()


@pytest.mark.parametrize("name", NAMES)
def test_assembly_matches_reference(api, name, tmp_path):
    gold = np.load(os.path.join(GOLDEN, f"topology_{name}.npz"))
    path = demo_model_path(name, str(tmp_path)) if name in DEMOS else model_path(name)
    m = api.Model(path)
    d = m.sim_desc()  # arrays point into m, which stays alive below
    C = d.n_cells
    assert C == len(gold["cell_sensor"])
    # cells: vertices bit for bit, sensor, specularity of every edge
    assert np.array_equal(arr(d.cell_vertices, (C, 6)), gold["cell_vertices"])
    assert np.array_equal(arr(d.cell_sensor, (C,)).astype(np.int64), gold["cell_sensor"])
    spec = arr(d.cell_spec, (C,))
    assert np.array_equal(np.repeat(spec[:, None], 3, axis=1), gold["cell_spec"])

    # edge sub-surfaces in the reference's order: the fixture lists them by (cell, edge), in order
    begin = arr(d.edge_sub_begin, (3 * C + 1,)).astype(np.int64)
    n = d.n_subs
    assert n == len(gold["sub_kind"]) and begin[-1] == n
    owner = np.repeat(np.arange(3 * C), np.diff(begin))
    assert np.array_equal(owner // 3, gold["sub_cell"])
    assert np.array_equal(owner % 3, gold["sub_edge"])
    kind = arr(d.sub_kind, (n,)).astype(np.int64)
    target = arr(d.sub_target, (n,)).astype(np.int64)
    line = arr(d.sub_line, (n, 4))
    assert np.array_equal(kind, gold["sub_kind"])
    assert np.array_equal(line, gold["sub_line"])
    trans = kind == 0
    assert np.array_equal(target[trans], gold["sub_target"][trans])

    # emitting sub-surfaces point at emitters that hold the reference's values
    E = d.n_emitters
    emit = ~trans
    assert E == int(emit.sum())
    k = target[emit]
    assert np.array_equal(np.sort(k), np.arange(E))  # each emitter on exactly one edge
    ecell = arr(d.emit_cell, (E,)).astype(np.int64)
    eedge = arr(d.emit_edge, (E,)).astype(np.int64)
    assert np.array_equal(ecell[k], gold["sub_target"][emit])
    assert np.array_equal(ecell[k], gold["sub_cell"][emit])
    assert np.array_equal(eedge[k], gold["sub_edge"][emit])
    assert np.array_equal(arr(d.emit_line, (E, 4))[k], gold["sub_line"][emit])
    vals = np.stack([arr(d.emit_temp, (E,)), arr(d.emit_duration, (E,)), arr(d.emit_start, (E,))], axis=1)
    assert np.array_equal(vals[k], gold["sub_emit"][emit])
    m.close()
