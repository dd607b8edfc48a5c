"""Seeded synthetic psim model files (the JSON schema psim reads).

The schema is the one psim_python's ModelBuilder writes
(psim_python/psim/builder_tools.py:187-238, 546-576) and psim reads
(psim/src/inputManager.cpp:17-105):

    settings{num_runs, num_measurements, sim_time [ns], num_phonons, t_eq,
             sim_type 0|1|2, step_interval, phasor_sim}
    materials[{name, d_data{la_data[3], max_freq_la, ta_data[3], max_freq_ta},
               r_data{b_l, b_tn, b_tu, b_i, w}}]
    sensors[{id, material, t_init}]
    cells[{triangle{p1, p2, p3: {x, y} [nm]}, sensorID, specularity}]
    emit_surfaces[{p1, p2, temp, duration [ns], start_time [ns], length}]

Rectangles are split into two triangles the way ModelBuilder.addRectangularCell
does (builder_tools.py:403-413) and quadrilaterals the way addQuadrilateralCell
does (builder_tools.py:433-462), so transition surfaces come out as full shared
edges.  Every emitting surface lies on a single cell edge (psim attaches an
emitting surface to the first cell edge that contains it, psim/src/model.cpp:125-138).

The workloads here are the named benchmark shapes:

* ``bar``      1000 x 100 nm bar, 10 cells, 310/290 K ends (deviational steady state)
               and the same bar in full mode at 60/40 K.
* ``kinked``   three 2000 x 200 nm arms meeting at a hub, with a 90 degree and a
               45 degree bend between them; 400 quadrilateral cells / sensors.
* ``plate``    4000 x 1000 nm plate, 64 x 16 cells, a 200 nm heat-pulse strip on
               the left edge that emits for 20 ps (transient).
* ``random_bar``  a seeded rectangle for the batched workload.
"""
from __future__ import annotations

import json
import math
import random
from typing import Dict, List, Sequence, Tuple

Point = Tuple[float, float]

# Si-like material: quadratic dispersion w = c0 k^2 + c1 k + c2 (SI units) with the
# branch maxima taken at k_max = 1.157e10 /m, and Holland relaxation coefficients
# (psim_python/psim/pre_builts.py:15-18 gives the same coefficient set).
K_MAX = 1.157e10
LA = (-2.0e-7, 9.01e3, 0.0)
TA = (-2.26e-7, 5.23e3, 0.0)


def _w_max(c: Sequence[float]) -> float:
    return c[0] * K_MAX * K_MAX + c[1] * K_MAX + c[2]


SILICON = {
    "name": "Silicon",
    "d_data": {
        "la_data": list(LA),
        "max_freq_la": _w_max(LA),
        "ta_data": list(TA),
        "max_freq_ta": _w_max(TA),
    },
    "r_data": {"b_l": 2.0e-24, "b_tn": 9.3e-13, "b_tu": 5.5e-18, "b_i": 1.2e-45, "w": 2.417e13},
}

# Germanium: the dispersion and relaxation set psim ships beside silicon
# (psim_python/psim/pre_builts.py:25-29).  Its branch maxima lie below silicon's, so a
# silicon phonon above them is backscattered at a Si|Ge interface
# (TransitionSurface::handlePhonon, psim/src/surface.cpp:71-109); its impurity
# coefficient is zero.
GERMANIUM = {
    "name": "Germanium",
    "d_data": {
        "la_data": [-1.50e-7, 5.63e3, 0.0],
        "max_freq_la": 4.45236386e13,
        "ta_data": [-1.13e-7, 2.60e3, 0.0],
        "max_freq_ta": 1.4937724175e13,
    },
    "r_data": {"b_l": 2.3e-24, "b_tn": 30.0e-13, "b_tu": 1.5e-18, "b_i": 0.0, "w": 1.23e13},
}


class Builder:
    """Accumulates sensors, cells and emitting surfaces in psim's JSON layout."""

    def __init__(self, *, num_measurements: int, sim_time: float, num_phonons: int, t_eq: float,
                 sim_type: int = 0, step_interval: int = 0, num_runs: int = 1, phasor_sim: bool = False,
                 material: dict = SILICON):
        self.settings = {
            "num_runs": int(num_runs),
            "num_measurements": int(num_measurements),
            "sim_time": float(sim_time),
            "num_phonons": int(num_phonons),
            "t_eq": float(t_eq),
            "sim_type": int(sim_type),
            "step_interval": int(step_interval),
            "phasor_sim": bool(phasor_sim),
        }
        self.material = material
        self.materials: List[dict] = [material]
        self.sensors: List[dict] = []
        self.cells: List[dict] = []
        self.surfaces: List[dict] = []

    def add_sensor(self, t_init: float, material: dict = None) -> int:
        """A sensor of ``material`` (the builder's material by default; another one is added
        to the model's material list on first use)."""
        mat = self.material if material is None else material
        if all(m["name"] != mat["name"] for m in self.materials):
            self.materials.append(mat)
        sid = len(self.sensors)
        self.sensors.append({"id": sid, "material": mat["name"], "t_init": float(t_init)})
        return sid

    def add_triangle(self, p1: Point, p2: Point, p3: Point, sensor: int, spec: float) -> None:
        tri = {"p1": {"x": p1[0], "y": p1[1]}, "p2": {"x": p2[0], "y": p2[1]}, "p3": {"x": p3[0], "y": p3[1]}}
        self.cells.append({"triangle": tri, "sensorID": int(sensor), "specularity": float(spec)})

    def add_rectangle(self, lo: Point, hi: Point, sensor: int, spec: float) -> None:
        # Same split as ModelBuilder.addRectangularCell.
        self.add_triangle(lo, (lo[0], hi[1]), (hi[0], lo[1]), sensor, spec)
        self.add_triangle(hi, (hi[0], lo[1]), (lo[0], hi[1]), sensor, spec)

    def add_quad(self, p1: Point, p2: Point, p3: Point, p4: Point, sensor: int, spec: float) -> None:
        # p1 anchor, p2 along the length, p3 across, p4 = opposite corner; split on the
        # p2-p3 diagonal as ModelBuilder.addQuadrilateralCell does.
        self.add_triangle(p1, p2, p3, sensor, spec)
        self.add_triangle(p4, p2, p3, sensor, spec)

    def add_surface(self, p1: Point, p2: Point, temp: float, duration: float = 0.0, start: float = 0.0) -> None:
        if duration == 0.0:
            duration = self.settings["sim_time"]
        length = (p2[1] - p1[1]) ** 2 + (p1[0] - p2[0]) ** 2  # written as ModelBuilder does; psim ignores it
        self.surfaces.append({"p1": {"x": p1[0], "y": p1[1]}, "p2": {"x": p2[0], "y": p2[1]},
                              "temp": float(temp), "duration": float(duration), "start_time": float(start),
                              "length": length})

    def to_dict(self) -> dict:
        # ModelBuilder sorts surfaces by decreasing 'length' before export.
        surfaces = sorted(self.surfaces, key=lambda s: s["length"], reverse=True)
        return {"settings": dict(self.settings), "materials": list(self.materials), "sensors": self.sensors,
                "cells": self.cells, "emit_surfaces": surfaces}


def write(model: dict, path: str) -> str:
    with open(path, "w", encoding="utf-8") as f:
        json.dump(model, f, indent=1)
    return path


def bar(*, num_cells: int = 10, length: float = 1000.0, width: float = 100.0, t_left: float = 310.0,
        t_right: float = 290.0, t_init: float = 300.0, t_eq: float = 300.0, spec: float = 0.0,
        num_measurements: int = 2000, sim_time: float = 10.0, num_phonons: int = 200000,
        sim_type: int = 0, step_interval: int = 0, num_runs: int = 1, phasor_sim: bool = False) -> dict:
    """A bar split lengthwise into ``num_cells`` rectangular cells, one sensor each, with
    emitting surfaces on the two short ends and walls of specularity ``spec``."""
    b = Builder(num_measurements=num_measurements, sim_time=sim_time, num_phonons=num_phonons, t_eq=t_eq,
                sim_type=sim_type, step_interval=step_interval, num_runs=num_runs, phasor_sim=phasor_sim)
    dx = length / num_cells
    for i in range(num_cells):
        s = b.add_sensor(t_init)
        b.add_rectangle((i * dx, 0.0), ((i + 1) * dx, width), s, spec)
    b.add_surface((0.0, 0.0), (0.0, width), t_left)
    b.add_surface((length, 0.0), (length, width), t_right)
    return b.to_dict()


def two_material_bar(*, num_cells: int = 10, split: int = 5, length: float = 1000.0, width: float = 100.0,
                     t_left: float = 310.0, t_right: float = 290.0, t_init: float = 300.0, t_eq: float = 300.0,
                     spec: float = 0.0, num_measurements: int = 1000, sim_time: float = 5.0,
                     num_phonons: int = 100000, sim_type: int = 0, step_interval: int = 0,
                     left: dict = SILICON, right: dict = GERMANIUM) -> dict:
    """The bar of ``bar`` with its first ``split`` cells of material ``left`` and the rest of
    ``right``: one interface between two materials, crossed by phonons both ways."""
    b = Builder(num_measurements=num_measurements, sim_time=sim_time, num_phonons=num_phonons, t_eq=t_eq,
                sim_type=sim_type, step_interval=step_interval, material=left)
    dx = length / num_cells
    for i in range(num_cells):
        s = b.add_sensor(t_init, left if i < split else right)
        b.add_rectangle((i * dx, 0.0), ((i + 1) * dx, width), s, spec)
    b.add_surface((0.0, 0.0), (0.0, width), t_left)
    b.add_surface((length, 0.0), (length, width), t_right)
    return b.to_dict()


def _arm_grid(origin: Point, angle_deg: float, length: float, width: float, n_len: int, n_wid: int,
              r0: float) -> List[List[Point]]:
    """Grid nodes of an arm that starts ``r0`` from ``origin`` and runs ``length`` along
    ``angle_deg``; node[i][j] is i steps along the arm and j steps across it."""
    a = math.radians(angle_deg)
    ux, uy = math.cos(a), math.sin(a)
    if angle_deg % 90.0 == 0.0:  # exact unit vectors for right angles
        ux, uy = float(round(ux)), float(round(uy))
    vx, vy = -uy, ux
    nodes = []
    for i in range(n_len + 1):
        r = r0 + length * i / n_len
        row = []
        for j in range(n_wid + 1):
            w = -width / 2 + width * j / n_wid
            row.append((origin[0] + r * ux + w * vx, origin[1] + r * uy + w * vy))
        nodes.append(row)
    return nodes


def kinked(*, seed: int = 0, arm_length: float = 2000.0, width: float = 200.0, n_len: int = 66, n_wid: int = 2,
           temps: Sequence[float] = (320.0, 280.0, 300.0), t_init: float = 300.0, t_eq: float = 300.0,
           spec_range: Tuple[float, float] = (0.0, 0.5), num_measurements: int = 5000, sim_time: float = 10.0,
           num_phonons: int = 1000000, sim_type: int = 1, step_interval: int = 50) -> dict:
    """Three arms meeting at a hub.  Arm A points west, arm B north (a 90 degree bend
    from A) and arm C south-east (a 45 degree bend from the line of A).  Each arm is
    ``n_len`` x ``n_wid`` quadrilateral cells with one sensor per quadrilateral; the hub
    is a triangle fan with four sensors.  The far end of each arm emits at ``temps``.
    Specularity is drawn per cell from U(spec_range) with ``seed`` (psim applies a
    cell's specularity to all three of its edges)."""
    rng = random.Random(seed)
    b = Builder(num_measurements=num_measurements, sim_time=sim_time, num_phonons=num_phonons, t_eq=t_eq,
                sim_type=sim_type, step_interval=step_interval)
    # The hub sits well away from the origin: psim's geometry tests a line for being vertical
    # with a tolerance relative to its x coordinates (psim/src/geometry.cpp:107-109) but takes
    # its slope with an absolute one (:325-327), so a vertical edge at |x| of order 1e-13 nm
    # would be intersected as if it were horizontal.
    centre = (3000.0, 3000.0)
    r0 = 150.0
    angles = (180.0, 90.0, -45.0)
    arms = [_arm_grid(centre, ang, arm_length, width, n_len, n_wid, r0) for ang in angles]
    for arm, temp in zip(arms, temps):
        for i in range(n_len):
            for j in range(n_wid):
                s = b.add_sensor(t_init)
                p1, p2, p3, p4 = arm[i][j], arm[i + 1][j], arm[i][j + 1], arm[i + 1][j + 1]
                b.add_quad(p1, p2, p3, p4, s, rng.uniform(*spec_range))
        for j in range(n_wid):
            b.add_surface(arm[n_len][j], arm[n_len][j + 1], temp)
    # Hub: fan from the centre over the inner end of each arm (split at its cross-nodes so
    # every hub edge is a full shared edge) and the wall gaps between arms.
    hub_arm_sensors = [b.add_sensor(t_init) for _ in arms]
    gap_sensor = b.add_sensor(t_init)
    ring: List[Tuple[Point, int]] = []
    order = sorted(range(len(arms)), key=lambda k: angles[k] % 360.0)
    for k in order:
        inner = arms[k][0]
        for j in range(n_wid):
            b.add_triangle(centre, inner[j], inner[j + 1], hub_arm_sensors[k], rng.uniform(*spec_range))
        ring.append((inner[n_wid], k))
    for idx, k in enumerate(order):
        nxt = order[(idx + 1) % len(order)]
        b.add_triangle(centre, arms[k][0][n_wid], arms[nxt][0][0], gap_sensor, rng.uniform(*spec_range))
    return b.to_dict()


def plate(*, length: float = 4000.0, width: float = 1000.0, nx: int = 64, ny: int = 16,
          strip: Tuple[float, float] = (400.0, 600.0), t_pulse: float = 400.0, pulse: float = 0.02,
          t_init: float = 300.0, t_eq: float = 300.0, spec: float = 0.0, num_measurements: int = 3000,
          sim_time: float = 3.0, num_phonons: int = 20000000, step_interval: int = 10) -> dict:
    """Transient plate: ``nx`` x ``ny`` rectangular cells, one sensor each, and a heat
    pulse of ``t_pulse`` on the part ``strip`` of the left edge for ``pulse`` ns.  The
    strip is split at cell boundaries so each piece lies on one cell edge."""
    b = Builder(num_measurements=num_measurements, sim_time=sim_time, num_phonons=num_phonons, t_eq=t_eq,
                sim_type=2, step_interval=step_interval)
    dx, dy = length / nx, width / ny
    for i in range(nx):
        for j in range(ny):
            s = b.add_sensor(t_init)
            b.add_rectangle((i * dx, j * dy), ((i + 1) * dx, (j + 1) * dy), s, spec)
    lo, hi = strip
    for j in range(ny):
        y0, y1 = max(lo, j * dy), min(hi, (j + 1) * dy)
        if y1 > y0:
            b.add_surface((0.0, y0), (0.0, y1), t_pulse, duration=pulse, start=0.0)
    return b.to_dict()


def random_bar_params(seed: int) -> Dict:
    """The batched workload's parameters drawn from ``seed``: length U(0.2, 5) um, width
    U(50, 500) nm, cells U{4..200}, phonons per step log-U(1e4, 1e6), end temperatures
    U(280, 320) K, wall specularity U(0, 1)."""
    rng = random.Random(seed)
    return {"length": rng.uniform(200.0, 5000.0), "width": rng.uniform(50.0, 500.0), "cells": rng.randint(4, 200),
            "per_step": 10 ** rng.uniform(4.0, 6.0), "t_left": rng.uniform(280.0, 320.0),
            "t_right": rng.uniform(280.0, 320.0), "spec": rng.uniform(0.0, 1.0)}


def random_bar(seed: int, *, dt_ps: float = 5.0, steps: int = 3000, pilot_lifetime_steps: float = 100.0,
               periodic: bool = False, per_step_scale: float = 1.0) -> Dict:
    """One model of the batched workload (``random_bar_params``).  The per-step population is
    turned into psim's total phonon budget with a pilot mean lifetime in steps.  Steady-state
    mode by default; ``periodic`` records every step (output every 50 steps) for measuring the
    time to steady state."""
    q = random_bar_params(seed)
    budget = int(q["per_step"] * per_step_scale * steps / pilot_lifetime_steps)
    return bar(num_cells=q["cells"], length=q["length"], width=q["width"], t_left=q["t_left"], t_right=q["t_right"],
               t_init=300.0, t_eq=300.0, spec=q["spec"], num_measurements=steps, sim_time=steps * dt_ps * 1e-3,
               num_phonons=max(budget, 1000), sim_type=1 if periodic else 0, step_interval=50 if periodic else 0)
