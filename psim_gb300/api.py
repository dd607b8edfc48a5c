"""Python front end of the psim_gb300 C ABI (include/psim_gb300.h) through ctypes.

``Model`` mirrors what psim's CLI does with one input file (InputManager::deserialize,
Model::runSimulation, Model::exportResults: psim/src/main.cpp:10-31); ``Simulator``
mirrors ModelSimulator (psim/include/psim/modelSimulator.h:12-41); ``interpret`` and
``final_temps`` mirror SensorInterpreter; the ``geom_*`` functions run psim's FP64
geometry routines on the GPU.

The library must have been built (``psim_gb300.build.build()``); loading fails with an
error otherwise.  There is no CPU fallback: GPU entry points fail on a machine without
a CUDA device.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Tuple

import numpy as np

from . import build as _build

PSIM_OK = 0
PSIM_ERR_INVALID = 1
PSIM_ERR_CUDA = 2
PSIM_ERR_IO = 3
PSIM_ERR_LIMIT = 4
FP32 = 0
FP64 = 1
NUM_FREQ_BINS = 1000

_c_dp = ctypes.POINTER(ctypes.c_double)
_c_u32p = ctypes.POINTER(ctypes.c_uint32)
_c_i32p = ctypes.POINTER(ctypes.c_int32)
_c_i64p = ctypes.POINTER(ctypes.c_int64)
_c_u64p = ctypes.POINTER(ctypes.c_uint64)
_c_fp = ctypes.POINTER(ctypes.c_float)


class PsimError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"psim error {code}: {message}")
        self.code = code


class RunCounters(ctypes.Structure):
    _fields_ = [("phonons", ctypes.c_uint64), ("phonon_steps", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("eff_energy", ctypes.c_double), ("seconds", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("max_population", ctypes.c_uint64), ("limit_hits", ctypes.c_uint64),
                ("event_limit_hits", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("transport_launches", ctypes.c_uint64), ("steps_per_launch", ctypes.c_uint64),
                ("backscatters", ctypes.c_uint64), ("state_bytes", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class SimDesc(ctypes.Structure):
    _fields_ = [
        ("measurement_steps", ctypes.c_uint64), ("simulation_time", ctypes.c_double), ("phasor_sim", ctypes.c_int32),
        ("sim_type", ctypes.c_int32), ("step_adjustment", ctypes.c_uint64), ("recorded_steps", ctypes.c_uint64),
        ("full_simulation", ctypes.c_int32),
        ("n_materials", ctypes.c_uint32), ("mat_freq", _c_dp), ("mat_vel", _c_dp), ("mat_params", _c_dp),
        ("n_tables", ctypes.c_uint32), ("tables", _c_dp),
        ("n_sensors", ctypes.c_uint32), ("sensor_material", _c_u32p), ("sensor_temp", _c_dp),
        ("sensor_base_table", _c_u32p), ("sensor_scatter_table", _c_u32p),
        ("n_cells", ctypes.c_uint32), ("cell_vertices", _c_dp), ("cell_sensor", _c_u32p), ("cell_spec", _c_dp),
        ("edge_sub_begin", _c_u32p), ("n_subs", ctypes.c_uint32), ("sub_kind", _c_i32p), ("sub_target", _c_u32p),
        ("sub_line", _c_dp),
        ("n_emitters", ctypes.c_uint32), ("emit_cell", _c_u32p), ("emit_edge", _c_u32p), ("emit_line", _c_dp),
        ("emit_temp", _c_dp), ("emit_start", _c_dp), ("emit_duration", _c_dp), ("emit_table", _c_u32p),
    ]


class InterpDesc(ctypes.Structure):
    _fields_ = [
        ("n_sensors", ctypes.c_uint32), ("recorded_steps", ctypes.c_uint64), ("t_eq", ctypes.c_double),
        ("eff_energy", ctypes.c_double), ("lower_bound", ctypes.c_double), ("upper_bound", ctypes.c_double),
        ("sensor_area", _c_dp), ("sensor_heat_capacity", _c_dp), ("sensor_init_temp", _c_dp),
        ("sensor_material", _c_u32p), ("n_materials", ctypes.c_uint32), ("mat_temp_begin", _c_u64p),
        ("temps", _c_dp), ("energies", _c_dp),
    ]


class BatchOptions(ctypes.Structure):
    _fields_ = [("workers", ctypes.c_int32), ("max_blocks", ctypes.c_int32), ("device_queue", ctypes.c_int32),
                ("per_thread", ctypes.c_int32)]


# Every symbol the C header declares, with (restype, argtypes).
SIGNATURES = {
    "psim_last_error": (ctypes.c_char_p, []),
    "psim_version": (ctypes.c_char_p, []),
    "psim_device_count": (ctypes.c_int, []),
    "psim_model_load_json": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "psim_model_set_options": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p]),
    "psim_model_run": (ctypes.c_int, [ctypes.c_void_p]),
    "psim_model_shape": (ctypes.c_int, [ctypes.c_void_p, _c_i64p, _c_i64p, _c_i64p, _c_i64p, _c_i64p]),
    "psim_model_measurements": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "psim_model_set_measurements": (ctypes.c_int, [ctypes.c_void_p, _c_dp, ctypes.c_int64]),
    "psim_model_series": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_dp, _c_dp]),
    "psim_model_tallies": (ctypes.c_int, [ctypes.c_void_p, _c_i64p, _c_dp]),
    "psim_model_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RunCounters)]),
    "psim_model_population": (ctypes.c_int, [ctypes.c_void_p, _c_u32p]),
    "psim_sim_population": (ctypes.c_int, [ctypes.c_void_p, _c_u32p]),
    "psim_model_sim_desc": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SimDesc)]),
    "psim_model_interp_desc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(InterpDesc)]),
    "psim_model_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double]),
    "psim_model_destroy": (None, [ctypes.c_void_p]),
    "psim_sim_create": (ctypes.c_int, [ctypes.POINTER(SimDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "psim_sim_init_phonon_builders": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _c_dp, _c_dp,
                                                     _c_dp, ctypes.c_uint64, _c_u64p]),
    "psim_sim_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p]),
    "psim_sim_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "psim_sim_set_step_adjustment": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "psim_sim_tallies": (ctypes.c_int, [ctypes.c_void_p, _c_i64p, _c_dp]),
    "psim_sim_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RunCounters)]),
    "psim_sim_destroy": (None, [ctypes.c_void_p]),
    "psim_interpret": (ctypes.c_int, [ctypes.POINTER(InterpDesc), _c_i64p, _c_dp, _c_dp, _c_dp, _c_dp]),
    "psim_final_temps": (ctypes.c_int, [ctypes.POINTER(InterpDesc), _c_i64p, ctypes.c_uint64, _c_dp]),
    "psim_final_temps_noalloc": (ctypes.c_int, [ctypes.POINTER(InterpDesc), ctypes.c_void_p, ctypes.c_uint64,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "psim_final_temps_noalloc_max_bytes": (ctypes.c_uint64, []),
    "psim_steady_state": (ctypes.c_int, [_c_i64p, _c_dp, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_double, ctypes.c_uint32, ctypes.c_double, _c_i64p, _c_i64p]),
    "psim_sim_steady_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_uint32,
                                             ctypes.c_double, _c_i64p, _c_i64p]),
    "psim_model_steady_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                               ctypes.c_uint32, ctypes.c_double, _c_i64p, _c_i64p]),
    "psim_model_set_steady_stop": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
                                                  ctypes.c_double, ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64]),
    "psim_sim_set_steady_stop": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
                                                ctypes.c_double, ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64]),
    "psim_model_steps_run": (ctypes.c_int, [ctypes.c_void_p, _c_u64p]),
    "psim_sim_steps_run": (ctypes.c_int, [ctypes.c_void_p, _c_u64p]),
    "psim_batch_run": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.POINTER(BatchOptions),
                                      _c_dp, _c_u64p]),
    "psim_batch_autotune": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.c_int32,
                                           ctypes.POINTER(BatchOptions), _c_dp]),
    "psim_model_start_temps": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "psim_model_set_start_temps": (ctypes.c_int, [ctypes.c_void_p, _c_dp]),
    "psim_mlp_create": (ctypes.c_int, [_c_i32p, ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    "psim_mlp_n_params": (ctypes.c_int, [ctypes.c_void_p, _c_u64p]),
    "psim_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, _c_fp]),
    "psim_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, _c_fp]),
    "psim_mlp_gradients": (ctypes.c_int, [ctypes.c_void_p, _c_fp, _c_fp, ctypes.c_int32, _c_fp, _c_fp]),
    "psim_mlp_train": (ctypes.c_int, [ctypes.c_void_p, _c_fp, _c_fp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_float, ctypes.c_uint64, _c_fp]),
    "psim_mlp_predict": (ctypes.c_int, [ctypes.c_void_p, _c_fp, ctypes.c_int32, _c_fp]),
    "psim_mlp_destroy": (None, [ctypes.c_void_p]),
    "psim_geom_intersect": (ctypes.c_int, [ctypes.c_int64, _c_dp, _c_dp, _c_dp, _c_i32p]),
    "psim_rates": (ctypes.c_int, [_c_dp, ctypes.c_int64, _c_dp, _c_dp, _c_i32p, ctypes.c_int, _c_dp]),
    "psim_geom_on_line": (ctypes.c_int, [ctypes.c_int64, _c_dp, _c_dp, _c_i32p]),
    "psim_geom_tri_contains": (ctypes.c_int, [ctypes.c_int64, _c_dp, _c_dp, _c_i32p]),
    "psim_geom_edge_index": (ctypes.c_int, [ctypes.c_int64, _c_dp, _c_dp, _c_i32p]),
    "psim_sampling_alias_table": (ctypes.c_int, [_c_dp, _c_u32p]),
}

_lib: Optional[ctypes.CDLL] = None


def lib_path() -> str:
    return _build.LIB


def lib() -> ctypes.CDLL:
    """Load libpsim_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: call psim_gb300.build.build() first")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != PSIM_OK:
        raise PsimError(rc, lib().psim_last_error().decode(errors="replace"))


def device_count() -> int:
    return int(lib().psim_device_count())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_c_dp)


def _i32(a: np.ndarray):
    return a.ctypes.data_as(_c_i32p)


def _i64(a: np.ndarray):
    return a.ctypes.data_as(_c_i64p)


class Model:
    """One psim input file on the GPU."""

    def __init__(self, json_path: str):
        self._h = ctypes.c_void_p()
        _check(lib().psim_model_load_json(json_path.encode(), ctypes.byref(self._h)))
        self.path = json_path
        self._shape()

    def _shape(self) -> None:
        s, k, c, n, r = (ctypes.c_int64() for _ in range(5))
        _check(lib().psim_model_shape(self._h, ctypes.byref(s), ctypes.byref(k), ctypes.byref(c), ctypes.byref(n),
                                      ctypes.byref(r)))
        self.n_sensors, self.n_recorded, self.n_cells, self.n_steps, self.n_runs = (
            s.value, k.value, c.value, n.value, r.value)

    def close(self) -> None:
        if self._h:
            lib().psim_model_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_options(self, seed: int = 1, precision: int = FP32, stream: Optional[int] = None) -> "Model":
        """Seed, precision and stream of later runs (psim_model_set_options)."""
        _check(lib().psim_model_set_options(self._h, seed, precision, ctypes.c_void_p(stream or 0)))
        return self

    def run(self, seed: int = 1, precision: int = FP32, stream: Optional[int] = None) -> "Model":
        _check(lib().psim_model_set_options(self._h, seed, precision, ctypes.c_void_p(stream or 0)))
        _check(lib().psim_model_run(self._h))
        self._shape()  # a run stopped at steady state records fewer steps
        return self

    def set_steady_stop(self, window: int = 250, batches: int = 5, z: float = 3.0, patience: int = 3, check_every: int = 0,
                        drift_z: float = 0.0,
                        enable: bool = True) -> None:
        """Stop later runs at steady state (single-run periodic or transient models)."""
        _check(lib().psim_model_set_steady_stop(self._h, 1 if enable else 0, window, batches, z, patience, drift_z, check_every))

    def steps_run(self) -> int:
        out = ctypes.c_uint64()
        _check(lib().psim_model_steps_run(self._h, ctypes.byref(out)))
        return int(out.value)

    def start_temps(self) -> np.ndarray:
        """The temperature each sensor starts runs from (file order)."""
        out = np.zeros(self.n_sensors)
        _check(lib().psim_model_start_temps(self._h, _dp(out)))
        return out

    def set_start_temps(self, temps: Optional[np.ndarray]) -> None:
        """Warm start: later runs start from these sensor temperatures (None: the file's)."""
        if temps is None:
            _check(lib().psim_model_set_start_temps(self._h, None))
            return
        t = np.ascontiguousarray(temps, dtype=np.float64)
        assert t.shape == (self.n_sensors,)
        _check(lib().psim_model_set_start_temps(self._h, _dp(t)))

    def measurements(self) -> np.ndarray:
        """[S, 6]: T, SE(T), flux x, SE, flux y, SE averaged over runs."""
        out = np.zeros((self.n_sensors, 6))
        _check(lib().psim_model_measurements(self._h, _dp(out)))
        return out

    def set_measurements(self, stats: np.ndarray) -> "Model":
        """Replaces the per-run results with stats[runs, S, 6] made elsewhere (psim_model_set_measurements)."""
        s = np.ascontiguousarray(stats, dtype=np.float64)
        if s.ndim != 3 or s.shape[1:] != (self.n_sensors, 6):
            raise ValueError(f"stats must be [runs, {self.n_sensors}, 6]")
        _check(lib().psim_model_set_measurements(self._h, _dp(s), s.shape[0]))
        return self

    def series(self, run: int = 0) -> Tuple[np.ndarray, np.ndarray]:
        temps = np.zeros((self.n_sensors, self.n_recorded))
        fluxes = np.zeros((self.n_sensors, self.n_recorded, 2))
        _check(lib().psim_model_series(self._h, run, _dp(temps), _dp(fluxes)))
        return temps, fluxes

    def tallies(self) -> Tuple[np.ndarray, np.ndarray]:
        energy = np.zeros((self.n_sensors, self.n_recorded), dtype=np.int64)
        flux = np.zeros((self.n_sensors, self.n_recorded, 2))
        _check(lib().psim_model_tallies(self._h, _i64(energy), _dp(flux)))
        return energy, flux

    def counters(self) -> dict:
        c = RunCounters()
        _check(lib().psim_model_counters(self._h, ctypes.byref(c)))
        return c.as_dict()

    def population(self) -> np.ndarray:
        """Phonons in flight at each measurement step of the last run."""
        out = np.zeros(self.n_steps, dtype=np.uint32)
        _check(lib().psim_model_population(self._h, out.ctypes.data_as(_c_u32p)))
        return out

    def export(self, json_path: Optional[str] = None, seconds: float = 0.0) -> None:
        _check(lib().psim_model_export(self._h, (json_path or self.path).encode(), seconds))

    def sim_desc(self) -> SimDesc:
        d = SimDesc()
        _check(lib().psim_model_sim_desc(self._h, ctypes.byref(d)))
        return d

    def steady_state(self, window: int = 250, batches: int = 5, z: float = 3.0, patience: int = 3,
                     drift_z: float = 0.0) -> Tuple[int, np.ndarray]:
        """Steady-state onset (step, -1 if none) and per-sensor onsets over the last run."""
        return _steady(lib().psim_model_steady_state, self._h, self.n_sensors, window, batches, z, patience, drift_z)

    def interp_desc(self, eff_energy: float = 0.0) -> InterpDesc:
        d = InterpDesc()
        _check(lib().psim_model_interp_desc(self._h, eff_energy, ctypes.byref(d)))
        return d

    def tables(self) -> np.ndarray:
        """[n_tables, 1000, 2] cumulative tables (probability, LA fraction) the model uses."""
        d = self.sim_desc()
        return np.ctypeslib.as_array(d.tables, shape=(d.n_tables, NUM_FREQ_BINS, 2)).copy()


class Simulator:
    """ModelSimulator seam: a flattened model description (SimDesc) on the GPU."""

    def __init__(self, desc: SimDesc):
        self._h = ctypes.c_void_p()
        self.desc = desc
        _check(lib().psim_sim_create(ctypes.byref(desc), ctypes.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().psim_sim_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_phonon_builders(self, t_eq: float, eff_energy: float, cell_energy: np.ndarray, emit_energy: np.ndarray,
                             sensor_init_temp: np.ndarray, seed: int) -> int:
        cell_energy = np.ascontiguousarray(cell_energy, dtype=np.float64)
        emit_energy = np.ascontiguousarray(emit_energy, dtype=np.float64)
        sensor_init_temp = np.ascontiguousarray(sensor_init_temp, dtype=np.float64)
        total = ctypes.c_uint64()
        _check(lib().psim_sim_init_phonon_builders(self._h, t_eq, eff_energy, _dp(cell_energy), _dp(emit_energy),
                                                   _dp(sensor_init_temp), seed, ctypes.byref(total)))
        return total.value

    def run(self, t_eq: float, precision: int = FP32, stream: Optional[int] = None) -> None:
        _check(lib().psim_sim_run(self._h, t_eq, precision, ctypes.c_void_p(stream or 0)))

    def reset(self) -> None:
        _check(lib().psim_sim_reset(self._h))

    def set_step_adjustment(self, adj: int) -> None:
        _check(lib().psim_sim_set_step_adjustment(self._h, adj))

    def tallies(self) -> Tuple[np.ndarray, np.ndarray]:
        S, K = self.desc.n_sensors, self.desc.recorded_steps
        energy = np.zeros((S, K), dtype=np.int64)
        flux = np.zeros((S, K, 2))
        _check(lib().psim_sim_tallies(self._h, _i64(energy), _dp(flux)))
        return energy, flux

    def steady_state(self, window: int = 250, batches: int = 5, z: float = 3.0, patience: int = 3,
                     drift_z: float = 0.0) -> Tuple[int, np.ndarray]:
        return _steady(lib().psim_sim_steady_state, self._h, self.desc.n_sensors, window, batches, z, patience, drift_z)

    def set_steady_stop(self, window: int = 250, batches: int = 5, z: float = 3.0, patience: int = 3, check_every: int = 0,
                        drift_z: float = 0.0,
                        enable: bool = True) -> None:
        _check(lib().psim_sim_set_steady_stop(self._h, 1 if enable else 0, window, batches, z, patience, drift_z, check_every))

    def steps_run(self) -> int:
        out = ctypes.c_uint64()
        _check(lib().psim_sim_steps_run(self._h, ctypes.byref(out)))
        return int(out.value)

    def counters(self) -> dict:
        c = RunCounters()
        _check(lib().psim_sim_counters(self._h, ctypes.byref(c)))
        return c.as_dict()

    def population(self) -> np.ndarray:
        out = np.zeros(self.desc.measurement_steps, dtype=np.uint32)
        _check(lib().psim_sim_population(self._h, out.ctypes.data_as(_c_u32p)))
        return out


def interpret(desc: InterpDesc, energy: np.ndarray, flux: np.ndarray):
    """scaleHeatParams for every sensor: (temps [S,K], fluxes [S,K,2], stats [S,6])."""
    S, K = desc.n_sensors, desc.recorded_steps
    energy = np.ascontiguousarray(energy, dtype=np.int64)
    flux = np.ascontiguousarray(flux, dtype=np.float64)
    temps = np.zeros((S, K))
    fluxes = np.zeros((S, K, 2))
    stats = np.zeros((S, 6))
    _check(lib().psim_interpret(ctypes.byref(desc), _i64(energy), _dp(flux), _dp(temps), _dp(fluxes), _dp(stats)))
    return temps, fluxes, stats


def _f32(a: np.ndarray):
    return a.ctypes.data_as(_c_fp)


class Mlp:
    """The warm-start surrogate's network on the GPU (psim_mlp_*): BF16 parameters and
    activations, FP32 accumulation, GELU hidden layers, Adam."""

    def __init__(self, widths, seed: int = 1):
        w = np.ascontiguousarray(widths, dtype=np.int32)
        self.widths = [int(v) for v in w]
        self._h = ctypes.c_void_p()
        _check(lib().psim_mlp_create(w.ctypes.data_as(_c_i32p), len(w), seed, ctypes.byref(self._h)))
        n = ctypes.c_uint64()
        _check(lib().psim_mlp_n_params(self._h, ctypes.byref(n)))
        self.n_params = int(n.value)

    def close(self) -> None:
        if self._h:
            lib().psim_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        _check(lib().psim_mlp_get_params(self._h, _f32(out)))
        return out

    @params.setter
    def params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (self.n_params,)
        _check(lib().psim_mlp_set_params(self._h, _f32(p)))

    def gradients(self, x: np.ndarray, y: np.ndarray) -> Tuple[float, np.ndarray]:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = ctypes.c_float()
        g = np.zeros(self.n_params, dtype=np.float32)
        _check(lib().psim_mlp_gradients(self._h, _f32(x), _f32(y), len(x), ctypes.byref(loss), _f32(g)))
        return float(loss.value), g

    def train(self, x: np.ndarray, y: np.ndarray, batch: int = 256, epochs: int = 200, lr: float = 1e-3,
              seed: int = 1) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = ctypes.c_float()
        _check(lib().psim_mlp_train(self._h, _f32(x), _f32(y), len(x), batch, epochs, lr, seed, ctypes.byref(loss)))
        return float(loss.value)

    def predict(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros((len(x), self.widths[-1]), dtype=np.float32)
        _check(lib().psim_mlp_predict(self._h, _f32(x), len(x), _f32(y)))
        return y


def _handles(models):
    arr = (ctypes.c_void_p * max(1, len(models)))()
    for i, m in enumerate(models):
        arr[i] = m._h
    return arr


def batch_run(models, workers: int = 8, max_blocks: int = 0, device_queue: bool = True,
              per_thread: int = 16) -> Tuple[float, int]:
    """Runs every Model once, together (psim_batch_run): (wall seconds, phonon-steps).  With
    device_queue the FP32 models share batched launches fed by a device work queue."""
    opt = BatchOptions(workers, max_blocks, 1 if device_queue else 0, per_thread)
    secs = ctypes.c_double()
    steps = ctypes.c_uint64()
    _check(lib().psim_batch_run(_handles(models), len(models), ctypes.byref(opt), ctypes.byref(secs),
                                ctypes.byref(steps)))
    for m in models:
        m._shape()
    return float(secs.value), int(steps.value)


def batch_autotune(models, sample: int = 16) -> Tuple[BatchOptions, float]:
    """The batch autotuner (psim_batch_autotune): the fastest options and their phonon-steps/s."""
    opt = BatchOptions()
    rate = ctypes.c_double()
    _check(lib().psim_batch_autotune(_handles(models), len(models), sample, ctypes.byref(opt), ctypes.byref(rate)))
    for m in models[:sample]:
        m._shape()
    return opt, float(rate.value)


def _steady(fn, handle, n_sensors: int, window: int, batches: int, z: float, patience: int,
            drift_z: float = 0.0) -> Tuple[int, np.ndarray]:
    onset = ctypes.c_int64()
    per = np.zeros(n_sensors, dtype=np.int64)
    _check(fn(handle, window, batches, z, patience, drift_z, ctypes.byref(onset), _i64(per)))
    return int(onset.value), per


def steady_state(energy: np.ndarray, flux: np.ndarray, window: int = 250, batches: int = 5, z: float = 3.0,
                 patience: int = 3, drift_z: float = 0.0) -> Tuple[int, np.ndarray]:
    """psim_steady_state on raw tallies energy [S,K] and flux [S,K,2]: (onset step or -1, per-sensor onsets)."""
    energy = np.ascontiguousarray(energy, dtype=np.int64)
    flux = np.ascontiguousarray(flux, dtype=np.float64)
    S, K = energy.shape
    assert flux.shape == (S, K, 2)
    onset = ctypes.c_int64()
    per = np.zeros(S, dtype=np.int64)
    _check(lib().psim_steady_state(_i64(energy), _dp(flux), S, K, window, batches, z, patience, drift_z, ctypes.byref(onset),
                                   _i64(per)))
    return int(onset.value), per


def final_temps(desc: InterpDesc, energy: np.ndarray, start_step: int) -> np.ndarray:
    energy = np.ascontiguousarray(energy, dtype=np.int64)
    out = np.zeros(desc.n_sensors)
    _check(lib().psim_final_temps(ctypes.byref(desc), _i64(energy), start_step, _dp(out)))
    return out


def final_temps_noalloc(desc: InterpDesc, energy_dev: int, start_step: int, out_dev: int,
                        stream: Optional[int] = None) -> None:
    """psim_final_temps_noalloc: device addresses in (int64 [S][K]) and out (float64 [S]),
    enqueued on ``stream`` (a cudaStream_t as an int) without waiting for it."""
    _check(lib().psim_final_temps_noalloc(ctypes.byref(desc), ctypes.c_void_p(energy_dev), start_step,
                                          ctypes.c_void_p(out_dev), ctypes.c_void_p(stream)))


def final_temps_noalloc_max_bytes() -> int:
    return int(lib().psim_final_temps_noalloc_max_bytes())


def rates(mat_params, T, freq, pol, precision=FP64) -> np.ndarray:
    """Material::relaxRates as the FP32 or FP64 transport kernel evaluates it on the GPU:
    [n, 3] normal, Umklapp and impurity rates (1/s) for the cases (T K, freq rad/s, pol 0/1)."""
    mp = np.ascontiguousarray(mat_params, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    f = np.ascontiguousarray(freq, dtype=np.float64)
    p = np.ascontiguousarray(pol, dtype=np.int32)
    n = T.shape[0]
    if mp.shape != (8,) or f.shape != (n,) or p.shape != (n,):
        raise ValueError("mat_params needs 8 values and T, freq, pol one value per case")
    out = np.zeros((n, 3))
    _check(lib().psim_rates(_dp(mp), n, _dp(T), _dp(f), _i32(p), int(precision), _dp(out)))
    return out


def geom_intersect(a: np.ndarray, b: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = a.shape[0]
    poi = np.zeros((n, 2))
    has = np.zeros(n, dtype=np.int32)
    _check(lib().psim_geom_intersect(n, _dp(a), _dp(b), _dp(poi), _i32(has)))
    return has, poi


def geom_on_line(lines: np.ndarray, pts: np.ndarray) -> np.ndarray:
    lines = np.ascontiguousarray(lines, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(lines.shape[0], dtype=np.int32)
    _check(lib().psim_geom_on_line(lines.shape[0], _dp(lines), _dp(pts), _i32(out)))
    return out


def geom_tri_contains(tris: np.ndarray, pts: np.ndarray) -> np.ndarray:
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(tris.shape[0], dtype=np.int32)
    _check(lib().psim_geom_tri_contains(tris.shape[0], _dp(tris), _dp(pts), _i32(out)))
    return out


def geom_edge_index(tris: np.ndarray, pts: np.ndarray) -> np.ndarray:
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(tris.shape[0], dtype=np.int32)
    _check(lib().psim_geom_edge_index(tris.shape[0], _dp(tris), _dp(pts), _i32(out)))
    return out


def alias_table(table: np.ndarray) -> np.ndarray:
    """psim_sampling_alias_table: the alias table (uint32[2048]) the kernels sample (bin,
    polarization) from, for one cumulative table [1000][2] = (cumulative probability, LA fraction)."""
    table = np.ascontiguousarray(table, dtype=np.float64)
    if table.shape != (1000, 2):
        raise ValueError("a cumulative table is [1000][2]")
    out = np.zeros(2048, dtype=np.uint32)
    _check(lib().psim_sampling_alias_table(_dp(table), out.ctypes.data_as(_c_u32p)))
    return out
