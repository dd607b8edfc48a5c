"""ctypes front end of the CPU oracle (oracle/psim_oracle.cpp).

Test infrastructure only: the tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use it as the test oracle.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_lib: Optional[ctypes.CDLL] = None


def build(quiet: bool = True) -> None:
    """Compile the oracle (a few seconds, g++ only)."""
    out = subprocess.run(["make", "-j4", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def build_reference(reference_root: str) -> bool:
    """Compile the reference sources into oracle/_ref when they are present (this
    container only; the reference tree is not available everywhere)."""
    if not os.path.isdir(os.path.join(reference_root, "psim", "src")):
        return False
    out = subprocess.run(["make", "-j8", "-C", os.path.join(HERE, "ref_recipe"), f"REF={reference_root}"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + out.stdout + out.stderr)
    return True


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_run.argtypes = [ctypes.c_char_p, ctypes.c_uint, ctypes.c_int, ip, ip, dp,
                                 ctypes.POINTER(ctypes.c_longlong), dp, ctypes.POINTER(ctypes.c_ulonglong), dp]
        L.oracle_run.restype = ctypes.c_int
        L.oracle_shape.argtypes = [ctypes.c_char_p, ip, ip, ip]
        L.oracle_shape.restype = ctypes.c_int
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_intersect.argtypes = [ctypes.c_int, dp, dp, dp, ip]
        L.oracle_on_line.argtypes = [ctypes.c_int, dp, dp, ip]
        L.oracle_tri_contains.argtypes = [ctypes.c_int, dp, dp, ip]
        L.oracle_tables.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.oracle_tables.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


@dataclass
class OracleResult:
    stats: np.ndarray        # [S, 6]: T, SE(T), fx, SE(fx), fy, SE(fy) averaged over runs
    energy: np.ndarray       # [S, K] int64 raw tallies of the last run
    flux: np.ndarray         # [S, K, 2] raw flux tallies (sum of sign * v)
    total_phonons: int
    phonons_simulated: int
    phonon_steps: int
    eff_energy: float
    seconds: float


def shape(path: str):
    L = lib()
    s, k, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    if L.oracle_shape(path.encode(), ctypes.byref(s), ctypes.byref(k), ctypes.byref(c)) != 0:
        raise RuntimeError(L.oracle_last_error().decode())
    return s.value, k.value, c.value


def run(path: str, seed: int, threads: int = 1) -> OracleResult:
    L = lib()
    S, K, _ = shape(path)
    stats = np.zeros((S, 6))
    energy = np.zeros((S, K), dtype=np.int64)
    flux = np.zeros((S, K, 2))
    counters = (ctypes.c_ulonglong * 4)()
    secs = ctypes.c_double()
    s, k = ctypes.c_int(), ctypes.c_int()
    rc = L.oracle_run(path.encode(), seed, threads, ctypes.byref(s), ctypes.byref(k), _dp(stats),
                      energy.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), _dp(flux), counters,
                      ctypes.byref(secs))
    if rc != 0:
        raise RuntimeError("oracle: " + L.oracle_last_error().decode())
    eff = struct.unpack("<d", struct.pack("<Q", counters[3]))[0]
    return OracleResult(stats, energy, flux, int(counters[0]), int(counters[1]), int(counters[2]), eff, secs.value)


def intersect(a: np.ndarray, b: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = a.shape[0]
    poi = np.zeros((n, 2))
    has = np.zeros(n, dtype=np.int32)
    lib().oracle_intersect(n, _dp(a), _dp(b), _dp(poi), _ip(has))
    return has, poi


def on_line(lines: np.ndarray, pts: np.ndarray) -> np.ndarray:
    lines = np.ascontiguousarray(lines, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(lines.shape[0], dtype=np.int32)
    lib().oracle_on_line(lines.shape[0], _dp(lines), _dp(pts), _ip(out))
    return out


def tri_contains(tris: np.ndarray, pts: np.ndarray) -> np.ndarray:
    tris = np.ascontiguousarray(tris, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(tris.shape[0], dtype=np.int32)
    lib().oracle_tri_contains(tris.shape[0], _dp(tris), _dp(pts), _ip(out))
    return out


def tables(path: str, out_path: str) -> None:
    if lib().oracle_tables(path.encode(), out_path.encode()) != 0:
        raise RuntimeError(lib().oracle_last_error().decode())
