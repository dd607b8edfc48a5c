"""Builds libpsim_gb300.so (CUDA kernels for sm_103a + the C++17 host library + the C ABI)
and the psim_gb300 command-line tool into psim_gb300/_lib/.

Translation units compile in parallel; a unit is rebuilt when it or any file it may include
is newer than its object file.  Device units that carry FP64 geometry or the FP64
interpreter compile with -fmad=false and host code with -ffp-contract=off, so those results
round exactly as the reference's do.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libpsim_gb300.so")
CLI = os.path.join(OUT, "psim_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
CXX_COMMON = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include")]

# units whose results must round like the reference's host arithmetic
FMAD_OFF = {"step_f64.cu", "interpret.cu"}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "device", "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "host", "*.cpp"))) + [os.path.join(CSRC, "capi.cpp")]
    return cu, cpp


def _headers():
    hs = glob.glob(os.path.join(CSRC, "**", "*.hpp"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


def _run(cmd, verbose: bool):
    if verbose:
        print(" ".join(cmd), flush=True)
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + out.stdout + out.stderr)
    return out.stdout + out.stderr


def build(verbose: bool = False, jobs: int = 0) -> str:
    """Compile every unit (in parallel) and link the shared library and the CLI; returns the
    library path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = _sources()
    headers = _headers()
    jobs = jobs or min(8, os.cpu_count() or 4)
    cmds = []
    objs = []
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        flags = list(NVCC_COMMON) + ARCH
        if os.path.basename(src) in FMAD_OFF:
            flags.append("-fmad=false")
        if _stale(obj, src, headers):
            cmds.append([nvcc] + flags + ["-c", src, "-o", obj])
    cxx = os.environ.get("CXX", "g++")
    for src in cpp:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            cmds.append([cxx] + CXX_COMMON + ["-I", _cuda_include(), "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs) as pool:
        list(pool.map(lambda c: _run(c, verbose), cmds))
    if cmds or not os.path.exists(LIB):
        _run([nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC"], verbose)
    cli_src = os.path.join(CSRC, "cli", "main.cpp")
    if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(LIB), os.path.getmtime(cli_src)):
        _run([cxx] + CXX_COMMON + [cli_src, "-o", CLI, "-L", OUT, "-lpsim_gb300", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
