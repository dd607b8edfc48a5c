"""The host library under AddressSanitizer and UndefinedBehaviorSanitizer, without a GPU.

libpsim_gb300.so is rebuilt from the same sources with -fsanitize=address,undefined (UBSan
set to stop at the first report) into a temporary directory.  A child Python process with
the sanitizer runtimes preloaded then drives the host side through the C ABI:
- every model file of the fixtures, the reference's demos included: loading, model assembly,
  material tables, the flattened and interpreter descriptions;
- a seeded fuzz of the JSON loader: truncated and byte-mutated files, and well-formed files
  with extreme numbers (negative, zero, huge, denormal) in their settings, sensors,
  materials and emitting surfaces.
Every input must load or be refused with a status code; any sanitizer report fails the test."""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import pytest

from conftest import GOLDEN, ROOT

CHILD = r'''
import copy, glob, gzip, json, os, random, sys, tempfile
sys.path.insert(0, ROOT)
import psim_gb300.build as B
B.LIB = LIB
B.build = lambda *a, **k: LIB
from psim_gb300 import api

td = tempfile.mkdtemp()
models = {}
for p in sorted(glob.glob(os.path.join(GOLDEN, "models", "*.json*"))):
    raw = gzip.open(p, "rb").read() if p.endswith(".gz") else open(p, "rb").read()
    q = os.path.join(td, os.path.basename(p).replace(".gz", ""))
    open(q, "wb").write(raw)
    m = api.Model(q)
    m.sim_desc(); m.interp_desc()
    m.close()
    models[os.path.basename(q)] = raw

rng = random.Random(5)
small = [models[n] for n in ("bar_ss.json", "plate_small.json", "kinked_small.json")]
p = os.path.join(td, "fuzz.json")

def attempt(data):
    open(p, "wb").write(data)
    try:
        m = api.Model(p)
        m.sim_desc(); m.interp_desc()
        m.close()
        return True
    except api.PsimError:
        return False

alphabet = b'{}[]:,"0123456789.-+eE \\ntrufalsn'
for i in range(600):
    b = bytearray(rng.choice(small))
    k = i % 3
    if k == 0:
        b = b[:rng.randrange(len(b))]
    elif k == 1:
        for _ in range(rng.randrange(1, 8)):
            b[rng.randrange(len(b))] = rng.choice(alphabet)
    else:
        j = rng.randrange(len(b))
        del b[j:j + rng.randrange(1, 40)]
    attempt(bytes(b))

VALUES = [-1, 0, 1, -1e308, 1e308, 1e-320, 2 ** 63, 2 ** 64 + 5, -(2 ** 63), 3.5, 1e12, 4294967296, -0.0, 1e6, 7]
bases = [json.loads(x) for x in small]

def leaves(o, path=()):
    if isinstance(o, dict):
        for key, v in o.items():
            yield from leaves(v, path + (key,))
    elif isinstance(o, list):
        for n, v in enumerate(o):
            yield from leaves(v, path + (n,))
    elif isinstance(o, (int, float)) and not isinstance(o, bool):
        yield path

loaded = 0
for i in range(400):
    m = copy.deepcopy(rng.choice(bases))
    ls = [q for q in leaves(m) if q[0] in ("settings", "sensors", "materials", "emit_surfaces")]
    for _ in range(rng.randrange(1, 4)):
        o = m
        path = rng.choice(ls)
        for key in path[:-1]:
            o = o[key]
        o[path[-1]] = rng.choice(VALUES)
    loaded += attempt(json.dumps(m).encode())
print("sanitized run ok", len(models), "models,", loaded, "of 400 value-fuzzed files loaded")
'''


def runtime(name):
    try:
        p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return p if os.path.isabs(p) and os.path.exists(p) else None


@pytest.fixture(scope="module")
def sanitized_lib(tmp_path_factory):
    asan, ubsan = runtime("libasan.so"), runtime("libubsan.so")
    if asan is None or ubsan is None or shutil.which("g++") is None:
        pytest.skip("the gcc sanitizer runtimes are not installed")
    from psim_gb300 import build as B
    out = str(tmp_path_factory.mktemp("sanitized"))
    san = ["-fsanitize=address", "-fsanitize=undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer"]
    nvcc = B._nvcc()
    cu, cpp = B._sources()
    cmds, objs = [], []
    for src in cu:
        obj = os.path.join(out, os.path.basename(src) + ".o")
        objs.append(obj)
        flags = [f for f in B.NVCC_COMMON if f != "-O3"] + ["-O1", "-g"] + B.ARCH
        if os.path.basename(src) in B.FMAD_OFF:
            flags.append("-fmad=false")
        for s in san:
            flags += ["-Xcompiler", s]
        cmds.append([nvcc] + flags + ["-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(out, os.path.basename(src) + ".o")
        objs.append(obj)
        flags = [f for f in B.CXX_COMMON if f != "-O2"] + ["-O1", "-g"] + san
        cmds.append(["g++"] + flags + ["-I", B._cuda_include(), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, " ".join(cmd) + "\n" + r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as pool:
        list(pool.map(run, cmds))
    lib = os.path.join(out, "libpsim_gb300.so")
    link = [nvcc, "-shared", "-o", lib] + objs + B.ARCH + ["-Xcompiler", "-fPIC"]
    for s in san[:2]:
        link += ["-Xcompiler", s]
    run(link + ["-lasan", "-lubsan"])
    return lib, asan, ubsan


def test_host_library_is_clean_under_sanitizers(sanitized_lib):
    lib, asan, ubsan = sanitized_lib
    env = dict(os.environ, LD_PRELOAD=f"{asan} {ubsan}", ASAN_OPTIONS="detect_leaks=0",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    code = f"ROOT = {ROOT!r}\nGOLDEN = {GOLDEN!r}\nLIB = {lib!r}\n" + CHILD
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=1200)
    report = out.stdout[-2000:] + out.stderr[-6000:]
    assert out.returncode == 0, report
    assert "AddressSanitizer" not in out.stderr and "runtime error:" not in out.stderr, report
    n_models = len(glob.glob(os.path.join(GOLDEN, "models", "*.json*")))
    assert f"sanitized run ok {n_models} models" in out.stdout, report
