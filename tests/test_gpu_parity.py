"""Statistical parity of the GPU Monte Carlo with the reference (tests/golden/runs_*.npz: the
reference's per-sensor results for 16 seeds).  Random streams differ, so per-sensor mean
temperature and heat flux are compared over 16 seeds each side, in units of the combined
standard error sqrt(SE_gpu^2 + SE_ref^2), SE = seed-to-seed standard deviation / sqrt(16).

Pass criterion per model (T, flux x, flux y of every sensor): no |z| above the bound of
max_z (4.5, or Student's t at a 1 % family-wise rate where the values are many) and at most 5 %
of the values (at least one allowed) above 3.  With independent z-scores the chance of a false
failure is about 1 %."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, demo_model_path, model_path

pytestmark = pytest.mark.gpu

SEEDS = range(1, 17)
COLUMNS = {"T": 0, "flux_x": 2, "flux_y": 4}


@pytest.fixture(scope="module")
def api(gpu):
    from psim_gb300 import api
    return api


def gpu_stats(api, name, precision):
    m = api.Model(model_path(name))
    out = []
    for seed in SEEDS:
        m.run(seed=1000 + seed, precision=precision)
        out.append(m.measurements())
    return np.stack(out)


def zscores(a, b):
    """a, b: [seeds, sensors, 6] -> z [sensors, 3] for T, flux x, flux y."""
    zs = []
    for col in COLUMNS.values():
        ma, mb = a[:, :, col].mean(axis=0), b[:, :, col].mean(axis=0)
        sa = a[:, :, col].std(axis=0, ddof=1) / np.sqrt(a.shape[0])
        sb = b[:, :, col].std(axis=0, ddof=1) / np.sqrt(b.shape[0])
        se = np.sqrt(sa ** 2 + sb ** 2)
        z = np.where(se > 0, (ma - mb) / np.where(se > 0, se, 1.0), np.where(ma == mb, 0.0, np.inf))
        zs.append(z)
    return np.stack(zs, axis=1)


def max_z(n: int) -> float:
    """Largest |z| allowed among n values: Student's t (the combined SE comes from two 16-seed
    spreads, about 30 degrees of freedom) at a 1 % family-wise rate over the n values, and never
    below 4.5.  Up to about a thousand values that is the plain 4.5; the reference's larger demo
    models compare 3000 and 9324 values, where a fixed 4.5 would fail on noise alone in about
    one run out of six."""
    from scipy.stats import t
    return max(4.5, float(t.ppf(1.0 - 0.005 / n, 30)))


def check(z, label):
    az = np.abs(z)
    over3 = int((az > 3.0).sum())
    allowed = max(1, int(0.05 * az.size))
    cap = max_z(az.size)
    print(f"{label}: max |z| {az.max():.2f} (bound {cap:.2f}), {over3}/{az.size} above 3")
    assert az.max() < cap, (label, az.max(), cap)
    assert over3 <= allowed, (label, over3)


@pytest.mark.parametrize("name", ["bar_ss", "bar_full", "bar_periodic", "kinked_small", "plate_small", "bar_runs",
                                  "bar_phasor"])
def test_fp32_matches_reference(api, name):
    ref = np.load(os.path.join(GOLDEN, f"runs_{name}.npz"))["stats"]
    got = gpu_stats(api, name, api.FP32)
    check(zscores(got, ref), f"{name} fp32")


@pytest.mark.parametrize("name", ["linear_demo", "linear_sides_demo_ss", "kinked_demo_120_35_spec"])
def test_fp32_matches_reference_on_its_demo_models(api, name, tmp_path):
    """The reference's own demo models (psim_python/json/), against 16 seeded runs of the
    reference built from its current sources.  The result tables the reference commits for
    these models came from an older version of psim and lie several combined SE from its
    current sources' runs; they are reported here, not used as the bar.  The kinked demo
    (6174 cells, 3108 sensors) is larger than the shared-memory tables and tallies hold, so it
    runs the transport kernel with global tables and global tally atomics."""
    gold = np.load(os.path.join(GOLDEN, f"runs_{name}.npz"))
    ref = gold["stats"].astype(np.float64)
    m = api.Model(demo_model_path(name, str(tmp_path)))
    out = []
    for seed in SEEDS:
        m.run(seed=1000 + seed, precision=api.FP32)
        out.append(m.measurements())
    got = np.stack(out)
    check(zscores(got, ref), f"{name} fp32")
    committed = gold["committed"].astype(np.float64)
    sd = ref[:, :, 0].std(axis=0, ddof=1)
    z = (committed[:, 0] - ref[:, :, 0].mean(axis=0)) / np.where(sd > 0, sd, 1.0)
    print(f"{name}: the reference's committed table against its current runs, mean z(T) {z.mean():.2f}, "
          f"max |z(T)| {np.abs(z).max():.2f} (in seed-to-seed SD)")


# The benchmark configurations as stated (tests/golden/make_golden.py: headline_specs): the
# steady-state bar of 2000 steps of 5 ps at 2e5 phonons per step, its full-mode twin at 60/40 K,
# the 64 x 16 transient plate (3000 steps of 1 ps, reduced budget), the 400-sensor kinked
# structure (periodic, 5000 steps of 2 ps, reduced budget) and the silicon | germanium bar.
HEADLINE = ["cfg0_bar_ss", "cfg2b_bar_full", "cfg2a_plate", "cfg1_kinked", "si_ge_bar"]


@pytest.mark.parametrize("name", HEADLINE)
def test_fp32_matches_reference_on_the_benchmark_configurations(api, name):
    ref = np.load(os.path.join(GOLDEN, f"runs_{name}.npz"))["stats"].astype(np.float64)
    got = gpu_stats(api, name, api.FP32)
    check(zscores(got, ref), f"{name} fp32")


def test_fp32_matches_reference_on_the_kinked_benchmark_at_its_own_budget(api, tmp_path):
    """The kinked structure exactly as the benchmark times it: 1e7 phonons per step, a budget of
    1.2e8 phonons (5000 steps over a mean lifetime of about 415 steps), against the reference's
    16 runs at a budget of 6e6.  The per-sensor means of a deviational run do not depend on the
    budget (the energy per phonon scales with it), so only the noise of the two sides differs."""
    import json
    ref = np.load(os.path.join(GOLDEN, "runs_cfg1_kinked.npz"))["stats"].astype(np.float64)
    d = json.load(open(model_path("cfg1_kinked")))
    d["settings"]["num_phonons"] = 120000000
    path = os.path.join(str(tmp_path), "cfg1_kinked_full.json")
    with open(path, "w") as f:
        json.dump(d, f)
    m = api.Model(path)
    out = []
    for seed in SEEDS:
        m.run(seed=3000 + seed, precision=api.FP32)
        out.append(m.measurements())
    c = m.counters()
    print(f"cfg1_kinked at 1.2e8 phonons: {c['phonon_steps']:.4g} phonon-steps per run, "
          f"{c['state_bytes'] / 1e9:.2f} GB of state buffers (peak population {c['max_population']})")
    check(zscores(np.stack(out), ref), "cfg1_kinked full budget fp32")
    # the state buffers follow the peak population (about 1e7), not the run's 1.2e8 phonons
    assert c["state_bytes"] < 1.5e9


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_two_materials_backscatter_and_match_reference(api, precision):
    """The silicon | germanium bar: phonons cross the interface both ways, and silicon phonons
    above germanium's branch maxima are diffusely backscattered (TransitionSurface::handlePhonon,
    psim/src/surface.cpp:71-109).  Per-sensor results match the reference's 16 runs."""
    ref = np.load(os.path.join(GOLDEN, "runs_si_ge_bar.npz"))["stats"]
    m = api.Model(model_path("si_ge_bar"))
    prec = api.FP32 if precision == "fp32" else api.FP64
    out = []
    backs = []
    for seed in SEEDS:
        m.run(seed=1000 + seed, precision=prec)
        out.append(m.measurements())
        backs.append(m.counters()["backscatters"])
    print(f"si_ge_bar {precision}: {np.mean(backs):.0f} backscatters per run")
    assert min(backs) > 0
    check(zscores(np.stack(out), ref), f"si_ge_bar {precision}")


@pytest.mark.parametrize("name", ["bar_ss", "bar_full", "kinked_small", "plate_small", "cfg0_bar_ss"])
def test_fp64_matches_reference(api, name):
    ref = np.load(os.path.join(GOLDEN, f"runs_{name}.npz"))["stats"]
    got = gpu_stats(api, name, api.FP64)
    check(zscores(got, ref), f"{name} fp64")


@pytest.mark.parametrize("name", ["bar_ss", "kinked_small"])
def test_fp32_error_against_fp64_same_stream(api, name):
    """The FP32 kernel's error, measured against the FP64 kernel on the same random stream:
    per-sensor differences stay well inside the statistical noise."""
    m = api.Model(model_path(name))
    d32 = []
    d64 = []
    for seed in range(1, 9):
        d32.append(m.run(seed=seed, precision=api.FP32).measurements())
        d64.append(m.run(seed=seed, precision=api.FP64).measurements())
    d32, d64 = np.stack(d32), np.stack(d64)
    ref = np.load(os.path.join(GOLDEN, f"runs_{name}.npz"))["stats"]
    noise = ref[:, :, 0].std(axis=0, ddof=1)
    diff = np.abs(d32[:, :, 0] - d64[:, :, 0])
    print(f"{name}: |T32 - T64| mean {diff.mean():.3e} K, max {diff.max():.3e} K; run-to-run noise {noise.mean():.3e} K")
    assert diff.mean() < 0.5 * noise.mean()
