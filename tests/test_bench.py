"""bench.py without a GPU: the reference arm's JSON line (the CPU oracle on host threads, on a
bounded sample of the kinked workload), its silence on ranks other than 0, the parsing of the
nvidia-smi clock samples that decide whether a timed run throttled, and the summary of the FP32
kernel's error against FP64 runs of the same random streams."""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def run_bench(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                          env=e, timeout=600)


def test_reference_arm_prints_one_contract_line(built):
    out = run_bench(["--impl", "reference", "--steps", "1", "--warmup", "0", "--measurements", "200",
                     "--cpu-budget", "20000"])
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "phonon-steps/s" and d["unit"] == "phonon-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    assert "kinked" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_is_silent_on_other_ranks():
    out = run_bench(["--impl", "reference", "--steps", "1", "--warmup", "0"], env={"RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""


def test_clock_samples_report_median_and_throttle_reasons():
    rows = [
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1965, 2070, 1395.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "1, 800, 2070, 300.0, 0x0000000000000008, Active, Not Active, Not Active, Not Active",  # another GPU
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",  # unreadable sample
    ]
    c = bench.parse_clocks(rows, 0)
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    c1 = bench.parse_clocks(rows, 1)
    assert c1["reasons"] == ["hw_slowdown"] and c1["sm_mhz"] == 800.0
    assert bench.parse_clocks([], 0)["reasons"] == ["no samples"]


def test_precision_error_covers_temperature_and_flux():
    rng = np.random.default_rng(0)
    s64 = rng.normal(300.0, 0.05, size=(4, 10, 6))
    s64[:, :, 2] = rng.normal(5e3, 40.0, size=(4, 10))
    s64[:, :, 4] = rng.normal(0.0, 40.0, size=(4, 10))
    s32 = s64.copy()
    s32[:, :, 0] += 0.01
    s32[1, 3, 2] += 8.0
    e = bench.precision_error(s32, s64)
    assert np.isclose(e["T"]["mean_abs_diff"], 0.01) and np.isclose(e["mean_abs_diff_K"], 0.01)
    assert np.isclose(e["max_abs_diff_K"], 0.01) and e["seed_to_seed_sd_K"] == e["T"]["seed_to_seed_sd"]
    assert np.isclose(e["flux_x"]["max_abs_diff"], 8.0) and np.isclose(e["flux_x"]["mean_abs_diff"], 8.0 / 40)
    assert e["flux_y"]["max_abs_diff"] == 0.0 and e["flux_y"]["mean_diff_over_sd"] == 0.0
    sd = s64[:, :, 2].std(axis=0, ddof=1).mean()
    assert np.isclose(e["flux_x"]["mean_diff_over_sd"], (8.0 / 40) / sd)


def test_extras_summary_is_short_and_keeps_each_measurement():
    """The headline line carries the extra measurements' figures in a compact form (their full
    records go on lines of their own before it), so the line stays short enough to be kept whole."""
    steady = {"onset_step": -1, "onset_ns": None, "criterion": "x"}
    fp = {"mean_abs_diff_K": 0.02, "max_abs_diff_K": 0.1, "seed_to_seed_sd_K": 0.04, "T": {}, "flux_x": {}}
    batch = {"value": 1.2e10, "models": 256, "alive_at_once": 256,
             "first_64": {"value": 7e9, "worker_threads_value": 9e9, "device_queue_value": 1.1e10, "seconds": 3.0}}
    warm = {"mean_onset_steps_cold": 2400.0, "mean_onset_steps_warm": 600.0, "steps_ratio_cold_over_warm": 4.0,
            "test_rmse_K": 0.2, "per_model": [1] * 500}
    others = {"bar": {"value": 1e10, "e2e": 5e9, "precision": "fp64", "cpu_oracle": {"value": 1e8}, "workload": "w" * 300}}
    ex = bench.summarize_extras(steady, fp, batch, warm, others)
    assert ex["steady_onset_step"] == -1 and ex["batch"]["value"] == 1.2e10
    assert ex["batch"]["first_64"]["device_queue_value"] == 1.1e10
    assert ex["warm_start"]["steps_ratio_cold_over_warm"] == 4.0 and "per_model" not in ex["warm_start"]
    assert ex["other_workloads"]["bar"] == {"value": 1e10, "e2e": 5e9, "precision": "fp64", "cpu": 1e8}
    assert len(json.dumps(ex)) < 1200
    # floats keep four significant digits on the headline line
    assert bench.summarize_extras(None, None, {"value": 11231946816.523619}, None, None)["batch"]["value"] == 1.123e10
    assert bench.summarize_extras(None, None, None, None, None) == {}


def test_demo_model_budget():
    d = bench.demo_model("kinked_demo_120_35_spec", 12345)
    assert d["settings"]["num_phonons"] == 12345 and len(d["cells"]) == 6174
