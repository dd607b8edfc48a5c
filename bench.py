"""Throughput benchmark of the GPU phonon step loop: phonon-steps/s on the kinked
three-arm structure (400 quadrilateral cells / sensors, periodic mode, dt 2 ps, 5000
measurement steps, output every 50 steps, 1e7 phonons per step, Si-like material).

A benchmark step is one complete simulation run of that model (Model::runSimulation).
  value   phonon-steps / device time of the transport kernels, model already on the GPU
  e2e     the same through the public C ABI call (psim_model_run on a freshly loaded model,
          results read back to the host), host<->device copies inside the timed region
Phonon-steps are counted by the kernels (phonons alive at a measurement boundary).

"1e7 phonons per step" is a steady population; psim's input takes a total phonon budget,
so the budget is num_phonons = 1e7 * steps / L with L the mean lifetime in steps measured
by an untimed pilot run of the same model.

Outside the timed region the line also carries:
  batch       256 independent random rectangles run together (autotuned: batched launches fed by a
              device work queue, or models on worker threads)
  warm_start  time to steady state (3 SE, against an independent longer run) of held-out
              rectangles started from the GPU-trained surrogate's temperatures vs the plain
              cold start
  fp32_vs_fp64  the FP32 kernel's error against the FP64 kernel on the same random streams
  other_workloads  the steady-state bar, its full-mode twin and the transient plate, each
              with its device and end-to-end rates beside the CPU oracle

--impl reference times the CPU oracle (the reference algorithm restated in C++, bit-exact
with the reference on the same seed) on a bounded sample of the same model with every host
thread.  Under torchrun each rank simulates its own phonons (weak scaling: the rank's seed
selects its share of the random streams); the tallies are summed once per run.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PER_STEP = 1.0e7
STEPS = 5000
DT_PS = 2.0
BYTES_PER_PHONON_STEP = 64  # one 32-byte state record read and one written
BATCH_CHUNK = 256  # batched models alive at once (state buffers follow each model's population)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, value: float) -> float:
    from psim_gb300 import shard
    return shard.reduce_max(value, dist)


def reduce_sum(dist, value: float) -> float:
    from psim_gb300 import shard
    return shard.reduce_sum(value, dist)


def model_json(path: str, num_phonons: int, steps: int = STEPS, dt_ps: float = DT_PS) -> str:
    from psim_gb300 import modelgen as mg
    m = mg.kinked(seed=0, num_phonons=int(num_phonons), num_measurements=steps, sim_time=steps * dt_ps * 1e-3,
                  step_interval=50)
    return mg.write(m, path)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, out_path: str):
        self.out_path = out_path
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.out_path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self, gpu_index: int = 0) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        return parse_clocks(open(self.out_path).read().splitlines(), gpu_index)


def parse_clocks(lines, gpu_index: int = 0) -> dict:
    """Median SM clock, maximum clock and the throttle reasons seen, from nvidia-smi samples
    (index, clocks.sm, clocks.max.sm, power.draw, active reasons, hw_slowdown,
    hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap) of one GPU."""
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in lines:
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != gpu_index:
            continue
        try:
            sm.append(float(parts[1]))
            mx.append(float(parts[2]))
        except ValueError:
            continue
        for name, flag in zip(names, parts[5:9]):
            if flag.lower() == "active":
                reasons.add(name)
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(path_dir: str, budget: int, threads: int, seed: int, steps: int = STEPS, dt_ps: float = DT_PS):
    """The oracle on a bounded sample of the workload (same model, smaller phonon budget)."""
    from oracle import oracle
    oracle.build()
    p = model_json(os.path.join(path_dir, "kinked_sample.json"), budget, steps, dt_ps)
    r = oracle.run(p, seed, threads=threads)
    return r.phonon_steps, r.seconds


def demo_model(name: str, num_phonons: int = 0) -> dict:
    """One of the reference's demo models kept in the test fixtures (gzipped psim JSON), with its
    phonon budget replaced when num_phonons is given."""
    import gzip
    with gzip.open(os.path.join(ROOT, "tests", "golden", "models", name + ".json.gz"), "rt") as f:
        d = json.load(f)
    if num_phonons:
        d["settings"]["num_phonons"] = int(num_phonons)
    return d


def other_workloads(td: str, precision: int, threads: int, cpu: bool) -> dict:
    """The other single-model workloads, untimed by the headline: per model the device rate
    (phonon-steps / transport-kernel time), the end-to-end rate of psim_model_run (host wall
    time of the call) and, where ``cpu``, the CPU oracle on ``threads`` host threads (the whole
    workload, or a bounded sample of it where stated).  Per-step populations become psim's
    phonon budgets through a pilot run's mean lifetime, as for the kinked model."""
    from psim_gb300 import api, modelgen as mg

    def budget(make, per_step, steps):
        pilot = api.Model(mg.write(make(200000), os.path.join(td, "pilot_w.json")))
        pilot.run(seed=3, precision=precision)
        c = pilot.counters()
        pilot.close()
        return int(per_step * steps / max(c["phonon_steps"] / max(c["phonons"], 1), 1.0))

    bar0 = lambda n: mg.bar(num_cells=10, length=1000.0, width=100.0, t_left=310.0, t_right=290.0, t_init=300.0,
                            t_eq=300.0, num_measurements=2000, sim_time=10.0, num_phonons=n)
    full = lambda n: mg.bar(num_cells=10, length=1000.0, width=100.0, t_left=60.0, t_right=40.0, t_init=50.0,
                            t_eq=0.0, num_measurements=2000, sim_time=10.0, num_phonons=n)
    n0 = budget(bar0, 2e5, 2000)
    cases = [
        ("bar_steady_state_fp64", "1000 x 100 nm bar, 10 cells, deviational steady state, ends 310/290 K, 2e5 phonons "
                                  "per step, dt 5 ps, 2000 steps, FP64 kernel (the configuration's stated precision)",
         bar0(n0), bar0(n0 // 4)),
        ("bar_steady_state", "the same bar with the FP32 kernel (CPU oracle: the row above)", bar0(n0), False),
        ("bar_full_mode", "the same bar in full (non-deviational) mode, ends 60/40 K, 2e5 phonons per step, dt 5 ps, "
                          "2000 steps", full(budget(full, 2e5, 2000)), None),
        ("plate_transient", "4 x 1 um plate, 64 x 16 cells, transient, 400 K pulse on a 200 nm strip of the left edge "
                            "for 20 ps, 2e7 phonons, dt 1 ps, 3000 steps", mg.plate(), mg.plate(num_phonons=100000)),
        ("reference_kinked_demo", "the reference's own kinked demo model (6174 cells, 3108 sensors: tables staged, cell "
                                  "records and tallies in global memory), steady state, 5000 steps, its 2e7 budget",
         demo_model("kinked_demo_120_35_spec"), demo_model("kinked_demo_120_35_spec", 100000)),
    ]
    out = {}
    for key, text, model, sample in cases:
        prec = api.FP64 if key.endswith("_fp64") else precision
        if key == "reference_kinked_demo":
            prec = api.FP32
        path = mg.write(model, os.path.join(td, key + ".json"))
        m = api.Model(path)
        m.run(seed=1, precision=prec)  # warm-up: tables, graph
        t0 = time.perf_counter()
        m.run(seed=2, precision=prec)
        m.measurements()
        wall = time.perf_counter() - t0
        c = m.counters()
        m.close()
        row = {"workload": text, "num_phonons": model["settings"]["num_phonons"], "phonon_steps": c["phonon_steps"],
               "value": c["phonon_steps"] / (c["kernel_ms"] / 1e3), "e2e": c["phonon_steps"] / wall,
               "unit": "phonon-steps/s", "mean_population": c["phonon_steps"] / model["settings"]["num_measurements"],
               "precision": "fp64" if prec == api.FP64 else "fp32"}
        if cpu and sample is not False:
            from oracle import oracle
            cpath = path if sample is None else mg.write(sample, os.path.join(td, key + "_sample.json"))
            r = oracle.run(cpath, 5, threads=threads)
            row["cpu_oracle"] = {"value": r.phonon_steps / r.seconds, "cores": threads, "seconds": r.seconds,
                                 "sample": "the whole workload" if sample is None else
                                 f"the same model with a {sample['settings']['num_phonons']}-phonon budget"}
        out[key] = row
    return out


def precision_error(s32: np.ndarray, s64: np.ndarray) -> dict:
    """Error of FP32 runs against FP64 runs of the same random streams.  s32, s64: per-seed
    measurement tables [seeds, sensors, 6] (T, SE, flux x, SE, flux y, SE).  Temperature keeps
    its historical keys; each quantity also gets its differences against the FP64 runs'
    seed-to-seed spread."""
    out = {"quantity": "per-sensor mean temperature over the run"}
    for name, col, unit in (("T", 0, "K"), ("flux_x", 2, "psim flux column"), ("flux_y", 4, "psim flux column")):
        diff = np.abs(s32[:, :, col] - s64[:, :, col])
        noise = float(s64[:, :, col].std(axis=0, ddof=1).mean())
        row = {"mean_abs_diff": float(diff.mean()), "max_abs_diff": float(diff.max()), "seed_to_seed_sd": noise,
               "mean_diff_over_sd": float(diff.mean() / noise) if noise > 0 else None, "unit": unit}
        if name == "T":
            out.update({"mean_abs_diff_K": row["mean_abs_diff"], "max_abs_diff_K": row["max_abs_diff"],
                        "seed_to_seed_sd_K": noise, "mean_diff_over_sd": row["mean_diff_over_sd"]})
        out[name] = row
    return out


def summarize_extras(steady, fp64_check, batch, warm, others) -> dict:
    """The headline figures of the extra measurements, small enough for the headline line (the
    full records are printed on their own lines before it)."""
    out = {}
    if steady is not None:
        out["steady_onset_step"] = steady["onset_step"]
    if fp64_check is not None:
        out["fp32_vs_fp64_T"] = {k: fp64_check[k] for k in ("mean_abs_diff_K", "max_abs_diff_K", "seed_to_seed_sd_K")}
    if batch is not None:
        out["batch"] = {"value": batch["value"], "mode": batch.get("mode"), "autotuned_value": batch.get("autotuned_value"),
                        "models": batch.get("models"), "alive_at_once": batch.get("alive_at_once"),
                        "first_64": {k: (batch.get("first_64") or {}).get(k) for k in ("value", "worker_threads_value",
                                                                                        "device_queue_value")}}
    if warm is not None:
        keep = ("mean_onset_steps_cold", "mean_onset_steps_warm", "steps_ratio_cold_over_warm",
                "wall_ratio_cold_over_warm_to_steady_stop", "mean_steps_run_cold_to_steady_stop",
                "mean_steps_run_warm_to_steady_stop", "test_rmse_K", "stopped_within_3se_cold",
                "stopped_within_3se_warm", "held_out_models", "train_fields")
        out["warm_start"] = {k: warm[k] for k in keep if k in warm}
    if others is not None:
        out["other_workloads"] = {k: {"value": v["value"], "e2e": v["e2e"], "precision": v["precision"],
                                      "cpu": (v.get("cpu_oracle") or {}).get("value")} for k, v in others.items()}
    return _rounded(out)


def _rounded(x, digits: int = 4):
    """Floats to `digits` significant digits (the full values are on the detail lines)."""
    if isinstance(x, float):
        return float(f"{x:.{digits}g}")
    if isinstance(x, dict):
        return {k: _rounded(v, digits) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [_rounded(v, digits) for v in x]
    return x


def workload_name(args) -> str:
    return (f"kinked 3-arm structure, 400 quadrilateral cells / sensors, periodic, dt {args.dt_ps:g} ps, "
            f"{args.measurements} steps, output every 50 steps, {args.per_step:.0e} phonons per step")


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm (CPU oracle) on every host thread."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    budget = args.cpu_budget
    with tempfile.TemporaryDirectory() as td:
        for _ in range(args.warmup):
            cpu_sample(td, budget, threads, 7, args.measurements, args.dt_ps)
        steps = 0
        secs = 0.0
        for k in range(args.steps):
            n, s = cpu_sample(td, budget, threads, 100 + k, args.measurements, args.dt_ps)
            steps += n
            secs += s
    rate = steps / secs
    line = {
        "impl": "reference", "metric": "phonon-steps/s", "value": rate, "unit": "phonon-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args), "num_phonons": budget,
                   "sample": f"budget {budget} phonons per run (a bounded CPU sample of the same model)"},
        "cpu_baseline": {"value": rate, "unit": "phonon-steps/s", "cores": threads, "kind": "port",
                         "sample": f"kinked model, {args.measurements} steps, {budget}-phonon budget per run, on {threads} host threads; "
                                   "the reference built from its sources (oracle/_ref) cannot be built without them, so "
                                   "the bit-exact C++ restatement of its algorithm (oracle/) runs"},
        "e2e": {"value": rate, "unit": "phonon-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--per-step", type=float, default=PER_STEP)
    ap.add_argument("--measurements", type=int, default=STEPS)
    ap.add_argument("--dt-ps", type=float, default=DT_PS, help="measurement step length in ps")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--cpu-budget", type=int, default=3000000)
    ap.add_argument("--population-out", default="", help="write the phonon population per step of the last timed run (JSON)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-others", action="store_true", help="skip the other single-model workloads")
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the FP32-vs-FP64 same-stream comparison")
    ap.add_argument("--batch-models", type=int, default=256,
                    help="models of the batched workload (random rectangles) to time concurrently; 0 skips it")
    ap.add_argument("--warm-start-train", type=int, default=1024,
                    help="training fields of the warm-start surrogate (0 skips the warm-start measurement)")
    ap.add_argument("--warm-start-test", type=int, default=32, help="held-out rectangles of the warm-start measurement")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = init_dist(world, "nccl")
    from psim_gb300 import api, build, shard
    # the once-per-run tally exchange runs on host buffers: a gloo group beside NCCL
    tally_group = dist.new_group(backend="gloo") if dist is not None else None
    build.build()
    precision = api.FP64 if args.precision == "fp64" else api.FP32
    steps_n = args.measurements
    td = tempfile.mkdtemp(prefix="psim_bench_")

    # pilot run (untimed): mean lifetime in steps -> phonon budget for the target population
    pilot = api.Model(model_json(os.path.join(td, "pilot.json"), 200000, steps_n, args.dt_ps))
    pilot.run(seed=shard.rank_seed(99, rank), precision=precision)
    pc = pilot.counters()
    lifetime = pc["phonon_steps"] / max(pc["phonons"], 1)
    budget = int(args.per_step * steps_n / lifetime)
    path = model_json(os.path.join(td, "kinked.json"), budget, steps_n, args.dt_ps)
    model = api.Model(path)

    stream = torch.cuda.Stream()
    for w in range(args.warmup):
        model.run(seed=shard.rank_seed(1000 + w, rank), precision=precision, stream=stream.cuda_stream)

    # ---- timed: device-resident runs
    clocks = ClockSampler(os.path.join(td, "clocks.csv"))
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    phonon_steps = 0
    kernel_ms = 0.0
    launches = 0
    transport_launches = 0
    t0 = time.perf_counter()
    ev0.record(stream)
    for k in range(args.steps):
        model.run(seed=shard.rank_seed(7000 + k, rank), precision=precision, stream=stream.cuda_stream)
        if dist is not None:
            shard.combine_tallies(*model.tallies(), dist, tally_group)
        c = model.counters()
        phonon_steps += c["phonon_steps"]
        kernel_ms += c["kernel_ms"]
        launches += c["kernel_launches"]
        transport_launches += c["transport_launches"]
    ev1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if args.population_out:
        with open(args.population_out, "w") as f:
            json.dump({"population": model.population().tolist(), "pilot_runs": 1, "warmup_runs": args.warmup,
                       "timed_runs": args.steps, "steps_per_run": steps_n}, f)
    clk = clocks.stop(local)
    barrier(dist)
    span_ms = ev0.elapsed_time(ev1)
    kernel_s = reduce_max(dist, kernel_ms / 1e3)
    span_s = reduce_max(dist, span_ms / 1e3)
    total_steps = reduce_sum(dist, float(phonon_steps))
    # value: phonon-steps over the CUDA-event span of the K timed runs (host work between runs,
    # births, graph set-up and buffer checks included); kernel_value: over the transport
    # kernels' own device time
    value = total_steps / span_s
    kernel_value = total_steps / kernel_s
    ms_per_step = 1e3 * span_s / args.steps

    # roofline of the dominant kernel (the FP32/FP64 transport step): 64 B per phonon-step (one
    # 32-byte state record read and one written) times the phonon-steps one launch covers; an FP32
    # launch covers several measurement steps, keeping phonons in registers across the inner ones
    per_launch_bytes = phonon_steps / transport_launches * BYTES_PER_PHONON_STEP * (2 if precision == api.FP64 else 1)
    avg_launch_s = kernel_ms / 1e3 / transport_launches
    peak, peak_kind = peaks()
    achieved = per_launch_bytes / avg_launch_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "peak_source": f"{peak_kind} hbm_gbs", "kernel": "step_kernel_" + args.precision,
                "algorithmic_bytes_per_launch": per_launch_bytes, "avg_launch_us": avg_launch_s * 1e6}
    profile = os.path.join(ROOT, "profiles", f"traffic_step_kernel_{args.precision}_kinked.json")
    if os.path.exists(profile):
        tr = json.load(open(profile))
        roofline["traffic"] = tr.get("dram_bytes_per_phonon_step", 0) * phonon_steps / transport_launches
        roofline["traffic_source"] = tr.get("source")
        if "issue_active_pct" in tr:  # the bound that holds: instruction issue, from the same kernel's capture
            roofline["issue_slot_utilisation"] = tr["issue_active_pct"] / 100.0
            roofline["lanes_per_instruction"] = tr.get("lanes_per_instruction")
            roofline["issue_source"] = tr.get("issue_source")

    # time to steady state of the last timed run (a cold start: every cell at T_ref), by the
    # detector on its device tallies; outside the timed region
    onset, _ = model.steady_state(window=250, batches=5, z=3.0, patience=3)
    steady = {"onset_step": onset, "onset_ns": onset * args.dt_ps * 1e-3 if onset >= 0 else None,
              "criterion": "windows of 250 steps (5 batch means) agree within 3 SE for 3 windows, energy and flux, every sensor"}

    # ---- e2e through the public C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        barrier(dist)
        e_steps = 0
        h2d = d2h = 0
        t0 = time.perf_counter()
        for k in range(args.steps):
            m = api.Model(path)
            m.run(seed=shard.rank_seed(9000 + k, rank), precision=precision)
            if dist is not None:
                shard.combine_tallies(*m.tallies(), dist, tally_group)
            stats = m.measurements()
            temps, fluxes = m.series(0)
            c = m.counters()
            e_steps += c["phonon_steps"]
            h2d += c["h2d_bytes"]
            d2h += c["d2h_bytes"] + stats.nbytes + temps.nbytes + fluxes.nbytes
            m.close()
        e_wall = time.perf_counter() - t0
        barrier(dist)
        e_wall = reduce_max(dist, e_wall)
        e_total = reduce_sum(dist, float(e_steps))
        e2e = {"value": e_total / e_wall, "unit": "phonon-steps/s", "h2d_bytes_per_step": int(h2d / args.steps),
               "d2h_bytes_per_step": int(d2h / args.steps)}

    # FP32 error against the FP64 kernel on the same random streams: the same geometry at a
    # budget the FP64 kernel runs in seconds (outside the timed region)
    fp64_check = None
    if rank == 0 and world == 1 and not args.no_fp64_check and precision == api.FP32:
        per_step = 2.0e4
        small = api.Model(model_json(os.path.join(td, "kinked_fp64.json"), int(per_step * steps_n / lifetime), steps_n,
                                     args.dt_ps))
        s32, s64 = [], []
        for seed in range(1, 5):
            s32.append(small.run(seed=seed, precision=api.FP32).measurements())
            s64.append(small.run(seed=seed, precision=api.FP64).measurements())
        fp64_check = {"workload": f"the same model at {per_step:.0e} phonons per step, 4 seeds, FP32 and FP64 kernels on the same random streams"}
        fp64_check.update(precision_error(np.array(s32), np.array(s64)))

    # the batched workload: independent random rectangles (uneven cells and populations) run
    # together with the autotuner's options (batched launches fed by a device work queue, or
    # models on worker threads), BATCH_CHUNK models alive at once; the first 64 models also run one
    # at a time, and with the worker-thread batch, for comparison
    batch = None
    if rank == 0 and world == 1 and args.batch_models > 0:
        from psim_gb300 import modelgen as mg
        opt = None
        secs = 0.0
        steps_b = 0
        other_secs = 0.0
        other_steps = 0
        single = None
        for c0 in range(0, args.batch_models, BATCH_CHUNK):
            ids = range(c0, min(c0 + BATCH_CHUNK, args.batch_models))
            paths = [mg.write(mg.random_bar(1000 + i), os.path.join(td, f"rect_{i}.json")) for i in ids]
            models = [api.Model(p).set_options(seed=i + 1, precision=precision) for i, p in zip(ids, paths)]
            if opt is None:
                opt, tuned_rate = api.batch_autotune(models, sample=min(16, len(models)))
            s_c, n_c = api.batch_run(models, workers=opt.workers, max_blocks=opt.max_blocks,
                                     device_queue=bool(opt.device_queue), per_thread=opt.per_thread)
            secs += s_c
            steps_b += n_c
            # the same models the other way, for comparison (the autotuner decides on up to 64 of
            # them; the device queue gains with the number of models it can spread over the SMs)
            s_o, n_o = api.batch_run(models, workers=16 if opt.device_queue else opt.workers, max_blocks=opt.max_blocks,
                                     device_queue=not bool(opt.device_queue), per_thread=opt.per_thread)
            other_secs += s_o
            other_steps += n_o
            if single is None:
                first = models[:64]
                t0 = time.perf_counter()
                steps_s = 0
                kernel_s = 0.0
                for i, m in zip(ids, first):
                    m.run(seed=i + 1, precision=precision)
                    c1 = m.counters()
                    steps_s += c1["phonon_steps"]
                    kernel_s += c1["kernel_ms"] / 1e3
                secs_s = time.perf_counter() - t0
                s_t, n_t = api.batch_run(first, workers=16, device_queue=False)
                s_q, n_q = api.batch_run(first, workers=16, device_queue=True, per_thread=opt.per_thread)
                # device_value: the same models' phonon-steps over their transport-kernel time
                # alone, the rate the batch would reach if concurrency added nothing
                single = {"models": len(first), "value": steps_s / secs_s, "seconds": secs_s,
                          "device_value": steps_s / kernel_s, "worker_threads_value": n_t / s_t,
                          "device_queue_value": n_q / s_q}
            for m in models:
                m.close()
        batch = {"workload": f"{args.batch_models} random rectangles: length U(0.2, 5) um, width U(50, 500) nm, 4-200 cells, "
                             "1e4-1e6 phonons per step (log-uniform), ends U(280, 320) K, walls U(0, 1) specular; "
                             f"3000 steps of 5 ps, steady state; {min(BATCH_CHUNK, args.batch_models)} alive at once",
                 "autotuned": {"device_queue": opt.device_queue, "per_thread": opt.per_thread, "workers": opt.workers,
                               "max_blocks": opt.max_blocks, "pilot_rate": tuned_rate, "pilot_models": min(16, args.batch_models),
                               "wider_models": min(64, args.batch_models)},
                 "autotuned_value": steps_b / secs, "unit": "phonon-steps/s",
                 "other_mode": {"device_queue": not bool(opt.device_queue), "value": other_steps / other_secs,
                                "seconds": other_secs},
                 "models": args.batch_models, "alive_at_once": min(BATCH_CHUNK, args.batch_models),
                 "first_64": single}
        # the batch's rate: the faster of the two ways, both measured on the same models
        queue_best = other_steps / other_secs > steps_b / secs if not opt.device_queue else steps_b / secs >= other_steps / other_secs
        batch.update({"value": max(steps_b / secs, other_steps / other_secs),
                      "mode": "device work queue" if queue_best else "worker threads"})

    # the learned warm start: a surrogate trained on GPU Monte Carlo steady fields (outside the
    # timed region), held-out rectangles run cold and warm, each timed to steady state at 3 SE
    # against an independent run twice as long
    warm = None
    if rank == 0 and world == 1 and args.warm_start_train > 0 and precision == api.FP32:
        from psim_gb300 import surrogate as sg
        t0 = time.perf_counter()
        X, Y = sg.generate(range(10000, 10000 + args.warm_start_train))
        t_gen = time.perf_counter() - t0
        net, loss = sg.train(X, Y)
        held = sg.held_out(args.warm_start_test)
        Xt, Yt = sg.generate(held)
        test_rmse = float(np.sqrt(np.mean((net.predict(Xt) - Yt) ** 2)) * sg.T_SCALE)
        rep = sg.summary(sg.evaluate(net, held, steps=6000))
        net.close()
        warm = {"workload": f"surrogate (12 -> 4 x 256 GELU -> 32 x 32, BF16 with FP32 sums) trained 200 epochs on "
                            f"{args.warm_start_train} steady fields of random rectangles; {len(held)} held-out rectangles "
                            "up to 2 um, 6000 steps of 5 ps, every step recorded",
                "train_fields_s": t_gen, "final_train_loss": loss, "test_rmse_K": test_rmse}
        warm.update(rep)

    others = None
    if rank == 0 and world == 1 and not args.no_others:
        others = other_workloads(td, precision, os.cpu_count() or 1, not args.no_cpu)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        n, s = cpu_sample(td, args.cpu_budget, threads, 5, steps_n, args.dt_ps)
        cpu = {"value": n / s, "unit": "phonon-steps/s", "cores": threads, "kind": "port",
               "sample": f"kinked model, {steps_n} steps, {args.cpu_budget}-phonon budget ({n} phonon-steps, {s:.1f} s) "
                         f"on {threads} host threads with the CPU oracle"}

    if rank == 0:
        # the extra measurements in full, one short JSON line each, before the headline line
        details = {"steady_state": steady, "fp32_vs_fp64": fp64_check, "batch": batch, "warm_start": warm}
        if others is not None:
            details.update({f"other_workloads.{k}": v for k, v in others.items()})
        for key, v in details.items():
            if v is not None:
                print(json.dumps({"detail": key, **v}), flush=True)
        line = {
            "metric": "phonon-steps/s", "value": value, "unit": "phonon-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if precision == api.FP32 else "f64",
            "data": "synthetic",
            "config": {"workload": workload_name(args),
                       "num_phonons_per_rank": budget, "mean_lifetime_steps": lifetime,
                       "mean_population": phonon_steps / args.steps / steps_n,
                       "l2": "inputs larger than L2 (phonon state 2 x 32 B x population)",
                       "precision": args.precision, "bench_step": "one full simulation run",
                       "steps_per_launch": c["steps_per_launch"], "state_bytes": c["state_bytes"]},
            "value_source": "phonon-steps / CUDA-event span of the timed runs",
            "kernel_value": kernel_value,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches * world,
            "clocks": clk, "wall_s_timed": wall,
            "extras": summarize_extras(steady, fp64_check, batch, warm, others),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
