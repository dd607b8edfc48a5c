"""Learned warm start for the batched rectangles.

A multilayer perceptron (``api.Mlp``: hand-written BF16 GPU kernels with FP32 accumulation,
Adam) maps a rectangle's 12 descriptors to its steady temperature map, rasterised to 32 x 32.
The training fields are steady states the GPU Monte Carlo computes itself, a batch of random
rectangles at a time (``api.batch_run``).  Starting a run from the map's temperatures instead of
the uniform reference temperature (the plain cold start) shortens the burn-in to steady state.
Both starts are timed against the steady temperatures of an independent longer run: the step
from which every sensor stays within 3 standard errors of them (``onset_vs_reference``).

    python -m psim_gb300.surrogate --train 2048 --test 64 --out report.json
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import time
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import api
from . import modelgen as mg

FEATURES = 12
RASTER = 32
T_REF = 300.0
T_SCALE = 20.0
WIDTHS = [FEATURES, 256, 256, 256, 256, RASTER * RASTER]


def features(q: Dict) -> np.ndarray:
    """Length, width, four wall specularities (one value for the whole wall here), the two end
    temperatures and four shape flags (a plain rectangle), scaled to order one."""
    s = q["spec"]
    return np.array([q["length"] / 5000.0, q["width"] / 500.0, s, s, s, s, (q["t_left"] - T_REF) / T_SCALE,
                     (q["t_right"] - T_REF) / T_SCALE, 1.0, 0.0, 0.0, 0.0], dtype=np.float32)


def raster(temps: Sequence[float], q: Dict) -> np.ndarray:
    """A bar's per-cell temperatures on a 32 x 32 map of its (length, width): the cell under
    each column's centre, every row alike, scaled as (T - T_REF) / T_SCALE."""
    temps = np.asarray(temps, dtype=np.float64)
    cells = len(temps)
    x = (np.arange(RASTER) + 0.5) / RASTER
    col = (temps[np.minimum((x * cells).astype(int), cells - 1)] - T_REF) / T_SCALE
    return np.tile(col, (RASTER, 1)).astype(np.float32).ravel()


def sensor_temps(r: np.ndarray, q: Dict, cells: int) -> np.ndarray:
    """Each cell's temperature read off a 32 x 32 map: the row mean, interpolated linearly along
    the length at the cell's centre."""
    col = np.asarray(r, dtype=np.float64).reshape(RASTER, RASTER).mean(axis=0)
    xc = (np.arange(RASTER) + 0.5) / RASTER
    xs = (np.arange(cells) + 0.5) / cells
    return T_REF + T_SCALE * np.interp(xs, xc, col)


def _models(seeds: Sequence[int], td: str, *, periodic: bool, steps: int, scale: float) -> List[Tuple[api.Model, Dict]]:
    out = []
    for k in seeds:
        path = mg.write(mg.random_bar(k, periodic=periodic, steps=steps, per_step_scale=scale), os.path.join(td, f"r{k}.json"))
        out.append((api.Model(path).set_options(seed=k), mg.random_bar_params(k)))
    return out


CHUNK = 128  # models alive at once: each keeps GPU buffers sized for its run's phonons


@dataclass(frozen=True)
class StopRule:
    """A steady stop: windows of ``window`` steps (``batches`` batch means) within ``z`` standard
    errors of the sensor's anchor window for ``patience`` windows, with no trend over them beyond
    ``drift_z`` standard errors (0: no trend test), checked every ``every`` steps (0: every
    ``patience`` + 1 windows)."""
    window: int
    batches: int
    z: float
    patience: int
    drift_z: float = 0.0
    every: int = 0

    def detector(self) -> Dict:
        return {"window": self.window, "batches": self.batches, "z": self.z, "patience": self.patience,
                "drift_z": self.drift_z}

    def describe(self) -> str:
        return (f"windows of {self.window} steps ({self.batches} batch means) within {self.z:g} SE of the anchor window "
                f"for {self.patience} windows" + (f", no trend beyond {self.drift_z:g} SE" if self.drift_z > 0 else "")
                + f", checked every {self.every if self.every > 0 else (self.patience + 1) * self.window} steps")

    @staticmethod
    def parse(text: str) -> "StopRule":
        """'window,batches,z,patience[,drift_z[,every]]'."""
        f = text.split(",")
        if not 4 <= len(f) <= 6:
            raise ValueError(f"a stop rule is window,batches,z,patience[,drift_z[,every]], not {text!r}")
        return StopRule(int(f[0]), int(f[1]), float(f[2]), int(f[3]), float(f[4]) if len(f) > 4 else 0.0,
                        int(f[5]) if len(f) > 5 else 0)


# The steady stops of the evaluation's runs, one for each kind of start.  Both stop runs that are
# within 3 SE of the steady state (window standard) about 65 % of the time on 512 held-out
# rectangles: a warm run, which starts close to its steady state, can be stopped by shorter
# windows at the same accuracy.  STOP_WARM is the warm runs' fastest rule of a grid at that
# accuracy; STOP_COLD is within 1 % of the cold runs' fastest.
STOP_COLD = StopRule(200, 10, 3.5, 2, 0.0, 200)
STOP_WARM = StopRule(50, 5, 3.0, 3, 0.0, 50)


def generate(seeds: Sequence[int], *, steps: int = 3000, scale: float = 1.0, workers: int = 16) -> Tuple[np.ndarray, np.ndarray]:
    """Steady fields of the rectangles drawn from ``seeds``: the Monte Carlo run of each (steady
    state mode), its sensors' mean temperatures rasterised."""
    seeds = list(seeds)
    X, Y = [], []
    with tempfile.TemporaryDirectory() as td:
        for c0 in range(0, len(seeds), CHUNK):
            pairs = _models(seeds[c0:c0 + CHUNK], td, periodic=False, steps=steps, scale=scale)
            api.batch_run([m for m, _ in pairs], workers=workers)
            X += [features(q) for _, q in pairs]
            Y += [raster(m.measurements()[:, 0], q) for m, q in pairs]
            for m, _ in pairs:
                m.close()
    return np.stack(X), np.stack(Y)


def train(X: np.ndarray, Y: np.ndarray, *, epochs: int = 200, batch: int = 256, lr: float = 1e-3, seed: int = 1) -> Tuple[api.Mlp, float]:
    net = api.Mlp(WIDTHS, seed=seed)
    loss = net.train(X, Y, batch=batch, epochs=epochs, lr=lr, seed=seed)
    return net, loss


def _final(m: api.Model, frac: float = 1.0 / 3.0, batches: int = 20) -> Tuple[np.ndarray, np.ndarray]:
    """Mean and standard error (batch means) of every sensor's temperature over the run's last
    ``frac`` of recorded steps."""
    temps, _ = m.series(0)
    k = temps.shape[1]
    tail = temps[:, k - int(k * frac):]
    n = tail.shape[1] // batches * batches
    bm = tail[:, tail.shape[1] - n:].reshape(tail.shape[0], batches, -1).mean(axis=2)
    return bm.mean(axis=1), bm.std(axis=1, ddof=1) / np.sqrt(batches)


def _bound(tests: int, dof: int = 0) -> float:
    """Two-sided bound for `tests` simultaneous comparisons with the family-wise error rate of
    one 3-SE test (0.27 %, Bonferroni): a normal quantile, or Student's t with `dof` degrees of
    freedom when the spread is itself estimated."""
    p = 1.0 - 0.00135 / max(tests, 1)
    if dof > 0:
        from scipy.stats import t
        return float(t.ppf(p, dof))
    from statistics import NormalDist
    return NormalDist().inv_cdf(p)


def _window_means(temps: np.ndarray, window: int) -> np.ndarray:
    nw = temps.shape[1] // window
    return temps[:, :nw * window].reshape(temps.shape[0], nw, window).mean(axis=2)


def steady_reference(temps: np.ndarray, window: int) -> Tuple[np.ndarray, np.ndarray, int]:
    """Each sensor's steady temperature and the spread of one window mean about it, from the
    second half of a long converged run: the mean; the standard deviation of its window means
    (so the steps' correlation is in it) combined with the reference mean's own error; and the
    degrees of freedom of that estimate."""
    half = temps[:, temps.shape[1] // 2:]
    wm = _window_means(half, window)
    sd = wm.std(axis=1, ddof=1)
    return half.mean(axis=1), np.sqrt(sd * sd + sd * sd / wm.shape[1]), wm.shape[1] - 1


def onset_vs_reference(temps: np.ndarray, t_inf: np.ndarray, spread: np.ndarray, dof: int, window: int) -> int:
    """First recorded step from which every later window mean of every sensor lies within the
    3-SE prediction bound of the steady temperature (Student's t on the reference's degrees of
    freedom, family-wise over all sensors and windows); -1 when the last window does not."""
    wm = _window_means(temps, window)
    z = _bound(wm.size, dof)
    ok = np.all(np.abs(wm - t_inf[:, None]) <= z * spread[:, None], axis=0)
    bad = np.flatnonzero(~ok)
    if bad.size == 0:
        return 0
    if bad[-1] == ok.size - 1:
        return -1
    return int(bad[-1] + 1) * window


def stopped_within(m: api.Model, ref: Tuple[np.ndarray, np.ndarray, int], window: int, rule: StopRule) -> Tuple[bool, bool]:
    """Whether a run stopped by the steady-state detector was steady at 3 SE where the detector
    said so, by two standards:
    - windows: every window mean of every sensor from the detector's onset to the stop lies
      within the prediction bound of the reference's steady temperature, the standard the time
      to steady state (``onset_vs_reference``) is measured by;
    - mean: each sensor's mean over the same steps lies within that bound scaled to the averaged
      length (spread x sqrt(window / steps), windows taken as independent), family-wise over the
      sensors: a much tighter standard, since the mean of many windows has a smaller error."""
    temps, _ = m.series(0)
    onset, _ = m.steady_state(**rule.detector())
    k = temps.shape[1]
    start = onset if 0 <= onset < k else max(k - window, 0)
    t_inf, spread, dof = ref
    wm = _window_means(temps[:, start:], window)
    windows_ok = bool(wm.size == 0 or np.all(np.abs(wm - t_inf[:, None]) <= _bound(wm.size, dof) * spread[:, None]))
    mean = temps[:, start:].mean(axis=1)
    se = np.sqrt(spread * spread * window / max(k - start, 1))
    mean_ok = bool(np.all(np.abs(mean - t_inf) <= _bound(len(t_inf), dof) * se))
    return windows_ok, mean_ok


def evaluate(net: api.Mlp, seeds: Sequence[int], *, steps: int = 3000, scale: float = 1.0, window: int = 100,
             stop_cold: StopRule = STOP_COLD, stop_warm: StopRule = STOP_WARM, workers: int = 16) -> Dict:
    """Cold and warm starts of the rectangles drawn from ``seeds``.

    A third, twice as long, warm-started run of each rectangle with its own seed gives the steady
    temperatures and their window tolerance (``steady_reference``).  The cold and warm runs (every
    step recorded) are timed to steady state against it (``onset_vs_reference``: at 3 SE) and by
    the run's own detector; then the same runs again with the steady stop on (``stop_cold`` for
    the cold runs, ``stop_warm`` for the warm ones) give the wall time and steps a batch of them
    takes to stop at steady state, and whether each stopped run's result lies within 3 SE of the
    steady state (``stopped_within``, by windows of ``window`` steps)."""
    seeds = list(seeds)
    rows = []
    t_cold = t_warm = 0.0
    ts_cold = ts_warm = 0.0
    with tempfile.TemporaryDirectory() as td:
        dirs = {k: os.path.join(td, k) for k in ("cold", "warm", "ref")}
        for d in dirs.values():
            os.makedirs(d)
        for c0 in range(0, len(seeds), CHUNK // 4):
            chunk = seeds[c0:c0 + CHUNK // 4]
            ref = _models(chunk, dirs["ref"], periodic=True, steps=2 * steps, scale=scale)
            pred = net.predict(np.stack([features(q) for _, q in ref]))
            for (m, q), r, k in zip(ref, pred, chunk):
                m.set_start_temps(sensor_temps(r, q, m.n_sensors))
                m.set_options(seed=k + 1000003)
            api.batch_run([m for m, _ in ref], workers=workers)
            refs = [steady_reference(m.series(0)[0], window) for m, _ in ref]
            for m, _ in ref:
                m.close()
            cold = _models(chunk, dirs["cold"], periodic=True, steps=steps, scale=scale)
            warm = _models(chunk, dirs["warm"], periodic=True, steps=steps, scale=scale)
            for (m, q), r in zip(warm, pred):
                m.set_start_temps(sensor_temps(r, q, m.n_sensors))
            t0 = time.perf_counter()
            api.batch_run([m for m, _ in cold], workers=workers)
            t_cold += time.perf_counter() - t0
            t0 = time.perf_counter()
            api.batch_run([m for m, _ in warm], workers=workers)
            t_warm += time.perf_counter() - t0
            for (mc, _), (mw, _), ref_k in zip(cold, warm, refs):
                tc, tw = mc.series(0)[0], mw.series(0)[0]
                t_inf = ref_k[0]
                rows.append({"cold": onset_vs_reference(tc, *ref_k, window),
                             "warm": onset_vs_reference(tw, *ref_k, window),
                             "cold_detector": mc.steady_state(**stop_cold.detector())[0],
                             "warm_detector": mw.steady_state(**stop_warm.detector())[0],
                             "start_error_K": float(np.sqrt(np.mean((tw[:, 0] - t_inf) ** 2))),
                             "cold_start_error_K": float(np.sqrt(np.mean((tc[:, 0] - t_inf) ** 2)))})
            for ms, rule in ((cold, stop_cold), (warm, stop_warm)):
                for m, _ in ms:
                    m.set_steady_stop(check_every=rule.every, **rule.detector())
            t0 = time.perf_counter()
            api.batch_run([m for m, _ in cold], workers=workers)
            ts_cold += time.perf_counter() - t0
            t0 = time.perf_counter()
            api.batch_run([m for m, _ in warm], workers=workers)
            ts_warm += time.perf_counter() - t0
            for r, (mc, _), (mw, _), ref_k in zip(rows[len(rows) - len(chunk):], cold, warm, refs):
                r["cold_stop"] = mc.steps_run()
                r["warm_stop"] = mw.steps_run()
                r["cold_stop_ok"], r["cold_stop_mean_ok"] = stopped_within(mc, ref_k, window, stop_cold)
                r["warm_stop_ok"], r["warm_stop_mean_ok"] = stopped_within(mw, ref_k, window, stop_warm)
                mc.close()
                mw.close()

    def onsets(key):
        # a run that is not steady by its end counts as steady at its last step (a lower bound)
        return np.array([r[key] if r[key] >= 0 else steps for r in rows], dtype=float)

    cold_on, warm_on = onsets("cold"), onsets("warm")
    both = np.array([r["cold"] >= 0 and r["warm"] >= 0 for r in rows])
    return {
        "models": len(rows), "steps": steps, "window": window,
        "criterion": "first step after which every window mean of every sensor stays within the prediction bound of "
                     "the steady temperature of an independent run twice as long (its second half's window means: "
                     "Student's t at the 3-SE family-wise rate, 0.27 %, over all sensors and windows)",
        "mean_onset_steps_cold": float(cold_on.mean()), "mean_onset_steps_warm": float(warm_on.mean()),
        "steps_ratio_cold_over_warm": float(cold_on.mean() / max(warm_on.mean(), 1.0)),
        "median_ratio_where_both_steady": float(np.median(cold_on[both] / np.maximum(warm_on[both], window)))
        if both.any() else None,
        "steady_in_both": int(both.sum()),
        "never_steady_cold": int(sum(r["cold"] < 0 for r in rows)),
        "never_steady_warm": int(sum(r["warm"] < 0 for r in rows)),
        "stop_rule_cold": stop_cold.describe(), "stop_rule_warm": stop_warm.describe(),
        "mean_detector_onset_cold": float(onsets("cold_detector").mean()),
        "mean_detector_onset_warm": float(onsets("warm_detector").mean()),
        "rms_start_error_K_cold": float(np.sqrt(np.mean([r["cold_start_error_K"] ** 2 for r in rows]))),
        "rms_start_error_K_warm": float(np.sqrt(np.mean([r["start_error_K"] ** 2 for r in rows]))),
        "wall_s_cold_batch": t_cold, "wall_s_warm_batch": t_warm,
        "wall_s_cold_to_steady_stop": ts_cold, "wall_s_warm_to_steady_stop": ts_warm,
        "wall_ratio_cold_over_warm_to_steady_stop": ts_cold / max(ts_warm, 1e-9),
        "mean_steps_run_cold_to_steady_stop": float(np.mean([r["cold_stop"] for r in rows])),
        "mean_steps_run_warm_to_steady_stop": float(np.mean([r["warm_stop"] for r in rows])),
        "stopped_within_3se_cold": float(np.mean([r["cold_stop_ok"] for r in rows])),
        "stopped_within_3se_warm": float(np.mean([r["warm_stop_ok"] for r in rows])),
        "stopped_mean_within_3se_cold": float(np.mean([r["cold_stop_mean_ok"] for r in rows])),
        "stopped_mean_within_3se_warm": float(np.mean([r["warm_stop_mean_ok"] for r in rows])),
        "per_model": rows,
    }


def held_out(n: int, max_length: float = 2000.0) -> List[int]:
    """Seeds of ``n`` held-out rectangles (seeds from 50000, disjoint from the training seeds)
    no longer than ``max_length`` nm: diffusion time <= ~12 ns at 2 um, so a cold start settles
    within the evaluation runs and the two final states can be compared."""
    return [k for k in range(50000, 60000) if mg.random_bar_params(k)["length"] <= max_length][:n]


def summary(report: Dict) -> Dict:
    """The evaluation without its per-model rows."""
    return {k: v for k, v in report.items() if k != "per_model"}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2048, help="training rectangles")
    ap.add_argument("--test", type=int, default=64, help="held-out rectangles")
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--steps", type=int, default=3000, help="steps of the training runs")
    ap.add_argument("--eval-steps", type=int, default=6000, help="steps of the warm/cold evaluation runs")
    ap.add_argument("--scale", type=float, default=1.0, help="population scale of the generated models")
    ap.add_argument("--max-eval-length", type=float, default=2000.0, help="longest held-out rectangle (nm)")
    ap.add_argument("--stop-cold", type=StopRule.parse, default=STOP_COLD,
                    help="steady stop of the cold runs: window,batches,z,patience[,drift_z[,every]]")
    ap.add_argument("--stop-warm", type=StopRule.parse, default=STOP_WARM,
                    help="steady stop of the warm runs: window,batches,z,patience[,drift_z[,every]]")
    ap.add_argument("--out", default="")
    args = ap.parse_args(argv)
    t0 = time.perf_counter()
    X, Y = generate(range(10000, 10000 + args.train), steps=args.steps, scale=args.scale)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    net, loss = train(X, Y, epochs=args.epochs)
    t_train = time.perf_counter() - t0
    held = held_out(args.test, args.max_eval_length)
    Xt, Yt = generate(held, steps=args.steps, scale=args.scale)
    test_mse = float(np.mean((net.predict(Xt) - Yt) ** 2))
    report = {"train_models": args.train, "epochs": args.epochs, "final_train_loss": loss,
              "test_mse_scaled": test_mse, "test_rmse_K": float(np.sqrt(test_mse) * T_SCALE),
              "generate_s": t_gen, "train_s": t_train}
    report["warm_start"] = evaluate(net, held, steps=args.eval_steps, scale=args.scale, stop_cold=args.stop_cold,
                                    stop_warm=args.stop_warm)
    report["warm_start"]["held_out"] = f"rectangles of the training distribution up to {args.max_eval_length:g} nm long"
    text = json.dumps(report, indent=1)
    if args.out:
        with open(args.out, "w", encoding="utf-8") as f:
            f.write(text)
    print(json.dumps({k: v for k, v in report.items() if k != "warm_start"}))
    print(json.dumps({k: v for k, v in report["warm_start"].items() if k != "per_model"}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
