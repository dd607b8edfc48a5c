"""The learned warm start: starting a run from good temperatures shortens the burn-in and ends
on the cold start's steady state; the surrogate pipeline (Monte Carlo training fields, the GPU
network, warm-started evaluation) runs end to end."""
import numpy as np
import pytest


def test_raster_round_trip():
    from psim_gb300 import modelgen as mg
    from psim_gb300 import surrogate as sg
    q = mg.random_bar_params(7)
    t = np.linspace(290.0, 310.0, q["cells"])
    back = sg.sensor_temps(sg.raster(t, q), q, q["cells"])
    # one raster column spans at most L/32: a linear profile is read back to half a column
    assert np.abs(back - t).max() <= 20.0 / 32 + 1e-6
    assert sg.features(q).shape == (sg.FEATURES,)


def test_workload_draws():
    """The random rectangles follow their stated distribution, and the held-out set is short
    enough to settle and disjoint from the training seeds."""
    from psim_gb300 import modelgen as mg
    from psim_gb300 import surrogate as sg
    qs = [mg.random_bar_params(k) for k in range(2000)]
    for q in qs:
        assert 200.0 <= q["length"] <= 5000.0 and 50.0 <= q["width"] <= 500.0 and 4 <= q["cells"] <= 200
        assert 1e4 <= q["per_step"] <= 1e6 and 280.0 <= q["t_left"] <= 320.0 and 280.0 <= q["t_right"] <= 320.0
        assert 0.0 <= q["spec"] <= 1.0
    # log-uniform populations: about half of the draws below 1e5
    assert 0.45 < np.mean([q["per_step"] < 1e5 for q in qs]) < 0.55
    held = sg.held_out(64)
    assert len(held) == 64 and len(set(held)) == 64 and min(held) >= 50000
    assert all(mg.random_bar_params(k)["length"] <= 2000.0 for k in held)
    assert held == sg.held_out(64)


def test_onset_against_a_reference():
    from psim_gb300 import surrogate as sg
    rng = np.random.default_rng(3)
    K, W = 2000, 50
    t_inf = np.array([300.0, 305.0, 310.0])
    steady = t_inf[:, None] + rng.normal(0.0, 0.5, size=(3, K))
    ref = sg.steady_reference(steady, W)
    assert np.allclose(ref[0], t_inf, atol=0.05) and np.all(ref[1] < 0.2) and ref[2] == 19
    # relaxing from 290 K with a 200-step time constant: steady once the gap is within tolerance
    approach = steady - (t_inf - 290.0)[:, None] * np.exp(-np.arange(K) / 200.0)
    on = sg.onset_vs_reference(approach, *ref, W)
    assert 500 <= on <= 1500 and on % W == 0
    assert sg.onset_vs_reference(steady + 0.0, *ref, W) == 0
    # still off by a kelvin at the end: never
    assert sg.onset_vs_reference(steady + 1.0, *ref, W) == -1


class _StoppedRun:
    """A run stopped by the detector, as stopped_within sees it: its recorded temperatures and
    the detector's onset."""

    def __init__(self, temps, onset):
        self.temps, self.onset = temps, onset

    def series(self, run=0):
        return self.temps, None

    def steady_state(self, **kw):
        return self.onset, None


def test_stopped_run_accuracy():
    from psim_gb300 import surrogate as sg
    RULE = sg.StopRule(50, 5, 3.0, 3)
    rng = np.random.default_rng(5)
    t_inf = np.array([300.0, 305.0, 310.0])
    ref = sg.steady_reference(t_inf[:, None] + rng.normal(0.0, 0.5, size=(3, 4000)), 50)
    steady = t_inf[:, None] + rng.normal(0.0, 0.5, size=(3, 600))
    assert sg.stopped_within(_StoppedRun(steady, 200), ref, 50, RULE) == (True, True)
    # stopped while still a kelvin away: both standards miss
    assert sg.stopped_within(_StoppedRun(steady - 1.0, 200), ref, 50, RULE) == (False, False)
    # a tenth of a kelvin off: inside one window's bound, outside the bound of a 400-step mean
    assert sg.stopped_within(_StoppedRun(steady - 0.1, 200), ref, 50, RULE) == (True, False)
    # no onset: the last window is taken
    assert sg.stopped_within(_StoppedRun(steady, -1), ref, 50, RULE) == (True, True)


def test_stop_rules():
    from psim_gb300 import surrogate as sg
    r = sg.StopRule.parse("200,10,3.5,2")
    assert r == sg.StopRule(200, 10, 3.5, 2, 0.0, 0)
    assert sg.StopRule.parse("50,5,3,3,2.5,50") == sg.StopRule(50, 5, 3.0, 3, 2.5, 50)
    assert r.detector() == {"window": 200, "batches": 10, "z": 3.5, "patience": 2, "drift_z": 0.0}
    with pytest.raises(ValueError):
        sg.StopRule.parse("200,10,3.5")
    # checked every patience + 1 windows unless told otherwise
    assert r.describe().endswith("checked every 600 steps")
    assert sg.STOP_WARM.describe().endswith("checked every 50 steps")
    # each rule's shortest stop fits the evaluation runs
    for rule in (sg.STOP_COLD, sg.STOP_WARM):
        assert (rule.patience + 1) * rule.window <= 6000 and rule.window % rule.batches == 0


@pytest.mark.gpu
def test_warm_start_reaches_the_steady_state_sooner(gpu, tmp_path):
    """A 300 nm bar (diffusion time ~0.3 ns) run for 5 ns: cold, then warm from the cold run's
    second-half temperatures, and a third warm run with its own seed as the reference.  Both
    starts end on the reference's steady state; the warm one starts on it."""
    from psim_gb300 import api
    from psim_gb300 import modelgen as mg
    from psim_gb300 import surrogate as sg
    path = mg.write(mg.bar(num_cells=10, length=300.0, width=100.0, t_left=315.0, t_right=285.0, num_measurements=1000,
                           sim_time=5.0, num_phonons=400000, sim_type=1, step_interval=50), str(tmp_path / "short.json"))
    cold = api.Model(path)
    cold.run(seed=11)
    tc = cold.series(0)[0]
    start = tc[:, tc.shape[1] // 2:].mean(axis=1)
    runs = []
    for seed in (12, 13):
        warm = api.Model(path)
        warm.set_start_temps(start)
        assert np.allclose(warm.start_temps(), start)
        warm.run(seed=seed)
        runs.append(warm.series(0)[0])
    # the first recorded temperature is the start temperature
    assert np.allclose(runs[0][:, 0], start)
    ref = sg.steady_reference(runs[1], 20)
    assert sg.onset_vs_reference(tc, *ref, 20) >= 0
    assert sg.onset_vs_reference(runs[0], *ref, 20) >= 0
    # the first 20-step window: the cold start is kelvins off, the warm one within noise
    err_cold = np.abs(tc[:, :20].mean(axis=1) - ref[0]).mean()
    err_warm = np.abs(runs[0][:, :20].mean(axis=1) - ref[0]).mean()
    assert err_warm < 3 * ref[1].mean() and err_warm < err_cold / 5, (err_warm, err_cold)


@pytest.mark.gpu
def test_surrogate_pipeline_end_to_end(gpu):
    from psim_gb300 import surrogate as sg
    X, Y = sg.generate(range(20000, 20032), steps=600, scale=0.1)
    assert X.shape == (32, sg.FEATURES) and Y.shape == (32, sg.RASTER * sg.RASTER)
    net, loss = sg.train(X, Y, epochs=50, batch=16)
    assert np.isfinite(loss)
    rep = sg.evaluate(net, range(20100, 20104), steps=600, scale=0.1, window=50)
    assert rep["models"] == 4 and rep["steady_in_both"] <= 4
    assert {"mean_onset_steps_cold", "mean_onset_steps_warm", "mean_detector_onset_warm"} <= set(rep)
    # the steady stop ends a run no later than its full length
    assert all(0 < r["cold_stop"] <= 600 and 0 < r["warm_stop"] <= 600 for r in rep["per_model"])
    # what the network gains over the plain start: even this small one, trained on 32 noisy
    # fields, starts the held-out bars closer to their steady temperatures than T_ref does
    print({k: rep[k] for k in ("rms_start_error_K_cold", "rms_start_error_K_warm", "mean_onset_steps_cold",
                               "mean_onset_steps_warm")})
    assert rep["rms_start_error_K_warm"] < rep["rms_start_error_K_cold"]
