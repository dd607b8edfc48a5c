"""Steady-state detection: the GPU detector (psim_steady_state, psim_model_steady_state) against
the CPU restatement of its criterion, on synthetic tally series and on a real run."""
import numpy as np
import pytest

from conftest import model_path
from steady_np import model_onset, sensor_onsets


def relaxing_series(seed: int, S: int = 6, K: int = 1200, tau: float = 120.0, level: float = 400.0):
    """Per-step tallies that relax towards a plateau (as a cold start heats up), with Poisson
    noise on the counts and fixed-point flux."""
    rng = np.random.default_rng(seed)
    k = np.arange(K)
    energy = np.zeros((S, K), dtype=np.int64)
    flux = np.zeros((S, K, 2))
    for s in range(S):
        mean = level * (s + 1) / S * (1.0 - np.exp(-k / (tau * (1 + 0.3 * s))))
        energy[s] = rng.poisson(mean + 5.0)
        # flux spread like a sum over the counted phonons: ~ velocity x sqrt(count)
        flux[s, :, 0] = np.rint(rng.normal(mean * 800.0, 2400.0 * np.sqrt(mean + 5.0)) * 1048576.0) / 1048576.0
        flux[s, :, 1] = np.rint(rng.normal(0.0, 500.0, K) * 1048576.0) / 1048576.0
    return energy, flux


def test_restatement_finds_the_plateau():
    energy, flux = relaxing_series(1)
    per = sensor_onsets(energy, flux, 50, 5, 3.0, 3)
    onset = model_onset(per)
    # the slowest sensor relaxes with tau = 120 * 2.5 steps: it settles well inside the run
    assert 300 <= onset <= 1000, per
    # a series that keeps drifting is never steady
    drift = energy.copy()
    drift[2] += (np.arange(energy.shape[1]) * 2).astype(np.int64)
    assert model_onset(sensor_onsets(drift, flux, 50, 5, 3.0, 3)) == -1


def drifting_series(seed: int, rate: float = 0.3, K: int = 1500, level: float = 400.0):
    """Counts that keep rising by `rate` per step: 15 per 50-step window, about two standard
    errors of a window mean, so neighbouring windows agree while the drift over three does not."""
    rng = np.random.default_rng(seed)
    energy = rng.poisson(level + rate * np.arange(K), size=(1, K)).astype(np.int64)
    return energy, np.zeros((1, K, 2))


def test_restatement_sees_a_slow_drift():
    for seed in range(10):
        energy, flux = drifting_series(seed)
        assert model_onset(sensor_onsets(energy, flux, 50, 5, 3.0, 3)) == -1, seed
    # and a flat series with the same noise is steady from the start
    energy, flux = drifting_series(0, rate=0.0)
    assert model_onset(sensor_onsets(energy, flux, 50, 5, 3.0, 3)) == 0


def test_restatement_trend_test_sees_a_slower_drift():
    """A drift of 0.1 per step (5 per 50-step window, under one standard error of a window mean)
    stays within 3 combined standard errors of the anchor over 3 windows in most seeds, which are
    then called steady early; the trend test over the anchor and those windows rejects most of
    those early calls, and keeps a flat series with the same noise steady from the start."""
    slow = [model_onset(sensor_onsets(*drifting_series(seed, rate=0.1), 50, 5, 3.0, 3)) for seed in range(20)]
    trend = [model_onset(sensor_onsets(*drifting_series(seed, rate=0.1), 50, 5, 3.0, 3, drift_z=2.0)) for seed in range(20)]
    early = lambda onsets: sum(0 <= o < 400 for o in onsets)
    assert early(slow) >= 10 and early(trend) <= early(slow) // 2, (slow, trend)
    flat = [model_onset(sensor_onsets(*drifting_series(seed, rate=0.0), 50, 5, 3.0, 3, drift_z=2.0)) for seed in range(20)]
    assert sum(0 <= o <= 100 for o in flat) >= 15, flat


def test_arguments_are_checked(built):
    from psim_gb300 import api
    e = np.zeros((2, 100), dtype=np.int64)
    f = np.zeros((2, 100, 2))
    for kw in ({"window": 1, "batches": 1}, {"window": 50, "batches": 3}, {"batches": 1}, {"z": 0.0}, {"patience": 0},
               {"drift_z": -1.0}, {"drift_z": float("nan")}):
        with pytest.raises(api.PsimError) as exc:
            api.steady_state(e, f, **kw)
        assert exc.value.code == api.PSIM_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("seed,window,batches,patience", [(1, 50, 5, 3), (2, 40, 4, 2), (3, 64, 8, 4), (4, 25, 5, 5),
                                                         (5, 100, 2, 3)])
def test_gpu_matches_restatement_on_synthetic_series(gpu, seed, window, batches, patience):
    from psim_gb300 import api
    energy, flux = relaxing_series(seed)
    onset, per = api.steady_state(energy, flux, window=window, batches=batches, z=3.0, patience=patience)
    want = sensor_onsets(energy, flux, window, batches, 3.0, patience)
    assert np.array_equal(per, want)
    assert onset == model_onset(want)


@pytest.mark.gpu
@pytest.mark.parametrize("seed,rate,patience,drift_z", [(0, 0.3, 3, 0.0), (1, 0.16, 3, 0.0), (2, 0.0, 3, 0.0), (3, 0.1, 5, 2.0),
                                                        (4, 0.1, 5, 2.0), (5, 0.0, 5, 2.0), (6, 0.05, 8, 2.5), (7, 0.1, 3, 2.0)])
def test_gpu_matches_restatement_on_drifting_series(gpu, seed, rate, patience, drift_z):
    from psim_gb300 import api
    energy, flux = drifting_series(seed, rate)
    onset, per = api.steady_state(energy, flux, window=50, batches=5, z=3.0, patience=patience, drift_z=drift_z)
    want = sensor_onsets(energy, flux, 50, 5, 3.0, patience, drift_z)
    assert np.array_equal(per, want) and onset == model_onset(want)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 3])
def test_gpu_matches_restatement_with_the_trend_test(gpu, seed):
    from psim_gb300 import api
    energy, flux = relaxing_series(seed)
    onset, per = api.steady_state(energy, flux, window=50, batches=5, z=3.0, patience=4, drift_z=2.0)
    want = sensor_onsets(energy, flux, 50, 5, 3.0, 4, 2.0)
    assert np.array_equal(per, want) and onset == model_onset(want)


@pytest.mark.gpu
def test_gpu_edge_cases(gpu):
    from psim_gb300 import api
    energy, flux = relaxing_series(5)
    drift = energy.copy()
    drift[0] += (np.arange(energy.shape[1]) * 3).astype(np.int64)
    onset, per = api.steady_state(drift, flux, window=50, batches=5)
    assert onset == -1 and per[0] == -1 and np.all(per[1:] >= 0)
    # constant tallies agree from the first window; too few windows for the patience: never
    const_e = np.full((3, 400), 7, dtype=np.int64)
    const_f = np.zeros((3, 400, 2))
    assert api.steady_state(const_e, const_f, window=50, batches=5, patience=3)[0] == 0
    assert api.steady_state(const_e[:, :150], const_f[:, :150], window=50, batches=5, patience=3)[0] == -1


@pytest.mark.gpu
def test_model_run_detector_matches_restatement(gpu):
    """The detector on a periodic run's own device tallies equals the restatement on the same
    tallies read back."""
    from psim_gb300 import api
    m = api.Model(model_path("kinked_small"))
    m.run(seed=3)
    energy, flux = m.tallies()
    for window, batches, patience in ((20, 4, 3), (40, 5, 2), (50, 5, 3)):
        onset, per = m.steady_state(window=window, batches=batches, z=3.0, patience=patience)
        want = sensor_onsets(energy, flux, window, batches, 3.0, patience)
        assert np.array_equal(per, want)
        assert onset == model_onset(want)


@pytest.mark.gpu
def test_run_stops_at_steady_state(gpu):
    """A periodic run with the stop on ends at a check where the recorded steps are steady; its
    tallies are the first steps of the same run without the stop (the chunked launches change
    nothing), and the model reports that many recorded steps."""
    from psim_gb300 import api
    full = api.Model(model_path("kinked_small"))
    full.run(seed=7)
    e_full, f_full = full.tallies()
    n = full.n_steps
    m = api.Model(model_path("kinked_small"))
    m.set_steady_stop(window=20, batches=4, z=3.0, patience=3, check_every=40)
    m.run(seed=7)
    k = m.steps_run()
    assert 80 <= k <= n and k % 40 == 0 or k == n
    assert m.n_recorded == k
    e, f = m.tallies()
    assert e.shape == (m.n_sensors, k)
    assert np.array_equal(e, e_full[:, :k]) and np.array_equal(f, f_full[:, :k])
    temps, fluxes = m.series(0)
    assert temps.shape == (m.n_sensors, k)
    if k < n:
        assert model_onset(sensor_onsets(e, f, 20, 4, 3.0, 3)) >= 0
        assert model_onset(sensor_onsets(e[:, :k - 40], f[:, :k - 40], 20, 4, 3.0, 3)) == -1 or k - 40 < 80
    # off again: the whole run
    m.set_steady_stop(enable=False)
    m.run(seed=7)
    assert m.steps_run() == n and m.n_recorded == n


@pytest.mark.gpu
def test_steady_stop_needs_every_step_recorded(gpu):
    from psim_gb300 import api
    m = api.Model(model_path("bar_ss"))
    m.set_steady_stop(window=10, batches=5)
    with pytest.raises(api.PsimError) as exc:
        m.run(seed=1)
    assert exc.value.code == api.PSIM_ERR_INVALID
