"""Many models on one GPU (psim_batch_run / psim_batch_autotune): each model's results equal
those of the same model run alone, whatever runs beside it, the stream or the grid, in the
batched launches fed by a device work queue as on worker threads."""
import numpy as np
import pytest

from conftest import model_path


def test_batch_arguments_are_checked(built):
    from psim_gb300 import api
    m = api.Model(model_path("bar_ss"))
    with pytest.raises(api.PsimError) as e:
        api.batch_run([m, m], workers=2)
    assert e.value.code == api.PSIM_ERR_INVALID
    with pytest.raises(api.PsimError) as e:
        api.batch_run([m], workers=0)
    assert e.value.code == api.PSIM_ERR_INVALID


def test_batch_fails_loudly_without_a_device(built):
    from psim_gb300 import api
    if api.device_count() > 0:
        pytest.skip("a CUDA device is present")
    m = api.Model(model_path("bar_ss"))
    with pytest.raises(api.PsimError) as e:
        api.batch_run([m], workers=1)
    assert e.value.code == api.PSIM_ERR_CUDA


CASES = [("bar_ss", 3, 0), ("kinked_small", 4, 0), ("plate_small", 5, 0), ("bar_periodic", 6, 0),
         ("bar_full", 7, 0), ("bar_phasor", 8, 0), ("kinked_small", 9, 1), ("bar_ss", 10, 0), ("bar_runs", 11, 0),
         ("kinked_small", 12, 0), ("plate_small", 13, 0)]


@pytest.mark.gpu
@pytest.mark.parametrize("workers,max_blocks,queue,per_thread", [(3, 8, False, 16), (8, 0, False, 16), (4, 0, True, 16),
                                                                 (8, 0, True, 1), (2, 0, True, 64)])
def test_batch_results_equal_single_runs(gpu, workers, max_blocks, queue, per_thread):
    """Models of several step counts, modes and precisions: steady state, full, periodic,
    transient, phasor, three averaged runs, and an FP64 model (which runs on its own).  With the
    device queue the FP32 models of each step count share launches; work items of 1, 16 and 64
    phonons per thread cut the models' phonons at different places."""
    from psim_gb300 import api
    alone = []
    for name, seed, prec in CASES:
        m = api.Model(model_path(name))
        m.run(seed=seed, precision=prec)
        alone.append((m.tallies(), m.measurements()))
    models = [api.Model(model_path(name)).set_options(seed=seed, precision=prec) for name, seed, prec in CASES]
    secs, steps = api.batch_run(models, workers=workers, max_blocks=max_blocks, device_queue=queue, per_thread=per_thread)
    assert secs > 0 and steps > 0
    total = 0
    for m, ((e, f), st) in zip(models, alone):
        e2, f2 = m.tallies()
        assert np.array_equal(e, e2) and np.array_equal(f, f2)
        assert np.array_equal(st, m.measurements())
        total += m.counters()["phonon_steps"]
    assert total == steps


@pytest.mark.gpu
def test_batch_autotune_picks_valid_options(gpu):
    from psim_gb300 import api
    models = [api.Model(model_path("bar_periodic")).set_options(seed=s) for s in range(1, 5)]
    opt, rate = api.batch_autotune(models, sample=4)
    assert opt.workers in (4, 8, 16, 32) and rate > 0
    assert (opt.device_queue == 1 and opt.per_thread in (4, 8, 16, 32)) or (opt.device_queue == 0 and opt.max_blocks >= 1)
    secs, steps = api.batch_run(models, workers=opt.workers, max_blocks=opt.max_blocks, device_queue=bool(opt.device_queue),
                                per_thread=opt.per_thread)
    assert steps > 0
