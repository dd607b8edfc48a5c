"""The full-size workloads on the GPU, checked through properties that hold at any size.

Statistical parity with the reference is tested on small models, where the reference finishes
in seconds.  At the sizes the throughput numbers are quoted on, the checks are the ones that
need no reference run:
- the same seed gives identical tallies and population history;
- a phonon count that only absorption can change stays constant once nothing absorbs;
- temperatures stay inside the range the boundaries impose and fall from the hot end to the
  cold end;
- the population averages the per-step figure the phonon budget was sized for.
A run whose phonon buffer overflowed or whose shared-memory staging timed out fails with an
error, so a run that returns also proves neither happened."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the kinked three-arm structure at 1e7 phonons per step: psim's total budget is the per-step
# population times 5000 steps over the mean lifetime, 415 steps on this model
KINKED_BUDGET = 120_000_000


@pytest.fixture(scope="module")
def api(gpu):
    from psim_gb300 import api
    return api


def test_kinked_full_size(api, tmp_path):
    from psim_gb300 import modelgen as mg
    path = mg.write(mg.kinked(seed=0, num_phonons=KINKED_BUDGET, num_measurements=5000, sim_time=10.0, step_interval=50),
                    str(tmp_path / "kinked.json"))
    m = api.Model(path)
    m.run(seed=21)
    e1, f1 = m.tallies()
    pop1 = m.population()
    st = m.measurements()
    c = m.counters()
    m.run(seed=21)
    e2, f2 = m.tallies()
    assert np.array_equal(e1, e2) and np.array_equal(f1, f2)
    assert np.array_equal(pop1, m.population())

    # 1e7 phonons in flight on average over the run; the arms are still heating after 10 ns,
    # so the population is still growing at the end
    pop = pop1.astype(np.float64)
    assert 0.9e7 < pop.mean() < 1.1e7, pop.mean()
    assert pop[2500:2600].mean() < pop[-100:].mean()
    assert c["max_population"] == pop1.max()
    assert c["phonon_steps"] > 4e10
    assert c["event_limit_hits"] < 1e-6 * c["phonon_steps"]

    # emitters at 320 K (arm A), 280 K (arm B), 300 K (arm C): every sensor lies between them
    t = st[:, 0]
    assert np.all(np.isfinite(st))
    assert t.min() > 279.0 and t.max() < 321.0, (t.min(), t.max())
    # arm A's 66 x 2 sensors come first, from the hub outwards: its 320 K end is warmer than
    # the hub, and arm B's 280 K end cooler
    per_arm = 66 * 2
    arm_a, arm_b = t[:per_arm], t[per_arm:2 * per_arm]
    assert arm_a[-10:].mean() > arm_a[:10].mean() + 1.0
    assert arm_b[-10:].mean() < arm_b[:10].mean() - 1.0
    m.close()


def test_transient_plate_full_size(api, tmp_path):
    """4 um x 1 um plate, 64 x 16 cells, a 400 K pulse on a 200 nm strip of the left edge for
    20 ps, 2e7 phonons, 3000 steps of 1 ps."""
    from psim_gb300 import modelgen as mg
    path = mg.write(mg.plate(), str(tmp_path / "plate.json"))
    m = api.Model(path)
    m.run(seed=5)
    e, _ = m.tallies()
    temps, _ = m.series(0)
    c = m.counters()
    assert c["phonons"] > 1e7
    # the strip absorbs only while it emits: afterwards the net count never changes
    total = e.sum(axis=0)
    assert np.all(total[30:] == total[30])
    assert total[30] > 0
    # the pulse warms the plate near the strip first; far cells warm later and less
    nx, ny = 64, 16
    assert temps.shape[0] == nx * ny
    # sensors run column by column from the left edge: the first column holds the strip
    near = temps[:ny].mean(axis=0)
    far = temps[-ny:].mean(axis=0)
    assert near[:200].max() > far[:200].max()
    assert np.all(np.isfinite(temps))
    m.close()
