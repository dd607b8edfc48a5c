"""The sharded (one GPU per rank, weak scaling) job's host logic with world_size 2 over gloo on
CPU: per-rank seeds and phonon shares, and the one exchange, an exact sum of the tallies."""
import os
import socket
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests"))
import shard_worker  # noqa: E402

from psim_gb300 import shard  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.fixture(scope="module")
def two_ranks():
    pytest.importorskip("torch")
    out = tempfile.mkdtemp(prefix="psim_shard_")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                   CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, os.path.join(ROOT, "tests", "shard_worker.py"), out], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    logs = []
    for p in procs:
        try:
            o, _ = p.communicate(timeout=240)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            pytest.fail("gloo ranks did not finish")
        logs.append(o.decode(errors="replace"))
    for p, log in zip(procs, logs):
        assert p.returncode == 0, log[-2000:]
    return [np.load(os.path.join(out, f"rank{r}.npz")) for r in range(2)]


def test_tally_sum_is_exact_on_every_rank(two_ranks):
    e0, f0 = shard_worker.synthetic(0)
    e1, f1 = shard_worker.synthetic(1)
    for res in two_ranks:
        assert res["energy"].dtype == np.int64
        assert np.array_equal(res["energy"], e0 + e1)
        # fixed-point flux: the double sum is exact, whatever order the ranks add in
        assert np.array_equal(res["flux"], f0 + f1)
        assert np.array_equal(res["flux"], f1 + f0)
        assert float(res["maxv"]) == 13.0


def test_run_shard_splits_phonons_and_streams(two_ranks):
    r0, r1 = two_ranks
    # each rank builds with world x the job's energy per phonon: 1/world of the phonons
    assert float(r0["init_eff"]) == float(r1["init_eff"]) == 2 * 2.5e-20
    assert float(r0["eff"]) == 2.5e-20
    # disjoint random streams: the rank selects the seed's high word
    assert int(r0["init_seed"]) == 11 and int(r1["init_seed"]) == 11 + (1 << 32)
    assert list(r0["order"]) == ["reset", "init", "run"]
    assert int(r0["total"]) == int(r0["n"]) + int(r1["n"]) == 2001
    # both ranks hold the same summed tallies, equal to the ranks' own tallies added locally
    want = shard.local_world(2, lambda r: _fake_tallies(shard.rank_seed(11, r)))
    for res in two_ranks:
        assert np.array_equal(res["shard_energy"], want[0])
        assert np.array_equal(res["shard_flux"], want[1])


def _fake_tallies(seed):
    sim = shard_worker.FakeSimulator()
    sim.init_phonon_builders(0.0, 1.0, None, None, None, seed)
    return sim.tallies()


def test_single_rank_is_unchanged():
    e, f = shard_worker.synthetic(3)
    se, sf = shard.combine_tallies(e, f, None)
    assert se is e and sf is f
    assert shard.rank_seed(5, 0) == 5
    assert shard.rank_eff_energy(3.0, 1) == 3.0 and shard.job_eff_energy(8.0, 4) == 2.0
    with pytest.raises(ValueError):
        shard.rank_seed(1 << 32, 1)
    with pytest.raises(ValueError):
        shard.rank_eff_energy(1.0, 0)
