"""One rank of the sharded-job checks in test_shard.py (gloo, CPU).  Writes what it saw to
<out>/rank<r>.npz.  Run with RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT set."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import torch.distributed as dist  # noqa: E402

from psim_gb300 import shard  # noqa: E402

S, K = 7, 33


def synthetic(rank: int):
    rng = np.random.default_rng(1000 + rank)
    energy = rng.integers(-50, 50, size=(S, K), dtype=np.int64)
    # fixed-point flux tallies as the engine returns them: integers times 2**-20, up to ~2**32 m/s
    flux = rng.integers(-(1 << 52), 1 << 52, size=(S, K, 2), dtype=np.int64).astype(np.float64) * 2.0**-20
    return energy, flux


class FakeSimulator:
    """Stands in for api.Simulator: tallies are a function of the seed and energy per phonon."""

    def __init__(self):
        self.calls = []

    def reset(self):
        self.calls.append(("reset",))

    def init_phonon_builders(self, t_eq, eff, cell, emit, init_t, seed):
        self.calls.append(("init", t_eq, eff, seed))
        self.seed, self.eff = seed, eff
        return int(1000 + (seed >> 32))

    def run(self, t_eq, precision, stream):
        self.calls.append(("run", t_eq, precision))

    def tallies(self):
        rng = np.random.default_rng([self.seed & 0xFFFFFFFF, self.seed >> 32])
        return rng.integers(0, 9, size=(S, K), dtype=np.int64), rng.integers(-99, 99, size=(S, K, 2)).astype(np.float64)


def main(out_dir: str):
    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    dist.init_process_group("gloo", rank=rank, world_size=world)
    energy, flux = synthetic(rank)
    se, sf = shard.combine_tallies(energy, flux, dist)
    mx = shard.reduce_max(float(10 * rank + 3), dist)
    sim = FakeSimulator()
    res = shard.run_shard(sim, 300.0, 2.5e-20, np.zeros(3), np.zeros(2), np.zeros(S), seed=11, rank=rank, world=world,
                          precision=0, stream=None, dist=dist)
    init = [c for c in sim.calls if c[0] == "init"][0]
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), energy=se, flux=sf, maxv=mx, shard_energy=res.energy,
             shard_flux=res.flux, eff=res.eff_energy, n=res.phonons, total=res.phonons_total, init_eff=init[2],
             init_seed=np.uint64(init[3]), order=np.array([c[0] for c in sim.calls]))
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1])
