"""One phonon simulation sharded over ranks, one GPU per rank.

psim's ModelSimulator (psim/src/modelSimulator.cpp:139-265) moves phonons that never interact:
each phonon's path depends only on its own random draws and the fixed geometry.  A job
therefore splits by phonons.  Each rank builds 1/world of the phonons (the energy per phonon
given to initPhononBuilders, psim/src/modelSimulator.cpp:43-85, is multiplied by world) and
draws from its own Philox streams (the rank selects the key's high word).  The ranks
exchange nothing while the step loop runs.  After a run, one all-reduce sums the sensors'
tallies, then the interpreter applies the job's energy per phonon to the sum.

The sum is exact and does not depend on the reduction order:
- energy tallies are int64 phonon counts;
- flux tallies are fixed-point integers times 2**-20, so every partial sum of doubles is
  exactly representable below 2**33 m/s per entry.

With per-rank work fixed (weak scaling), the job's energy per phonon is the single-rank
value divided by world.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional, Tuple

import numpy as np

_U64 = (1 << 64) - 1


def rank_seed(seed: int, rank: int) -> int:
    """Seed of rank `rank`: the high 32 bits pick the second Philox key word, so the ranks'
    streams are disjoint for any seed below 2**32."""
    if not 0 <= seed < (1 << 32):
        raise ValueError("seed must be below 2**32 when sharded")
    if not 0 <= rank < (1 << 32):
        raise ValueError("rank out of range")
    return (seed + (rank << 32)) & _U64


def rank_eff_energy(eff_energy: float, world: int) -> float:
    """Energy per phonon a rank builds with so that it creates 1/world of the job's phonons."""
    if world < 1:
        raise ValueError("world must be >= 1")
    return eff_energy * world


def job_eff_energy(rank_eff: float, world: int) -> float:
    """Energy per phonon of the summed tallies."""
    if world < 1:
        raise ValueError("world must be >= 1")
    return rank_eff / world


def combine_tallies(energy: np.ndarray, flux: np.ndarray, dist=None, group=None) -> Tuple[np.ndarray, np.ndarray]:
    """Sum the ranks' tallies (energy int64 [S][K], flux float64 [S][K][2]) on every rank.
    With no process group (one rank) the inputs are returned unchanged."""
    if dist is None or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return energy, flux
    import torch
    e = torch.from_numpy(np.ascontiguousarray(energy, dtype=np.int64))
    f = torch.from_numpy(np.ascontiguousarray(flux, dtype=np.float64))
    dist.all_reduce(e, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(f, op=dist.ReduceOp.SUM, group=group)
    return e.numpy(), f.numpy()


def reduce_max(value: float, dist=None, group=None) -> float:
    """Largest value over the ranks (the job's time is its slowest rank's)."""
    if dist is None or not dist.is_initialized():
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def reduce_sum(value: float, dist=None, group=None) -> float:
    if dist is None or not dist.is_initialized():
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return float(t.item())


@dataclass
class ShardResult:
    energy: np.ndarray      # summed over ranks
    flux: np.ndarray        # summed over ranks
    eff_energy: float       # energy per phonon of the summed tallies
    phonons: int            # this rank's phonons
    phonons_total: int      # over all ranks


def run_shard(sim, t_eq: float, eff_energy: float, cell_energy: np.ndarray, emit_energy: np.ndarray,
              sensor_init_temp: np.ndarray, seed: int, rank: int, world: int, precision: int = 0,
              stream: Optional[int] = None, dist=None, group=None) -> ShardResult:
    """One run of the ModelSimulator seam on this rank's share of a job whose energy per phonon
    is `eff_energy`.  `sim` is an api.Simulator (or anything with its reset /
    init_phonon_builders / run / tallies methods)."""
    sim.reset()
    n = sim.init_phonon_builders(t_eq, rank_eff_energy(eff_energy, world), cell_energy, emit_energy,
                                 sensor_init_temp, rank_seed(seed, rank))
    sim.run(t_eq, precision, stream)
    energy, flux = sim.tallies()
    energy, flux = combine_tallies(energy, flux, dist, group)
    total = int(reduce_sum(float(n), dist, group))
    return ShardResult(energy, flux, eff_energy, n, total)


def local_world(world: int, run_rank: Callable[[int], Tuple[np.ndarray, np.ndarray]]) -> Tuple[np.ndarray, np.ndarray]:
    """Runs the ranks of a `world`-rank job one after another in this process and sums their
    tallies (the same sum the all-reduce forms); used to check a sharded job on one device."""
    energy = flux = None
    for r in range(world):
        e, f = run_rank(r)
        energy = e.copy() if energy is None else energy + e
        flux = f.copy() if flux is None else flux + f
    return energy, flux
