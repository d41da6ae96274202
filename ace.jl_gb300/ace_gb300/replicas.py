"""Replica (data-parallel) helpers for several GPUs.

Environments are independent, so N GPUs evaluate N disjoint batches with no
data-path collective.  A batch that is split over ranks is cut into
contiguous CSR ranges of (nearly) equal estimated cost; the cost model is
per neighbour (1p basis, A accumulation, force contraction) plus per
environment (the correlation products), both proportional to the spec's
sizes.  The only collectives are the optional sum of energies (one FP64
scalar) and the max over ranks of a timing.
"""
from __future__ import annotations

import numpy as np

from .configs import Batch


def env_costs(offsets: np.ndarray, cost_per_nbr: float, cost_per_env: float) -> np.ndarray:
    return np.diff(np.asarray(offsets, dtype=np.int64)) * cost_per_nbr + cost_per_env


def partition(offsets: np.ndarray, world: int, cost_per_nbr: float = 1.0, cost_per_env: float = 0.0) -> np.ndarray:
    """Environment boundaries (world + 1,) of contiguous ranges with nearly
    equal summed cost."""
    c = env_costs(offsets, cost_per_nbr, cost_per_env)
    cum = np.concatenate([[0.0], np.cumsum(c)])
    targets = cum[-1] * np.arange(world + 1) / world
    b = np.searchsorted(cum, targets, side="left")
    b[0], b[-1] = 0, len(c)
    return np.maximum.accumulate(b)


def spec_costs(spec) -> tuple[float, float]:
    """(per neighbour, per environment) cost weights of a spec for partition."""
    nY = (spec.Leff + 1) ** 2
    per_nbr = 10.0 * len(spec.radial.J.A) + 36.0 * nY + 38.0 * spec.nA
    per_env = 0.0
    for k, n in spec.info.get("nAA_by_order", {}).items():
        per_env += n * (6.0 * max(k - 1, 0) + 2.0 + 18.0 * max(k - 2, 0) + 6.0 + 4.0 * k)
    return per_nbr, per_env


def local_batch(b: Batch, rank: int, world: int, cost_per_nbr: float = 1.0, cost_per_env: float = 0.0) -> Batch:
    """This rank's contiguous share of the batch."""
    bnd = partition(b.offsets, world, cost_per_nbr, cost_per_env)
    e0, e1 = int(bnd[rank]), int(bnd[rank + 1])
    o0, o1 = int(b.offsets[e0]), int(b.offsets[e1])
    return Batch(b.offsets[e0:e1 + 1] - o0, b.rr[o0:o1], None if b.species is None else b.species[o0:o1])


def total_energy(E_local: np.ndarray, group=None) -> float:
    """Sum of all ranks' site energies (one FP64 all-reduce)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(np.sum(E_local))], dtype=torch.float64)
    if dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return float(t.item())


def max_over_ranks(x: float, group=None, device=None) -> float:
    """max over ranks of a per-rank number (timings are reported as the max)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
