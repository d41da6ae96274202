"""Replicas on several ranks (CPU, gloo, world sizes 2 and 4): cost-balanced
contiguous partitions of a batch, the FP64 energy sum over ranks and the
max-over-ranks timing, with the oracle evaluating each rank's share."""
import os
import socket

import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.replicas import local_batch, partition, spec_costs


def test_partition_balances_cost():
    b = random_batch(1001, 8, 80, seed=3, bimodal=(0.6, (40, 80), (8, 20)))
    for world in (1, 2, 3, 8):
        bnd = partition(b.offsets, world, 5.0, 100.0)
        assert bnd[0] == 0 and bnd[-1] == b.nenv and np.all(np.diff(bnd) >= 0)
        cost = np.diff(b.offsets) * 5.0 + 100.0
        parts = [cost[bnd[r]:bnd[r + 1]].sum() for r in range(world)]
        assert max(parts) - min(parts) <= 2 * cost.max()
    # empty and tiny batches
    assert partition(np.array([0]), 2).tolist() == [0, 0, 0]
    assert partition(np.array([0, 3]), 4)[-1] == 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from ace_gb300.replicas import max_over_ranks, total_energy
    from ace_gb300.spec import random_coefficients, symmetric_basis
    spec = symmetric_basis(3, 6, maxL=6)
    c = random_coefficients(spec, seed=1)
    b = random_batch(300, 6, 20, seed=2)
    lb = local_batch(b, rank, world, *spec_costs(spec))
    E = oracle.Oracle(spec, c).evaluate(lb.offsets, lb.rr, nthreads=1)
    tot = total_energy(E)
    tmax = max_over_ranks(float(rank + 1))
    out.put((rank, tot, tmax, len(E)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
def test_replicas_over_ranks(oracle_mod, world):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from ace_gb300.spec import random_coefficients, symmetric_basis
    spec = symmetric_basis(3, 6, maxL=6)
    b = random_batch(300, 6, 20, seed=2)
    Eall = oracle_mod.Oracle(spec, random_coefficients(spec, seed=1)).evaluate(b.offsets, b.rr)
    for rank, tot, tmax, n in res:
        assert abs(tot - Eall.sum()) <= 1e-10 * max(1.0, abs(Eall.sum()))
        assert tmax == float(world)
    assert sum(r[3] for r in res) == b.nenv
