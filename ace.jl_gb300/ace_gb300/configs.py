"""Seeded synthetic workloads (the five benchmark configurations).

Neighbour directions are normalised 3-vectors of N(0,1) draws, as ACE.jl's
``rand_sphere`` makes them (``src/utils/auxiliary.jl:81-84``); radii are
uniform on [rlo, rhi].  Environments are stored CSR: ``offsets[e]:offsets[e+1]``
indexes the neighbours of environment e in the (nNbr, 3) array ``rr``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Batch:
    offsets: np.ndarray      # (nEnv+1,) int64
    rr: np.ndarray           # (nNbr, 3) float64, neighbour positions relative to the centre
    species: np.ndarray | None  # (nNbr,) int32 or None

    @property
    def nenv(self):
        return len(self.offsets) - 1

    @property
    def nnbr(self):
        return len(self.rr)

    def env(self, e):
        o0, o1 = self.offsets[e], self.offsets[e + 1]
        return self.rr[o0:o1], (None if self.species is None else self.species[o0:o1])


def random_batch(nenv: int, jlo: int, jhi: int, rlo: float = 0.8, rhi: float = 5.0,
                 nspecies: int = 1, seed: int = 0, bimodal=None) -> Batch:
    """J ~ U{jlo..jhi}; with ``bimodal=(p, (lo1, hi1), (lo2, hi2))`` J is drawn
    from U{lo1..hi1} with probability p and U{lo2..hi2} otherwise."""
    rng = np.random.default_rng(seed)
    if bimodal is None:
        J = rng.integers(jlo, jhi + 1, size=nenv)
    else:
        p, (a1, b1), (a2, b2) = bimodal
        pick = rng.random(nenv) < p
        J = np.where(pick, rng.integers(a1, b1 + 1, size=nenv), rng.integers(a2, b2 + 1, size=nenv))
    offsets = np.zeros(nenv + 1, dtype=np.int64)
    np.cumsum(J, out=offsets[1:])
    n = int(offsets[-1])
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rlo + (rhi - rlo) * rng.random(n)
    rr = d * r[:, None]
    species = rng.integers(0, nspecies, size=n).astype(np.int32) if nspecies > 1 else None
    return Batch(offsets, rr, species)


# The benchmark configurations: (maxorder, maxdeg, maxL, nspecies) and workload.
CONFIGS = {
    1: dict(basis=dict(maxorder=3, maxdeg=8, maxL=6, nspecies=1),
            work=dict(nenv=1000, jlo=12, jhi=24)),
    2: dict(basis=dict(maxorder=4, maxdeg=12, maxL=12, nspecies=1),
            work=dict(nenv=100_000, jlo=20, jhi=60)),
    3: dict(basis=dict(maxorder=4, maxdeg=14, maxL=14, nspecies=4),
            work=dict(nenv=250_000, jlo=8, jhi=80, nspecies=4,
                      bimodal=(0.6, (40, 80), (8, 20)))),
    4: dict(basis=dict(maxorder=5, maxdeg=16, maxL=16, nspecies=1),
            work=dict(nenv=500_000, jlo=30, jhi=30)),
}
