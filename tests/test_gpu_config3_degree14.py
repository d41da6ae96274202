"""GPU parity on config 3 at its full basis size: 4 species, order 4, degree
14, L 14 (24.8M AA functions, 6.33M items of the correlation schedule), with
the bimodal neighbour counts, against the FP64 CPU oracle, in every
precision form.

The spec is built once per session (about 40 s of host time) and a few
environments are evaluated: the CPU oracle needs about a second per
environment at this size."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

pytestmark = pytest.mark.gpu

TOL = {"fp64": dict(E=1e-12, G=1e-10), "fp32": dict(E=3e-5, G=1e-4), "fp32x2": dict(E=1e-6, G=1e-5),
       "fp32c": dict(E=1e-6, G=1e-5)}


@pytest.fixture(scope="module")
def case(oracle_mod):
    spec = symmetric_basis(4, 14, maxL=14, nspecies=4)
    c = random_coefficients(spec, seed=8)
    b = random_batch(4, 8, 80, nspecies=4, seed=13, bimodal=(0.6, (40, 80), (8, 20)))
    Eref, Gref = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr, b.species)
    return spec, c, b, Eref, Gref


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
def test_config3_degree14(case, prec):
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    build()
    spec, c, b, Eref, Gref = case
    ctx = L.Context(spec, prec)
    ctx.set_params(c)
    E, G = ctx.energy_forces(b.offsets, b.rr, b.species)
    ctx.close()
    scale = np.maximum(np.abs(Eref), np.sqrt(np.mean(Eref ** 2)))
    eE = float(np.max(np.abs(E - Eref) / scale))
    eG = float(np.max(np.abs(G - Gref)) / np.max(np.abs(Gref)))
    print(f"config 3 degree 14 {prec}: E relerr {eE:.3g}  G relerr {eG:.3g}")
    assert eE <= TOL[prec]["E"] and eG <= TOL[prec]["G"]
