"""Spec-bundle round trip: a saved and re-loaded model is bit-identical and
evaluates to the same energies (the role write_dict/read_dict play for
LinearACEModel in the reference, src/linearmodel.jl:80-93)."""
import json

import numpy as np
import pytest

from ace_gb300 import bundle
from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis


def test_round_trip(tmp_path, oracle_mod):
    spec = symmetric_basis(3, 6, maxL=6, nspecies=2)
    c = random_coefficients(spec, seed=4)
    p = tmp_path / "model.json"
    bundle.save(str(p), spec, c)
    spec2, c2 = bundle.load(str(p))
    assert np.array_equal(c, c2)
    for f in ("orders", "iAA2iA", "Bdeg", "Bclass"):
        assert np.array_equal(getattr(spec, f), getattr(spec2, f))
    for f in ("mu", "n", "l", "m"):
        assert np.array_equal(getattr(spec.aspec, f), getattr(spec2.aspec, f))
    assert (spec.U != spec2.U).nnz == 0
    assert np.array_equal(spec.radial.J.A, spec2.radial.J.A)
    b = random_batch(5, 10, 10, nspecies=2, seed=1)
    E1 = oracle_mod.Oracle(spec, c).evaluate(b.offsets, b.rr, b.species)
    E2 = oracle_mod.Oracle(spec2, c2).evaluate(b.offsets, b.rr, b.species)
    assert np.array_equal(E1, E2)


def test_rejects_foreign_or_newer(tmp_path):
    spec = symmetric_basis(2, 4, maxL=4)
    d = bundle.to_dict(spec)
    d["version"] = bundle.VERSION + 1
    with pytest.raises(ValueError):
        bundle.from_dict(d)
    with pytest.raises(ValueError):
        bundle.from_dict({"format": "something-else"})
