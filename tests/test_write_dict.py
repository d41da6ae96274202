"""The write_dict importer (ace_gb300/writedict.py): ACE.jl model dictionaries
(src/linearmodel.jl:80-93, src/symmbasis.jl:50-61, src/pibasis.jl:235-252,
src/product_1pbasis.jl:57-66, src/polynomials/orthpolys.jl:119-140) into the
spec this library evaluates.

* a small model written out by hand in that shape: its basis functions are
  recomputed from the oracle's A and checked, and its energies are rotation
  invariant;
* a built spec written to that shape, through JSON and back: the same index
  lists, U and coefficients, and the same oracle energies bit for bit;
* a four-species spec with the categorical component first;
* on the GPU: a context created from the imported spec against the oracle."""
import json

import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.radial import rn_basis
from ace_gb300.spec import random_coefficients, symmetric_basis
from ace_gb300.writedict import from_write_dict, to_write_dict

S3 = 1.0 / np.sqrt(3.0)


def hand_written_model():
    """Rn with 2 polynomials, Ylm up to l = 1; A = (n,l,m) in
    [(1,0,0), (2,0,0), (1,1,-1), (1,1,0), (1,1,1)]; AA functions (rows stored
    descending, 1-based, 0-padded): A1, A2, A1 A1, A2 A1, A2 A2, A5 A3, A4 A4;
    B1..B5 are the first five AA, B6 = (A4 A4 - 2 A5 A3) / sqrt(3), the l = 1
    coupling to an invariant."""
    J = rn_basis(maxdeg=2, r0=1.0, rcut=5.0).J
    opb = {"__id__": "ACE_OrthPolyBasis", "T": {"__id__": "Type", "T": "Float64"},
           "pl": J.pl, "tl": J.tl, "pr": J.pr, "tr": J.tr,
           "A": list(J.A), "B": list(J.B), "C": list(J.C), "tdf": list(J.tdf), "ww": list(J.ww)}
    rn = {"__id__": "ACE_B1pComponent", "syms": ["n"],
          "basis": {"__id__": "ACE_SChain", "F": [{"__id__": "ACE_Lambda", "exstr": "rr -> norm(rr)"},
                                                  {"__id__": "ACE_Lambda", "exstr": "r -> ((1+1.0)/(1+r))^2"},
                                                  opb]},
          "fval": {"__id__": "ACE_StaticGet", "expr": "ACE.Transforms.GetVal{:rr}"},
          "spec": [{"n": 1}, {"n": 2}], "degrees": [0, 1], "label": "Rn"}
    ylm = {"__id__": "ACE_B1pComponent", "syms": ["l", "m"],
           "basis": {"__id__": "ACE_SHBasis", "T": {"__id__": "Type", "T": "Float64"}, "maxL": 1},
           "fval": {"__id__": "ACE_StaticGet", "expr": "ACE.Transforms.GetVal{:rr}"},
           "spec": [{"l": 0, "m": 0}, {"l": 1, "m": -1}, {"l": 1, "m": 0}, {"l": 1, "m": 1}],
           "degrees": [0, 1, 1, 1], "label": "Ylm"}
    inv = lambda v: {"__id__": "ACE_Invariant", "val": v, "T": {"__id__": "Type", "T": "Float64"}}  # noqa: E731
    # A2Bmap 6 x 7, CSC: columns AA1..AA7
    a2b = {"__id__": "SparseMatrixCSC", "m": 6, "n": 7,
           "colptr": [1, 2, 3, 4, 5, 6, 7, 8], "rowval": [1, 2, 3, 4, 5, 6, 6],
           "nzval": [inv(1.0), inv(1.0), inv(1.0), inv(1.0), inv(1.0), inv(-2 * S3), inv(S3)]}
    basis = {"__id__": "ACE_SymmetricBasis",
             "pibasis": {"__id__": "ACE_PIBasis",
                         "basis1p": {"__id__": "ACE_Product1pBasis", "bases": [rn, ylm],
                                     "indices": [[1, 1], [2, 1], [1, 2], [1, 3], [1, 4]]},
                         "spec": {"__id__": "ACE_PIBasisSpec", "orders": [1, 1, 2, 2, 2, 2, 2],
                                  "iAA2iA": [[1, 0], [2, 0], [1, 1], [2, 1], [2, 2], [5, 3], [4, 4]]},
                         "real": True},
             "A2Bmap": a2b, "symgrp": {"__id__": "ACE_O3", "lsym": "l", "msym": "m"}, "isreal": True}
    c = [0.3, -0.2, 0.5, 0.1, -0.4, 0.7]
    return {"__id__": "ACE_LinearACEModel", "basis": basis, "c": c,
            "evaluator": {"__id__": "ACE_ProductEvaluator"}}


def _rotation(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    return q * np.sign(np.diag(r))


def test_hand_written_dictionary(oracle_mod):
    D = json.loads(json.dumps(hand_written_model()))
    spec, c = from_write_dict(D)
    assert spec.nA == 5 and spec.nAA == 7 and spec.nB == 6 and spec.maxorder == 2
    assert list(spec.aspec.n) == [1, 2, 1, 1, 1] and list(spec.aspec.l) == [0, 0, 1, 1, 1]
    assert list(spec.aspec.m) == [0, 0, -1, 0, 1]
    assert spec.iAA2iA.tolist() == [[0, -1], [1, -1], [0, 0], [1, 0], [1, 1], [4, 2], [3, 3]]
    assert spec.radial.trans.p == 2 and spec.radial.trans.r0 == 1.0
    b = random_batch(20, 6, 14, seed=1)
    orc = oracle_mod.Oracle(spec, c)
    A = orc.A(b.offsets, b.rr)
    AA = np.stack([A[:, 0], A[:, 1], A[:, 0] ** 2, A[:, 1] * A[:, 0], A[:, 1] ** 2, A[:, 4] * A[:, 2],
                   A[:, 3] ** 2], axis=1)
    Bexp = np.real(AA[:, :5])
    Bexp = np.concatenate([Bexp, np.real(S3 * AA[:, 6] - 2 * S3 * AA[:, 5])[:, None]], axis=1)
    B = orc.basis(b.offsets, b.rr)
    assert np.max(np.abs(B - Bexp)) <= 1e-13 * np.max(np.abs(Bexp))
    E = orc.evaluate(b.offsets, b.rr)
    assert np.max(np.abs(E - Bexp @ np.asarray(c))) <= 1e-13 * np.max(np.abs(E))
    Er = orc.evaluate(b.offsets, b.rr @ _rotation(3).T)
    assert np.max(np.abs(Er - E)) <= 1e-12 * np.max(np.abs(E))


@pytest.mark.parametrize("ns", [1, 4])
def test_round_trip(oracle_mod, ns):
    spec = symmetric_basis(3, 6, maxL=6, nspecies=ns)
    c = random_coefficients(spec, seed=2)
    D = json.loads(json.dumps(to_write_dict(spec, c)))
    if ns > 1:
        assert D["basis"]["pibasis"]["basis1p"]["bases"][0]["__id__"] == "ACE_Categorical1pBasis"
    s2, c2 = from_write_dict(D)
    assert s2.nspecies == ns
    for f in ("mu", "n", "l", "m"):
        assert np.array_equal(getattr(s2.aspec, f), getattr(spec.aspec, f))
    assert np.array_equal(s2.orders, spec.orders) and np.array_equal(s2.iAA2iA, spec.iAA2iA)
    assert (s2.U != spec.U).nnz == 0
    assert np.array_equal(c2, c)
    for x in ("A", "B", "C"):
        assert np.array_equal(getattr(s2.radial.J, x), getattr(spec.radial.J, x))
    assert abs(s2.radial.rcut - spec.radial.rcut) < 1e-12 and abs(s2.radial.rin - spec.radial.rin) < 1e-12
    b = random_batch(30, 8, 20, nspecies=ns, seed=3)
    E1, G1 = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr, b.species)
    E2, G2 = oracle_mod.Oracle(s2, c2).energy_forces(b.offsets, b.rr, b.species)
    assert np.array_equal(E1, E2) and np.array_equal(G1, G2)


def test_matrix_encodings_agree():
    """iAA2iA as a list of rows and as {size, data} in column-major order."""
    D = hand_written_model()
    rows = D["basis"]["pibasis"]["spec"]["iAA2iA"]
    a = np.array(rows)
    D2 = json.loads(json.dumps(D))
    D2["basis"]["pibasis"]["spec"]["iAA2iA"] = {"__id__": "Matrix", "size": list(a.shape),
                                                "data": a.T.ravel().tolist()}
    s1, _ = from_write_dict(D)
    s2, _ = from_write_dict(D2)
    assert np.array_equal(s1.iAA2iA, s2.iAA2iA)


def test_rejects_unsupported():
    D = hand_written_model()
    D["basis"]["isreal"] = False
    with pytest.raises(ValueError):
        from_write_dict(D)
    D = hand_written_model()
    D["basis"]["pibasis"]["basis1p"]["bases"][0]["basis"]["F"][1]["exstr"] = "r -> exp(- 2.0 * (r / 1.0 - 1))"
    with pytest.raises(ValueError):
        from_write_dict(D)


@pytest.mark.gpu
def test_imported_model_on_gpu(oracle_mod):
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    build()
    spec = symmetric_basis(4, 8, maxL=6, nspecies=2)
    c = random_coefficients(spec, seed=5)
    s2, c2 = from_write_dict(json.loads(json.dumps(to_write_dict(spec, c))))
    b = random_batch(200, 10, 30, nspecies=2, seed=6)
    Eref, Gref = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr, b.species)
    ctx = L.Context(s2, "fp64")
    ctx.set_params(c2)
    E, G = ctx.energy_forces(b.offsets, b.rr, b.species)
    assert np.max(np.abs(E - Eref)) <= 1e-12 * np.max(np.abs(Eref))
    assert np.max(np.abs(G - Gref)) <= 1e-10 * np.max(np.abs(Gref))
    ctx.close()
