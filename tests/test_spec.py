"""Basis construction rules: sizes, ordering and index lists."""
import itertools

import numpy as np
import pytest

from ace_gb300.coupling import (coupling_tree, mrange, re_basis_reference, rpe_basis,
                                stabiliser)
from ace_gb300.spec import gensparse_ordered, init1pspec, symmetric_basis


def test_sizes_match_reference_counts():
    # maxdeg=6, ord=3 (test/test_linearmodel.jl:22-25): 139 A pre-clean -> 43;
    # AA by order 1:6, 2:59, 3:181 after cleaning.
    s = symmetric_basis(3, 6, maxL=6)
    assert s.info["nA_pre"] == 139 and s.nA == 43
    assert s.info["nAA_by_order"] == {0: 1, 1: 6, 2: 59, 3: 181}
    s1 = symmetric_basis(3, 8, maxL=6)
    assert s1.info["nA_pre"] == 237 and s1.nA == 84


def test_init1pspec_order():
    a = init1pspec(6, 6, 6)
    deg = a.degree
    assert np.all(np.diff(deg) >= 0)
    # ties in CartesianIndices order (n fastest, then l, then m) -> key (m, l, n)
    for d in np.unique(deg):
        idx = np.nonzero(deg == d)[0]
        keys = list(zip(a.m[idx], a.l[idx], a.n[idx]))
        assert keys == sorted(keys)
    assert len(a) == 139


def test_gensparse_bruteforce():
    a = init1pspec(5, 5, 5)
    deg = a.degree.astype(float)
    got = gensparse_ordered(deg, a.l, a.m, 3, 5)
    nA = len(a)
    for k in range(1, 4):
        want = []
        for tup in itertools.combinations_with_replacement(range(nA), k):
            if deg[list(tup)].sum() > 5:
                continue
            if k >= 2 and (a.l[list(tup)].sum() % 2 or a.m[list(tup)].sum() != 0):
                continue
            want.append(tup)
        want.sort()
        assert [tuple(r) for r in got[k].tolist()] == want


def test_iAA2iA_descending_and_orders():
    s = symmetric_basis(3, 6, maxL=6)
    assert s.orders[0] == 0
    for i in range(s.nAA):
        k = s.orders[i]
        row = s.iAA2iA[i]
        assert np.all(row[k:] == -1) and np.all(row[:k] >= 0)
        assert np.all(np.diff(row[:k]) <= 0)
    assert np.all(np.diff(s.orders) >= 0)


@pytest.mark.parametrize("ll", [(1, 1), (2, 1, 1), (1, 1, 1, 1), (2, 2, 2), (0, 0, 0), (3, 2, 1)])
def test_coupling_tree_spans_reference_re_basis(ll):
    T = coupling_tree(ll)
    assert np.allclose(T @ T.T, np.eye(T.shape[0]), atol=1e-12)
    Ure = re_basis_reference(ll)
    # same subspace: projectors agree
    assert np.allclose(T.T @ T, Ure.T @ Ure, atol=1e-10)


def test_rpe_basis_symmetric_and_invariant():
    ll = (1, 1, 1, 1)
    pat = (0, 0, 0, 0)
    U = rpe_basis(ll, pat)
    mm = mrange(ll)
    stab = stabiliser(pat, ll)
    assert len(stab) == 24
    # each row is invariant under the stabiliser's permutations of mm
    keys = {tuple(r): i for i, r in enumerate(mm.tolist())}
    for sig in stab:
        idx = [keys[tuple(r[t] for t in sig)] for r in mm.tolist()]
        assert np.allclose(U[:, idx], U, atol=1e-12)


@pytest.mark.parametrize("N,pcut,pin,Nquad", [(8, 2, 0, None), (16, 2, 0, None), (12, 2, 2, 500), (6, 0, 0, 300)])
def test_radial_polynomials_orthonormal_on_their_grid(N, pcut, pin, Nquad):
    # The discrete Stieltjes procedure (src/polynomials/orthpolys.jl:153-218)
    # makes P_1..P_N orthonormal in the weighted discrete inner product on
    # the grid it was built on; the reference's own test asks for this check
    # (test/polynomials/test_orthpolys.jl: "replace this test with an
    # orthogonality test").
    from ace_gb300.radial import PolyTransform, discrete_jacobi
    J = discrete_jacobi(N, pcut=pcut, xcut=5.0, pin=pin, xin=0.8, Nquad=Nquad, trans=PolyTransform(2, 1.0))
    P = J.evaluate(J.tdf)
    G = P.T @ (J.ww[:, None] * P)
    assert np.max(np.abs(G - np.eye(N))) < 1e-10
    # the envelope vanishes at the cutoff end of the transformed interval
    tc = J.tl if J.pl > 0 else J.tr
    if pcut > 0:
        assert np.max(np.abs(J.evaluate(np.array([tc])))) < 1e-14


@pytest.mark.parametrize("deg,nspecies,order,prop", [(8, 1, 4, "invariant"), (8, 2, 3, "invariant"),
                                                     (8, 1, 5, "vector"), (7, 1, 4, ("spherical", 2))])
def test_gensparse_bounded_enumeration_is_order_preserving(deg, nspecies, order, prop):
    # splitting the prefix sets (small row budget) must give the same tuples
    # in the same (lexicographic) order as one unsplit enumeration
    from ace_gb300.spec import init1pspec
    a = init1pspec(deg, deg, deg, nspecies)
    full = gensparse_ordered(a.degree.astype(float), a.l, a.m, order, deg, prop, chunk_rows=1 << 30)
    split = gensparse_ordered(a.degree.astype(float), a.l, a.m, order, deg, prop, chunk_rows=64)
    assert len(full) == len(split)
    for x, y in zip(full, split):
        assert x.shape == y.shape and np.array_equal(x, y)


@pytest.mark.parametrize("order,deg,nspecies", [(3, 8, 1), (4, 8, 2), (5, 8, 1), (2, 8, 4)])
def test_grouped_coupling_matches_the_per_function_loop(order, deg, nspecies, monkeypatch):
    # U, row degrees and class indices of the grouped construction are
    # bit-identical to one loop over the reference functions
    import ace_gb300.spec as S
    grouped = S.symmetric_basis(order, deg, maxL=deg, nspecies=nspecies)
    monkeypatch.setattr(S, "_coupling_rows", S._coupling_rows_loop)
    loop = S.symmetric_basis(order, deg, maxL=deg, nspecies=nspecies)
    for attr in ("indptr", "indices", "data"):
        assert np.array_equal(getattr(grouped.U, attr), getattr(loop.U, attr))
    assert np.array_equal(grouped.Bdeg, loop.Bdeg) and np.array_equal(grouped.Bclass, loop.Bclass)
    assert np.array_equal(grouped.iAA2iA, loop.iAA2iA) and grouped.info == loop.info
