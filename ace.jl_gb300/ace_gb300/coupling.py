"""Rotation-invariant coupling coefficients (host-side, cold path).

Restates the O(3)-invariant part of ACE.jl's coupling-coefficient
construction:

* ``clebschgordan`` (``src/rotations3d.jl:108-137``): exact Racah formula with
  big integers, rounded once to Float64.
* ``Rot3DCoeffs`` generalized CG recursion (``src/rotations3d.jl:216-248``):
  couples the last two (l, m) pairs into j, recursing down to the
  invariant seed ``coco_init`` (l = m = 0, ``src/properties.jl:139-142``).
  Unrolled, the recursion is a sum over coupling paths J of
  T_J(mm) * T_J(kk), where T_J(mm) is the product of the CG coefficients
  along the path.  ``coupling_tree`` returns the rows T_J.
* ``re_basis`` (``src/rotations3d.jl:257-273``) takes an SVD of the Gram
  matrix of the rows A(ll, ., kk).  Because the T_J are orthonormal that Gram
  matrix is the projector T^T T, all of its non-zero singular values are 1,
  and any orthonormal basis of its range is an equally valid output; the
  reference's choice is whatever its LAPACK returns.  Here the orthonormal
  basis is the coupling-tree basis T itself (same span, deterministic);
  ``re_basis_reference`` restates the reference's SVD route for testing.
* ``rpe_basis`` (``src/symmetrygroups.jl:119-146``): permutation Gramian over
  the permutations that fix (nn, ll), SVD, rank with rtol 1e-7, then
  U = diag(sqrt(S)) V^T Ure — restated as written.
"""
from __future__ import annotations

import itertools
from decimal import Decimal, getcontext
from fractions import Fraction
from functools import lru_cache
from math import comb, factorial

import numpy as np

getcontext().prec = 60


def _cg_conditions(j1, m1, j2, m2, J, M):
    return (abs(j1 - j2) <= J <= j1 + j2) and (M == m1 + m2) and \
        abs(m1) <= j1 and abs(m2) <= j2 and abs(M) <= J


@lru_cache(maxsize=None)
def clebschgordan(j1: int, m1: int, j2: int, m2: int, J: int, M: int) -> float:
    """C_{j1 m1 j2 m2}^{J M}; same formula and argument order as
    ``src/rotations3d.jl:108-137``, evaluated exactly and rounded once."""
    if not _cg_conditions(j1, m1, j2, m2, J, M):
        return 0.0
    N = Fraction((2 * J + 1) * factorial(j1 + m1) * factorial(j1 - m1)
                 * factorial(j2 + m2) * factorial(j2 - m2)
                 * factorial(J + M) * factorial(J - M),
                 factorial(j1 + j2 - J) * factorial(j1 - j2 + J)
                 * factorial(-j1 + j2 + J) * factorial(j1 + j2 + J + 1))
    lb = max(0, j2 - J - m1, j1 - J + m2)
    ub = min(j1 + j2 - J, j1 - m1, j2 + m2)
    G = 0
    for k in range(lb, ub + 1):
        G += (-1) ** k * comb(j1 + j2 - J, k) * comb(j1 - j2 + J, j1 - m1 - k) \
            * comb(-j1 + j2 + J, j2 + m2 - k)
    if G == 0:
        return 0.0
    val = (Decimal(N.numerator) / Decimal(N.denominator)).sqrt() * Decimal(G)
    return float(val)


@lru_cache(maxsize=None)
def _cg_table(l1: int, l2: int, J: int) -> np.ndarray:
    """tab[m1 + l1, m2 + l2] = C_{l1 m1 l2 m2}^{J, m1+m2}."""
    tab = np.zeros((2 * l1 + 1, 2 * l2 + 1))
    for m1 in range(-l1, l1 + 1):
        for m2 in range(-l2, l2 + 1):
            if abs(m1 + m2) <= J:
                tab[m1 + l1, m2 + l2] = clebschgordan(l1, m1, l2, m2, J, m1 + m2)
    return tab


@lru_cache(maxsize=None)
def mrange(ll: tuple) -> np.ndarray:
    """All mm with |m_t| <= l_t and sum(mm) == 0, for even sum(ll); iterated in
    Julia CartesianIndices order (first index fastest) as
    ``_mrange`` / ``coco_filter`` do (``src/rotations3d.jl:49-66``,
    ``src/properties.jl:146-150``).  Returns an int array (nM, N)."""
    N = len(ll)
    if N == 0 or sum(ll) % 2 != 0:
        return np.zeros((0, N), dtype=np.int64)
    grids = np.meshgrid(*[np.arange(-l, l + 1) for l in ll], indexing="ij")
    # CartesianIndices: first index fastest -> flatten in Fortran order
    mm = np.stack([g.ravel(order="F") for g in grids], axis=1)
    return mm[mm.sum(axis=1) == 0].astype(np.int64)


@lru_cache(maxsize=None)
def coupling_tree(ll: tuple) -> np.ndarray:
    """Rows T_J(mm) over ``mrange(ll)``, one per coupling path J.

    The path couples (l_{N-1}, m_{N-1}) with (l_N, m_N) into j_{N-1}, then
    l_{N-2} with j_{N-1}, ..., finally l_1 with j_2 into 0, as the recursion
    in ``src/rotations3d.jl:216-248`` does."""
    mm = mrange(ll)
    N = len(ll)
    nM = mm.shape[0]
    if nM == 0:
        return np.zeros((0, 0))
    if N == 1:
        return np.ones((1, 1)) if ll[0] == 0 else np.zeros((0, nM))
    # states: list of (j, coefficient array over mm); M is determined by mm
    Mcur = mm[:, N - 1].copy()
    states = [(ll[N - 1], np.ones(nM))]
    for s in range(N - 2, -1, -1):
        ls = ll[s]
        ms = mm[:, s]
        Mnew = Mcur + ms
        new_states = []
        for (j, coef) in states:
            if s == 0:
                jrange = [0] if ls == j else []
            else:
                jrange = range(abs(ls - j), ls + j + 1)
            for jn in jrange:
                tab = _cg_table(ls, j, jn)
                ok = np.abs(Mnew) <= jn
                c = np.where(ok, tab[ms + ls, np.clip(Mcur + j, 0, 2 * j)], 0.0)
                c = np.where(np.abs(Mcur) <= j, c, 0.0)
                cn = coef * c
                if np.any(cn != 0):
                    new_states.append((jn, cn))
        states = new_states
        Mcur = Mnew
    if not states:
        return np.zeros((0, nM))
    return np.stack([c for (_, c) in states], axis=0)


def generalized_cg_reference(ll, mm, kk, _cache=None):
    """Literal restatement of the recursion of ``src/rotations3d.jl:191-248``
    (memoised); used by tests on small cases only."""
    if _cache is None:
        _cache = {}
    key = (tuple(ll), tuple(mm), tuple(kk))
    if key in _cache:
        return _cache[key]
    N = len(ll)
    if N == 1:
        val = 1.0 if (ll[0] == 0 and mm[0] == 0 and kk[0] == 0) else 0.0
        _cache[key] = val
        return val
    val = 0.0
    jmin = max(abs(ll[N - 2] - ll[N - 1]), abs(kk[N - 2] + kk[N - 1]), abs(mm[N - 2] + mm[N - 1]))
    jmax = ll[N - 2] + ll[N - 1]
    for j in range(jmin, jmax + 1):
        cgk = clebschgordan(ll[N - 2], kk[N - 2], ll[N - 1], kk[N - 1], j, kk[N - 2] + kk[N - 1])
        cgm = clebschgordan(ll[N - 2], mm[N - 2], ll[N - 1], mm[N - 1], j, mm[N - 2] + mm[N - 1])
        if cgk * cgm != 0:
            a = generalized_cg_reference(
                tuple(ll[:N - 2]) + (j,), tuple(mm[:N - 2]) + (mm[N - 2] + mm[N - 1],),
                tuple(kk[:N - 2]) + (kk[N - 2] + kk[N - 1],), _cache)
            val += cgk * cgm * a
    _cache[key] = val
    return val


def re_basis_reference(ll: tuple) -> np.ndarray:
    """The reference's re_basis route (``src/rotations3d.jl:257-273``):
    CC[a][i] = A(ll, mm_i, kk_a), G = CC CC^T, SVD, rank rtol 1e-7,
    Ure = diag(sqrt(S)) U^T CC.  Small cases only (tests)."""
    mm = mrange(ll)
    nM = mm.shape[0]
    if nM == 0:
        return np.zeros((0, 0))
    cache = {}
    CC = np.array([[generalized_cg_reference(ll, tuple(mm[i]), tuple(mm[a]), cache)
                    for i in range(nM)] for a in range(nM)])
    G = CC @ CC.T
    U, S, _ = np.linalg.svd(G)
    rk = int(np.sum(S > 1e-7 * S[0])) if S.size and S[0] > 0 else 0
    return np.diag(np.sqrt(S[:rk])) @ U[:, :rk].T @ CC


def stabiliser(nn: tuple, ll: tuple) -> list:
    """Permutations sigma with nn[sigma] == nn and ll[sigma] == ll, in
    Combinatorics.permutations order (lexicographic)."""
    N = len(ll)
    out = []
    for sig in itertools.permutations(range(N)):
        if all(nn[sig[t]] == nn[t] and ll[sig[t]] == ll[t] for t in range(N)):
            out.append(sig)
    return out


def _nn_pattern(nn: tuple) -> tuple:
    """Equality pattern of nn: first-occurrence labels (the stabiliser and so
    the class's U only depend on this and on ll)."""
    seen = {}
    return tuple(seen.setdefault(x, len(seen)) for x in nn)


@lru_cache(maxsize=None)
def rpe_basis(ll: tuple, pattern: tuple) -> np.ndarray:
    """U for one (nn, ll) class over ``mrange(ll)`` (symmetrygroups.jl:119-146):
    G = sum_sigma Ure P_sigma Ure^T, SVD, rank rtol 1e-7,
    U = diag(sqrt(S[:rk])) V[:, :rk]^T Ure."""
    Ure = coupling_tree(ll)
    mm = mrange(ll)
    nre = Ure.shape[0]
    if nre == 0 or mm.shape[0] == 0:
        return np.zeros((0, mm.shape[0]))
    N = len(ll)
    # index of each mm tuple
    lmax = max(ll)
    base = 2 * lmax + 1
    keys = ((mm + lmax) * (base ** np.arange(N))).sum(axis=1)
    order = np.argsort(keys)
    skeys = keys[order]
    G = np.zeros((nre, nre))
    for sig in stabiliser(pattern, ll):
        perm_mm = mm[:, list(sig)]
        pk = ((perm_mm + lmax) * (base ** np.arange(N))).sum(axis=1)
        idx = order[np.searchsorted(skeys, pk)]
        # mm1[sigma] == mm2  ->  G += Ure[:, mm1] Ure[:, mm2]^T
        G += Ure @ Ure[:, idx].T
    U, S, _ = np.linalg.svd(G)
    if S.size == 0 or S[0] <= 0:
        return np.zeros((0, mm.shape[0]))
    rk = int(np.sum(S > 1e-7 * S[0]))
    return np.diag(np.sqrt(S[:rk])) @ U[:, :rk].T @ Ure


# ---------------------------------------------------------------------------
# Equivariant vector (EuclideanVector) couplings, src/properties.jl:154-248.
#
# The coupling tree above, ended in total angular momentum L instead of 0,
# gives rows T_J(mm) over the m-tuples with |sum mm| <= L; for L = 1 each row
# defines a spherical vector F_M = sum_{sum mm = M} T_J(mm) prod Y_{l_t m_t}
# that rotates like Y_1^M.  With Y_1^{-1} = (x - iy)/sqrt2, Y_1^0 = z,
# Y_1^{+1} = -(x + iy)/sqrt2 (up to a common factor, Condon-Shortley phase),
# the Cartesian components are x = (F_{-1} - F_{+1})/sqrt2,
# y = i (F_{-1} + F_{+1})/sqrt2, z = F_0.  Their real and imaginary parts
# are real O(3)-equivariant vector functions (for odd sum(ll)); a real
# function is represented by coefficients u with u(mm) = (-1)^{sum mm}
# conj(u(-mm)), for which sum_mm u(mm) AA(mm) is real.


@lru_cache(maxsize=None)
def mrange_L(ll: tuple, L: int) -> np.ndarray:
    """All mm with |m_t| <= l_t and |sum(mm)| <= L, in CartesianIndices order."""
    N = len(ll)
    if N == 0:
        return np.zeros((0, 0), dtype=np.int64)
    grids = np.meshgrid(*[np.arange(-l, l + 1) for l in ll], indexing="ij")
    mm = np.stack([g.ravel(order="F") for g in grids], axis=1)
    return mm[np.abs(mm.sum(axis=1)) <= L].astype(np.int64)


@lru_cache(maxsize=None)
def coupling_tree_L(ll: tuple, L: int) -> np.ndarray:
    """Rows T_J(mm) over ``mrange_L(ll, L)``: coupling paths as in
    ``coupling_tree`` whose last step couples l_1 with j_2 into L (M = sum mm)."""
    mm = mrange_L(ll, L)
    N = len(ll)
    nM = mm.shape[0]
    if nM == 0:
        return np.zeros((0, 0))
    if N == 1:
        return np.ones((1, nM)) if ll[0] == L else np.zeros((0, nM))
    Mcur = mm[:, N - 1].copy()
    states = [(ll[N - 1], np.ones(nM))]
    for s in range(N - 2, -1, -1):
        ls = ll[s]
        ms = mm[:, s]
        Mnew = Mcur + ms
        new_states = []
        for (j, coef) in states:
            if s == 0:
                jrange = [L] if abs(ls - j) <= L <= ls + j else []
            else:
                jrange = range(abs(ls - j), ls + j + 1)
            for jn in jrange:
                tab = _cg_table(ls, j, jn)
                ok = np.abs(Mnew) <= jn
                c = np.where(ok, tab[ms + ls, np.clip(Mcur + j, 0, 2 * j)], 0.0)
                c = np.where(np.abs(Mcur) <= j, c, 0.0)
                cn = coef * c
                if np.any(cn != 0):
                    new_states.append((jn, cn))
        states = new_states
        Mcur = Mnew
    if not states:
        return np.zeros((0, nM))
    return np.stack([c for (_, c) in states], axis=0)


def _neg_index(mm: np.ndarray, ll: tuple) -> np.ndarray:
    """Index of -mm for every row of mm (the set is closed under negation)."""
    N = len(ll)
    lmax = max(ll)
    base = 2 * lmax + 1
    w = base ** np.arange(N)
    keys = ((mm + lmax) * w).sum(axis=1)
    order = np.argsort(keys)
    nk = ((-mm + lmax) * w).sum(axis=1)
    return order[np.searchsorted(keys[order], nk)]


def _real_rows(G: np.ndarray, neg: np.ndarray, sgn: np.ndarray) -> np.ndarray:
    """(G + sigma(G))/2 with sigma(G)(mm) = (-1)^{sum mm} conj(G(-mm)); G is
    (..., 3, nM)."""
    return 0.5 * (G + sgn * np.conj(G[..., neg]))


@lru_cache(maxsize=None)
def vector_rpe_basis(ll: tuple, pattern: tuple) -> np.ndarray:
    """Coefficients (nb, 3, nM) over ``mrange_L(ll, 1)`` of an independent,
    permutation-symmetrised set of real equivariant vector functions of one
    (nn, ll) class (the role of src/symmetrygroups.jl:119-146 for
    EuclideanVector): real and imaginary parts of every coupling path's
    Cartesian vector, reduced to a basis by an SVD (rank rtol 1e-7), then
    the permutation Gramian over the stabiliser of (nn, ll), SVD and rank
    rtol 1e-7 as in ``rpe_basis``."""
    mm = mrange_L(ll, 1)
    nM = mm.shape[0]
    T = coupling_tree_L(ll, 1)
    if T.shape[0] == 0 or nM == 0:
        return np.zeros((0, 3, nM), dtype=complex)
    M = mm.sum(axis=1)
    s2 = 1.0 / np.sqrt(2.0)
    cart = np.zeros((3, nM), dtype=complex)      # F_i = sum_M cart[i, M] F_M, per mm
    cart[0] = np.where(M == -1, s2, 0.0) - np.where(M == 1, s2, 0.0)
    cart[1] = 1j * (np.where(M == -1, s2, 0.0) + np.where(M == 1, s2, 0.0))
    cart[2] = np.where(M == 0, 1.0, 0.0)
    G = T[:, None, :] * cart[None, :, :]         # (npath, 3, nM)
    neg = _neg_index(mm, ll)
    sgn = np.where(M % 2 == 0, 1.0, -1.0)
    rows = np.concatenate([_real_rows(G, neg, sgn), _real_rows(-1j * G, neg, sgn)], axis=0)
    R = np.concatenate([rows.real.reshape(len(rows), -1), rows.imag.reshape(len(rows), -1)], axis=1)
    _, S, Vh = np.linalg.svd(R, full_matrices=False)
    if S.size == 0 or S[0] <= 0:
        return np.zeros((0, 3, nM), dtype=complex)
    W = Vh[:int(np.sum(S > 1e-7 * S[0]))]          # orthonormal real rows (re | im)
    # permutation Gramian
    N = len(ll)
    lmax = max(ll)
    base = 2 * lmax + 1
    w = base ** np.arange(N)
    keys = ((mm + lmax) * w).sum(axis=1)
    order = np.argsort(keys)
    skeys = keys[order]
    half = 3 * nM
    Gm = np.zeros((len(W), len(W)))
    for sig in stabiliser(pattern, ll):
        pk = ((mm[:, list(sig)] + lmax) * w).sum(axis=1)
        idx = order[np.searchsorted(skeys, pk)]
        full = np.concatenate([(np.arange(3)[:, None] * nM + idx[None, :]).ravel(),
                               half + (np.arange(3)[:, None] * nM + idx[None, :]).ravel()])
        Gm += W @ W[:, full].T
    U, S, _ = np.linalg.svd(Gm)
    if S.size == 0 or S[0] <= 0:
        return np.zeros((0, 3, nM), dtype=complex)
    rk = int(np.sum(S > 1e-7 * S[0]))
    Wr = np.diag(np.sqrt(S[:rk])) @ U[:, :rk].T @ W
    return (Wr[:, :half] + 1j * Wr[:, half:]).reshape(rk, 3, nM)


@lru_cache(maxsize=None)
def rpe_basis_L(ll: tuple, pattern: tuple, L: int) -> np.ndarray:
    """``rpe_basis`` for a spherical-tensor output of total angular momentum L
    (SphericalVector, src/properties.jl:431-520): the coupling-tree rows
    ending in L (``coupling_tree_L``) over ``mrange_L(ll, L)``, symmetrised
    with the permutation Gramian (SVD, rank rtol 1e-7).  Row b defines the
    components B_b^M = sum_{sum mm = M} U[b, mm] prod Y_{l_t m_t}, which
    rotate like Y_L^M."""
    Ure = coupling_tree_L(ll, L)
    mm = mrange_L(ll, L)
    nre = Ure.shape[0]
    if nre == 0 or mm.shape[0] == 0:
        return np.zeros((0, mm.shape[0]))
    N = len(ll)
    lmax = max(ll)
    base = 2 * lmax + 1
    w = base ** np.arange(N)
    keys = ((mm + lmax) * w).sum(axis=1)
    order = np.argsort(keys)
    skeys = keys[order]
    G = np.zeros((nre, nre))
    for sig in stabiliser(pattern, ll):
        pk = ((mm[:, list(sig)] + lmax) * w).sum(axis=1)
        idx = order[np.searchsorted(skeys, pk)]
        G += Ure @ Ure[:, idx].T
    U, S, _ = np.linalg.svd(G)
    if S.size == 0 or S[0] <= 0:
        return np.zeros((0, mm.shape[0]))
    rk = int(np.sum(S > 1e-7 * S[0]))
    return np.diag(np.sqrt(S[:rk])) @ U[:, :rk].T @ Ure
