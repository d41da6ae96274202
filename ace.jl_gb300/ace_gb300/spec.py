"""Basis specification: 1-particle spec, AA spec, coupling matrix U.

Host-side restatement of ACE.jl's cold construction path, producing the
index lists every evaluator (GPU kernels and the oracle) consumes:

* 1p spec  -- ``init1pspec!`` (``src/sparsegrids.jl:9-31``): all admissible
  (mu, n, l, m) in Julia ``CartesianIndices`` order (first symbol fastest),
  ``m`` forced to -maxL:maxL (``src/product_1pbasis.jl:283-304``), kept when
  level = (n-1) + l <= maxdeg, then stably sorted by level.
* AA spec  -- ``gensparse(ordered=true)`` (``src/sparsegrids.jl:55-148``):
  ascending index tuples of a downset in lexicographic order (so order-major),
  filtered by the Invariant rule even(sum l) and sum m == 0 for length >= 2
  (``src/properties.jl:115-125``); rows are then stored reversed
  (``src/pibasis.jl:90-101``).
* U        -- ``SymmetricBasis`` (``src/symmbasis.jl:89-162``): one class per
  AA with all m == 0 (``is_refbasisfcn``, ``src/symmetrygroups.jl:91``),
  rows from ``rpe_basis``, columns mapped to AA indices through
  ``_get_ordered`` (A index descending, ``src/symmbasis.jl:174-177``),
  duplicates summed as ``sparse`` does.
* cleaning -- ``clean_pibasis!`` / ``clean_1pbasis!``
  (``src/symmbasis.jl:225-236``, ``src/pibasis.jl:194-207``,
  ``src/product_1pbasis.jl:345-374``): drop AA columns of U that are zero,
  then A entries no AA uses, preserving order.

A U entry whose magnitude is below 1e-12 of its row maximum is treated as an
exact zero before cleaning (the reference keeps round-off-sized columns,
which depend on its LAPACK).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from .coupling import _nn_pattern, mrange, rpe_basis
from .radial import RadialBasis, rn_basis


@dataclass
class OnePSpec:
    """The A basis: entry i is R_{n_i}(r) Y_{l_i}^{m_i}(rhat) [delta(mu_i, mu_j)]."""
    mu: np.ndarray       # species index (0-based), all 0 for one species
    n: np.ndarray        # 1-based radial index
    l: np.ndarray
    m: np.ndarray

    def __len__(self):
        return len(self.n)

    @property
    def degree(self):
        return (self.n - 1) + self.l

    def tuples(self):
        return list(zip(self.mu.tolist(), self.n.tolist(), self.l.tolist(), self.m.tolist()))


def init1pspec(nR: int, maxL: int, maxdeg: float, nspecies: int = 1) -> OnePSpec:
    """init1pspec! for (Categorical?) x Rn x Ylm with SimpleSparseBasis."""
    mu, n, l, m = [], [], [], []
    # CartesianIndices over (mu?, n, l, m): first symbol fastest.
    for mm in range(-maxL, maxL + 1):
        for ll in range(0, maxL + 1):
            for nn in range(1, nR + 1):
                for s in range(nspecies):
                    if abs(mm) > ll:           # Ylm component admissibility
                        continue
                    if (nn - 1) + ll <= maxdeg:  # level1 <= maxlevel1
                        mu.append(s); n.append(nn); l.append(ll); m.append(mm)
    mu, n, l, m = map(lambda x: np.array(x, dtype=np.int64), (mu, n, l, m))
    deg = (n - 1) + l
    p = np.argsort(deg, kind="stable")     # sort!(spec, by=level): stable
    return OnePSpec(mu[p], n[p], l[p], m[p])


# partial tuples expanded per step of the enumeration: bounds its memory
# (rows of k indices and three sums) independently of the basis size
_ENUM_ROWS = 1 << 22


def gensparse_ordered(deg: np.ndarray, ls: np.ndarray, ms: np.ndarray,
                      maxorder: int, maxdeg: float, prop: str = "invariant",
                      chunk_rows: int = _ENUM_ROWS) -> list:
    """All ascending tuples v_1 <= ... <= v_k (0-based A indices, k = 0..maxorder)
    with sum(deg[v]) <= maxdeg, kept when k <= 1 or (sum l even and sum m == 0)
    for the Invariant property (src/properties.jl:133-150), or when sum l is
    odd and |sum m| <= 1 (k >= 1, no constant) for EuclideanVector
    (src/properties.jl:189-203,240-246).
    Returned per order k as int arrays (N_k, k), each in lexicographic order,
    which is gensparse's enumeration order (order-major because shorter
    tuples are padded with leading zeros).

    The enumeration extends partial tuples one index at a time; a set of
    prefixes whose extension would exceed ``chunk_rows`` rows is split in two
    (in order) and each half is enumerated to the end and filtered before
    the next, so memory stays bounded while the output order is unchanged."""
    deg = np.asarray(deg)
    assert np.all(np.diff(deg) >= 0), "A spec must be sorted by degree"
    ls = np.asarray(ls, dtype=np.int64)
    ms = np.asarray(ms, dtype=np.int64)
    vec = prop == "vector"
    sphL = prop[1] if isinstance(prop, tuple) and prop[0] == "spherical" else None
    mslack = 1 if vec else (sphL if sphL is not None else 0)
    const = not vec and (sphL is None or sphL == 0)

    def final_filter(tup, msum, lsum, k):
        if not len(tup):
            return tup
        if vec:
            return tup[(lsum % 2 == 1) & (np.abs(msum) <= 1)]
        if sphL is not None:
            if k >= 2 or sphL > 0:
                return tup[(lsum % 2 == sphL % 2) & (np.abs(msum) <= sphL)]
            return tup
        if k >= 2:
            return tup[(lsum % 2 == 0) & (msum == 0)]
        return tup

    # invariant functions of order >= 2 end with an index whose m and l
    # parity are fixed by the prefix (sum m = 0, sum l even): the A indices of
    # each (m, l parity), ascending, enumerate just those
    invariant = not vec and sphL is None
    by_mp = {}
    if invariant:
        for mv in np.unique(ms):
            for par in (0, 1):
                by_mp[(int(mv), par)] = np.nonzero((ms == mv) & (ls % 2 == par))[0]

    def last_invariant(tup, dsum, msum, lsum, parts):
        """The last index of invariant tuples: per prefix row, the A indices
        v in [lo, hi) with m_v = -msum and l_v = lsum (mod 2), ascending, so
        rows and their completions come out in lexicographic order."""
        lo = tup[:, -1]
        hi = np.searchsorted(deg, maxdeg - dsum, side="right")
        tm = -msum
        tp = lsum % 2
        cnt = np.zeros(len(tup), dtype=np.int64)
        first = np.zeros(len(tup), dtype=np.int64)
        keys = tm * 2 + tp
        for key in np.unique(keys):
            sel = np.nonzero(keys == key)[0]
            P = by_mp.get((int(key // 2), int(key % 2)))
            if P is None or not len(P):
                continue
            a = np.searchsorted(P, lo[sel], side="left")
            b = np.searchsorted(P, hi[sel], side="left")
            cnt[sel] = np.maximum(b - a, 0)
            first[sel] = a
        total = int(cnt.sum())
        if total == 0:
            return
        off = np.concatenate([[0], np.cumsum(cnt)])
        rows = np.repeat(np.arange(len(tup)), cnt)
        j = np.arange(total) - off[rows]
        v = np.empty(total, dtype=np.int64)
        for key in np.unique(keys[cnt > 0]):
            P = by_mp[(int(key // 2), int(key % 2))]
            m_ = keys[rows] == key
            v[m_] = P[first[rows[m_]] + j[m_]]
        parts.append(np.concatenate([tup[rows], v[:, None]], axis=1))

    def extend(tup, dsum, msum, lsum, t, k, parts):
        """Enumerate the completions of the prefixes `tup` (t indices each)
        to order k; append the filtered tuples to `parts` in order."""
        if t == k:
            f = final_filter(tup, msum, lsum, k)
            if len(f):
                parts.append(f)
            return
        rem = k - t
        lo = tup[:, -1] if t > 0 else np.zeros(len(tup), dtype=np.int64)
        # remaining rem entries all have degree >= deg[v]
        hi = np.searchsorted(deg, (maxdeg - dsum) / rem, side="right")
        cnt = np.maximum(hi - lo, 0)
        total = int(cnt.sum())
        if invariant and k >= 2 and t == k - 1 and total > 0:
            if total > chunk_rows and len(tup) > 1:
                h = len(tup) // 2
                extend(tup[:h], dsum[:h], msum[:h], lsum[:h], t, k, parts)
                extend(tup[h:], dsum[h:], msum[h:], lsum[h:], t, k, parts)
            else:
                last_invariant(tup, dsum, msum, lsum, parts)
            return
        if total == 0:
            return
        if total > chunk_rows and len(tup) > 1:
            h = len(tup) // 2
            extend(tup[:h], dsum[:h], msum[:h], lsum[:h], t, k, parts)
            extend(tup[h:], dsum[h:], msum[h:], lsum[h:], t, k, parts)
            return
        rows = np.repeat(np.arange(len(tup)), cnt)
        starts = np.repeat(lo - np.cumsum(np.concatenate([[0], cnt[:-1]])), cnt)
        v = np.arange(total) + starts
        tup2 = np.concatenate([tup[rows], v[:, None]], axis=1)
        dsum2 = dsum[rows] + deg[v]
        msum2 = msum[rows] + ms[v]
        lsum2 = lsum[rows] + ls[v]
        keep = dsum2 <= maxdeg + 1e-12
        if t < k - 1:
            # prune: the remaining entries have |m| <= l <= deg <= maxdeg - dsum
            keep &= np.abs(msum2) <= (maxdeg - dsum2) + mslack + 1e-12
        del rows, starts, v
        extend(tup2[keep], dsum2[keep], msum2[keep], lsum2[keep], t + 1, k, parts)

    out = [np.zeros((1 if const else 0, 0), dtype=np.int64)]  # order 0: the constant (L = 0 outputs only)
    for k in range(1, maxorder + 1):
        parts = []
        extend(np.zeros((1, 0), dtype=np.int64), np.zeros(1), np.zeros(1, dtype=np.int64),
               np.zeros(1, dtype=np.int64), 0, k, parts)
        tup = np.concatenate(parts, axis=0) if parts else np.zeros((0, k), dtype=np.int64)
        if len(tup) > 1:
            # generated in lexicographic order already; keep the guarantee explicit
            order = np.lexsort(tup.T[::-1])
            if np.any(order != np.arange(len(tup))):
                tup = tup[order]
        out.append(tup)
    return out


@dataclass
class ACESpec:
    """Everything an evaluator needs: the radial basis, maxL, the A spec,
    the AA spec (descending rows, -1 padded), U (CSR nB x nAA) and the
    per-B degree used for coefficient scaling."""
    radial: RadialBasis
    maxL: int
    nspecies: int
    aspec: OnePSpec
    orders: np.ndarray          # (nAA,)
    iAA2iA: np.ndarray          # (nAA, maxorder), 0-based, -1 padded
    U: sp.csr_matrix            # (nB, nAA)
    Bdeg: np.ndarray            # (nB,)
    Bclass: np.ndarray          # (nB,) index of the class each B row belongs to
    info: dict = field(default_factory=dict)

    @property
    def nA(self):
        return len(self.aspec)

    @property
    def nAA(self):
        return len(self.orders)

    @property
    def nB(self):
        return self.U.shape[0]

    @property
    def maxorder(self):
        return self.iAA2iA.shape[1]

    @property
    def Leff(self):
        """Largest l any A entry uses (SH only need to be evaluated to here)."""
        return int(self.aspec.l.max()) if self.nA else 0

    def ctilde(self, c: np.ndarray) -> np.ndarray:
        """c~ = U^T c (``_get_eff_coeffs!``, src/evaluator.jl:59-60)."""
        return np.asarray(self.U.T @ np.asarray(c, dtype=np.float64)).ravel()


def _encode(rows: np.ndarray, base: int) -> np.ndarray:
    """Integer key of each (descending, -1 padded) index row."""
    k = np.zeros(rows.shape[0], dtype=np.int64)
    for t in range(rows.shape[1]):
        k = k * base + (rows[:, t] + 1)
    return k


def _coupling_rows_loop(aspec, iAA2iA, orders, skeys, korder, aidx, base, maxorder, maxL, zero_tol):
    """U rows of every class, one reference function (all m == 0) at a time in
    AA order (src/symmbasis.jl:89-162): the class's rpe_basis over mrange(ll),
    columns collapsed onto the ordered AA functions (_get_ordered), small
    entries dropped.  The reference implementation of _coupling_rows."""
    a_m = aspec.m
    refmask = np.all(np.where(iAA2iA >= 0, a_m[np.maximum(iAA2iA, 0)] == 0, True), axis=1)
    adeg = aspec.degree
    Irow, Jcol, vals, Bdeg, Bclass = [], [], [], [], []
    nB = 0
    nclass = 0
    for iAA in np.nonzero(refmask)[0]:
        k = int(orders[iAA])
        vs = iAA2iA[iAA, :k]
        if k == 0:
            Irow.append(np.array([nB])); Jcol.append(np.array([iAA])); vals.append(np.array([1.0]))
            Bdeg.append(0.0); Bclass.append(nclass)
            nB += 1; nclass += 1
            continue
        ll = tuple(int(x) for x in aspec.l[vs])
        nn = tuple((int(a), int(b)) for a, b in zip(aspec.mu[vs], aspec.n[vs]))
        U = rpe_basis(ll, _nn_pattern(nn))
        if U.shape[0] == 0:
            continue
        mm = mrange(ll)
        A = np.stack([aidx[aspec.mu[vs[t]], aspec.n[vs[t]], ll[t], mm[:, t] + maxL]
                      for t in range(k)], axis=1)
        assert np.all(A >= 0)
        A = -np.sort(-A, axis=1)                       # _get_ordered
        r = -np.ones((len(A), maxorder), dtype=np.int64)
        r[:, :k] = A
        pk = _encode(r, base)
        pos = np.searchsorted(skeys, pk)
        if np.any(pos >= len(skeys)) or np.any(skeys[np.minimum(pos, len(skeys) - 1)] != pk):
            raise RuntimeError("bcol_ordered not in AA-spec")
        cols = korder[pos]
        ucols, inv = np.unique(cols, return_inverse=True)
        Uc = np.zeros((U.shape[0], len(ucols)))
        np.add.at(Uc.T, inv, U.T)
        rmax = np.abs(Uc).max(axis=1, keepdims=True)
        Uc[np.abs(Uc) <= zero_tol * rmax] = 0.0
        d = float(sum(adeg[vs]))
        for irow in range(U.shape[0]):
            nzm = Uc[irow] != 0
            Irow.append(np.full(int(nzm.sum()), nB)); Jcol.append(ucols[nzm]); vals.append(Uc[irow, nzm])
            Bdeg.append(d); Bclass.append(nclass)
            nB += 1
        nclass += 1
    return Irow, Jcol, vals, Bdeg, Bclass, nB, nclass


def _coupling_rows(aspec, iAA2iA, orders, skeys, korder, aidx, base, maxorder, maxL, zero_tol):
    """The rows of _coupling_rows_loop, computed once per class signature.

    A class's U depends only on ll and the equality pattern of its (mu, n)
    (rpe_basis), and so does the partition of its m-tuples into AA functions
    (two m-tuples collapse onto one ordered function iff they agree up to
    permutations within equal (mu, n, l) entries).  So the column sums, the
    dropped entries and the row count are computed once per signature and
    every member only looks up its own AA columns; rows are placed at the
    offsets the loop would give them (same values, same row order)."""
    a_m = aspec.m
    refmask = np.all(np.where(iAA2iA >= 0, a_m[np.maximum(iAA2iA, 0)] == 0, True), axis=1)
    ref = np.nonzero(refmask)[0]
    F = len(ref)
    V = iAA2iA[ref]
    ks = orders[ref].astype(np.int64)
    valid = V >= 0
    Vc = np.maximum(V, 0)
    Ls = np.where(valid, aspec.l[Vc], -1).astype(np.int64)
    MU = aspec.mu[Vc].astype(np.int64)
    NN = aspec.n[Vc].astype(np.int64)
    nnkey = np.where(valid, MU * (int(NN.max(initial=0)) + 1) + NN, -1)
    # first-occurrence labels of (mu, n) along each row (_nn_pattern)
    lab = np.full(V.shape, -1, dtype=np.int64)
    nlab = np.zeros(F, dtype=np.int64)
    for t in range(maxorder):
        first = np.full(F, -1, dtype=np.int64)
        for s_ in range(t - 1, -1, -1):
            first = np.where(valid[:, t] & (nnkey[:, s_] == nnkey[:, t]), lab[:, s_], first)
        new = valid[:, t] & (first < 0)
        lab[:, t] = np.where(new, nlab, first)
        nlab += new
    sig = ks.copy()
    for t in range(maxorder):
        sig = sig * 512 + (Ls[:, t] + 1) * 8 + (lab[:, t] + 1)
    usig, ginv = np.unique(sig, return_inverse=True)
    dsum = np.where(valid, aspec.degree[Vc], 0).sum(axis=1).astype(np.float64)

    # per signature: U (rows), the m-tuples, and the collapse pattern
    groups = []
    nrows = np.zeros(F, dtype=np.int64)
    for g in range(len(usig)):
        mem = np.nonzero(ginv == g)[0]
        f0 = mem[0]
        k = int(ks[f0])
        if k == 0:
            groups.append((mem, None))
            nrows[mem] = 1
            continue
        ll = tuple(int(x) for x in Ls[f0, :k])
        pattern = tuple(int(x) for x in lab[f0, :k])
        U = rpe_basis(ll, pattern)
        if U.shape[0] == 0:
            groups.append((mem, None))
            continue
        mm = mrange(ll)

        def lookup(sub):
            """AA index of every (member, m-tuple): (len(sub), len(mm))."""
            A = np.stack([aidx[MU[sub, t][:, None], NN[sub, t][:, None], ll[t], (mm[:, t] + maxL)[None, :]]
                          for t in range(k)], axis=2)
            assert np.all(A >= 0)
            A = -np.sort(-A, axis=2)                       # _get_ordered
            r = -np.ones(A.shape[:2] + (maxorder,), dtype=np.int64)
            r[:, :, :k] = A
            pk = _encode(r.reshape(-1, maxorder), base)
            pos = np.searchsorted(skeys, pk)
            if np.any(pos >= len(skeys)) or np.any(skeys[np.minimum(pos, len(skeys) - 1)] != pk):
                raise RuntimeError("bcol_ordered not in AA-spec")
            return korder[pos].reshape(len(sub), -1)

        # members in slices of ~2M (member, m-tuple) entries
        step = max(1, (1 << 21) // max(1, len(mm)))
        parts = []
        for c0 in range(0, len(mem), step):
            cols = lookup(mem[c0:c0 + step])
            if c0 == 0:
                _, first_idx, inv = np.unique(cols[0], return_index=True, return_inverse=True)
                Uc = np.zeros((U.shape[0], len(first_idx)))
                np.add.at(Uc.T, inv, U.T)
                rmax = np.abs(Uc).max(axis=1, keepdims=True)
                Uc[np.abs(Uc) <= zero_tol * rmax] = 0.0
            parts.append(cols[:, first_idx])
        groups.append((mem, (np.concatenate(parts, axis=0), Uc)))
        nrows[mem] = U.shape[0]

    off = np.concatenate([[0], np.cumsum(nrows)])
    nB = int(off[-1])
    has = nrows > 0
    cls = np.cumsum(has) - 1                               # class index of each function with rows
    nclass = int(has.sum())
    Bdeg = np.repeat(dsum, nrows)
    Bclass = np.repeat(cls, nrows)
    Irow, Jcol, vals = [], [], []
    for mem, data in groups:
        if data is None:
            if nrows[mem[0]] == 1:                         # the constant (order 0)
                Irow.append(off[mem]); Jcol.append(ref[mem]); vals.append(np.ones(len(mem)))
            continue
        ccols, Uc = data
        for irow in range(Uc.shape[0]):
            nz = np.nonzero(Uc[irow])[0]
            Irow.append(np.repeat(off[mem] + irow, len(nz)))
            Jcol.append(ccols[:, nz].ravel())
            vals.append(np.tile(Uc[irow, nz], len(mem)))
    return Irow, Jcol, vals, list(Bdeg), list(Bclass), nB, nclass


def symmetric_basis(maxorder: int, maxdeg: float, nR: int | None = None,
                    maxL: int | None = None, nspecies: int = 1,
                    r0: float = 1.0, rcut: float = 5.0, rin: float | None = None,
                    pcut: int = 2, pin: int = 0, p: int = 2,
                    zero_tol: float = 1e-12) -> ACESpec:
    """SymmetricBasis(Invariant(), [Categorical *] RnYlm_1pbasis(maxdeg, maxL),
    SimpleSparseBasis(maxorder, maxdeg)) with cleaning, as ACE.jl builds it."""
    if nR is None:
        nR = int(maxdeg)
    if maxL is None:
        maxL = int(maxdeg)
    radial = rn_basis(maxdeg=nR, r0=r0, rcut=rcut, rin=rin, pcut=pcut, pin=pin, p=p)

    aspec = init1pspec(nR, maxL, maxdeg, nspecies)
    nA0 = len(aspec)
    deg = aspec.degree.astype(np.float64)
    per_order = gensparse_ordered(deg, aspec.l, aspec.m, maxorder, maxdeg)

    # PIBasisSpec: reverse rows (descending), pad with -1
    rows = []
    orders = []
    for k, tup in enumerate(per_order):
        if len(tup) == 0:
            continue
        r = -np.ones((len(tup), maxorder), dtype=np.int64)
        r[:, :k] = tup[:, ::-1]
        rows.append(r)
        orders.append(np.full(len(tup), k, dtype=np.int64))
    iAA2iA = np.concatenate(rows, axis=0)
    orders = np.concatenate(orders)
    nAA0 = len(orders)
    base = nA0 + 1
    keys = _encode(iAA2iA, base)
    korder = np.argsort(keys)
    skeys = keys[korder]

    # dense lookup (mu, n, l, m) -> A index
    aidx = -np.ones((nspecies, nR + 1, maxL + 1, 2 * maxL + 1), dtype=np.int64)
    aidx[aspec.mu, aspec.n, aspec.l, aspec.m + maxL] = np.arange(nA0)

    # coupling over the reference functions (all m == 0), grouped by class
    # signature; row order as one loop over them (_coupling_rows_loop)
    Irow, Jcol, vals, Bdeg, Bclass, nB, nclass = _coupling_rows(
        aspec, iAA2iA, orders, skeys, korder, aidx, base, maxorder, maxL, zero_tol)
    Irow = np.concatenate(Irow); Jcol = np.concatenate(Jcol); vals = np.concatenate(vals)
    Ufull = sp.csr_matrix((vals, (Irow, Jcol)), shape=(nB, nAA0))
    Ufull.sum_duplicates()

    # clean_pibasis!: keep non-zero columns (order preserved)
    colnorm = np.asarray(abs(Ufull).sum(axis=0)).ravel()
    Inz = np.nonzero(colnorm > 0.0)[0]
    U = Ufull[:, Inz].tocsr()
    iAA2iA = iAA2iA[Inz]
    orders = orders[Inz]
    # clean_1pbasis!: keep used A entries (order preserved)
    used = np.zeros(nA0, dtype=bool)
    used[iAA2iA[iAA2iA >= 0]] = True
    new_inds = -np.ones(nA0, dtype=np.int64)
    new_inds[used] = np.arange(used.sum())
    iAA2iA = np.where(iAA2iA >= 0, new_inds[np.maximum(iAA2iA, 0)], -1)
    aspec = OnePSpec(aspec.mu[used], aspec.n[used], aspec.l[used], aspec.m[used])

    info = dict(nA_pre=nA0, nAA_pre=nAA0, nclass=nclass,
                nAA_by_order={int(k): int((orders == k).sum()) for k in np.unique(orders)},
                maxorder=maxorder, maxdeg=maxdeg, nR=nR, maxL=maxL, nspecies=nspecies)
    return ACESpec(radial=radial, maxL=maxL, nspecies=nspecies, aspec=aspec,
                   orders=orders, iAA2iA=iAA2iA, U=U,
                   Bdeg=np.array(Bdeg), Bclass=np.array(Bclass), info=info)


@dataclass
class VectorSpec(ACESpec):
    """An EuclideanVector basis: B_b = Re(sum_k U[b, k] AA_k) in R^3, with
    Uvec = (U_x, U_y, U_z) complex CSR (nB x nAA).  ``U`` (real, used by the
    invariant paths) is empty; ``nB`` counts vector basis functions."""
    Uvec: tuple = ()

    @property
    def nB(self):
        return self.Uvec[0].shape[0]

    def ctilde_vector(self, c: np.ndarray) -> np.ndarray:
        """c~^(i) = U_i^T c for i = x, y, z: complex (3, nAA)."""
        c = np.asarray(c, dtype=np.float64)
        return np.stack([np.asarray(Ui.T @ c).ravel() for Ui in self.Uvec])


def vector_basis(maxorder: int, maxdeg: float, nR: int | None = None, maxL: int | None = None,
                 nspecies: int = 1, r0: float = 1.0, rcut: float = 5.0, rin: float | None = None,
                 pcut: int = 2, pin: int = 0, p: int = 2, zero_tol: float = 1e-12) -> VectorSpec:
    """SymmetricBasis(EuclideanVector(), [Categorical *] RnYlm_1pbasis(maxdeg, maxL),
    SimpleSparseBasis(maxorder, maxdeg)): rotation-equivariant vector basis
    functions (src/properties.jl:154-248), built class by class from the
    coupling tree ended in L = 1 (``coupling.vector_rpe_basis``), cleaned as
    ``symmetric_basis`` cleans.  The orthonormal basis within a class is the
    coupling-tree one, not the reference's SVD rotation (parity unpinned, as
    for invariants)."""
    from .coupling import mrange_L, vector_rpe_basis
    if nR is None:
        nR = int(maxdeg)
    if maxL is None:
        maxL = int(maxdeg)
    radial = rn_basis(maxdeg=nR, r0=r0, rcut=rcut, rin=rin, pcut=pcut, pin=pin, p=p)
    aspec = init1pspec(nR, maxL, maxdeg, nspecies)
    nA0 = len(aspec)
    per_order = gensparse_ordered(aspec.degree.astype(np.float64), aspec.l, aspec.m, maxorder, maxdeg,
                                  prop="vector")
    rows, orders = [], []
    for k, tup in enumerate(per_order):
        if len(tup) == 0:
            continue
        r = -np.ones((len(tup), maxorder), dtype=np.int64)
        r[:, :k] = tup[:, ::-1]
        rows.append(r)
        orders.append(np.full(len(tup), k, dtype=np.int64))
    iAA2iA = np.concatenate(rows, axis=0)
    orders = np.concatenate(orders)
    nAA0 = len(orders)
    base = nA0 + 1
    keys = _encode(iAA2iA, base)
    korder = np.argsort(keys)
    skeys = keys[korder]
    aidx = -np.ones((nspecies, nR + 1, maxL + 1, 2 * maxL + 1), dtype=np.int64)
    aidx[aspec.mu, aspec.n, aspec.l, aspec.m + maxL] = np.arange(nA0)
    a_m = aspec.m
    refmask = np.all(np.where(iAA2iA >= 0, a_m[np.maximum(iAA2iA, 0)] == 0, True), axis=1)
    Irow, Jcol, vals, Bdeg, Bclass = [], [], [], [], []
    nB = 0
    nclass = 0
    for iAA in np.nonzero(refmask)[0]:
        k = int(orders[iAA])
        vs = iAA2iA[iAA, :k]
        ll = tuple(int(x) for x in aspec.l[vs])
        nn = tuple((int(a), int(b)) for a, b in zip(aspec.mu[vs], aspec.n[vs]))
        U = vector_rpe_basis(ll, _nn_pattern(nn))          # (nb, 3, nM)
        if U.shape[0] == 0:
            continue
        mm = mrange_L(ll, 1)
        A = np.stack([aidx[aspec.mu[vs[t]], aspec.n[vs[t]], ll[t], mm[:, t] + maxL] for t in range(k)], axis=1)
        if np.any(A < 0):
            raise RuntimeError("m-tuple outside the 1p basis")
        A = -np.sort(-A, axis=1)
        r = -np.ones((len(A), maxorder), dtype=np.int64)
        r[:, :k] = A
        pk = _encode(r, base)
        pos = np.searchsorted(skeys, pk)
        if np.any(pos >= len(skeys)) or np.any(skeys[np.minimum(pos, len(skeys) - 1)] != pk):
            raise RuntimeError("bcol_ordered not in AA-spec")
        cols = korder[pos]
        ucols, inv = np.unique(cols, return_inverse=True)
        Uc = np.zeros((U.shape[0], 3, len(ucols)), dtype=complex)
        for i in range(3):
            np.add.at(Uc[:, i, :].T, inv, U[:, i, :].T)
        rmax = np.abs(Uc).max(axis=(1, 2), keepdims=True)
        Uc[np.abs(Uc) <= zero_tol * rmax] = 0.0
        d = float(sum(aspec.degree[vs]))
        for irow in range(U.shape[0]):
            nzm = np.any(Uc[irow] != 0, axis=0)
            Irow.append(np.full(int(nzm.sum()), nB)); Jcol.append(ucols[nzm]); vals.append(Uc[irow][:, nzm])
            Bdeg.append(d); Bclass.append(nclass)
            nB += 1
        nclass += 1
    Irow = np.concatenate(Irow); Jcol = np.concatenate(Jcol); V = np.concatenate(vals, axis=1)
    Ufull = [sp.csr_matrix((V[i], (Irow, Jcol)), shape=(nB, nAA0)) for i in range(3)]
    colnorm = sum(np.asarray(abs(Ui).sum(axis=0)).ravel() for Ui in Ufull)
    Inz = np.nonzero(colnorm > 0.0)[0]
    Uvec = tuple(Ui[:, Inz].tocsr() for Ui in Ufull)
    iAA2iA = iAA2iA[Inz]
    orders = orders[Inz]
    used = np.zeros(nA0, dtype=bool)
    used[iAA2iA[iAA2iA >= 0]] = True
    new_inds = -np.ones(nA0, dtype=np.int64)
    new_inds[used] = np.arange(used.sum())
    iAA2iA = np.where(iAA2iA >= 0, new_inds[np.maximum(iAA2iA, 0)], -1)
    aspec = OnePSpec(aspec.mu[used], aspec.n[used], aspec.l[used], aspec.m[used])
    info = dict(nA_pre=nA0, nAA_pre=nAA0, nclass=nclass, prop="vector",
                nAA_by_order={int(k): int((orders == k).sum()) for k in np.unique(orders)},
                maxorder=maxorder, maxdeg=maxdeg, nR=nR, maxL=maxL, nspecies=nspecies)
    return VectorSpec(radial=radial, maxL=maxL, nspecies=nspecies, aspec=aspec, orders=orders, iAA2iA=iAA2iA,
                      U=sp.csr_matrix((0, len(orders))), Bdeg=np.array(Bdeg), Bclass=np.array(Bclass), info=info,
                      Uvec=Uvec)


@dataclass
class SphericalSpec(ACESpec):
    """A SphericalVector{L} basis: complex components B_b^M = sum_k
    U_M[b, k] AA_k, M = -L..L, rotating like Y_L^M (src/properties.jl:431-520);
    Usph = (U_{-L}, ..., U_L), real CSR (nB x nAA)."""
    Usph: tuple = ()
    Lout: int = 0

    @property
    def nB(self):
        return self.Usph[0].shape[0]

    def ctilde_spherical(self, c: np.ndarray) -> np.ndarray:
        """c~^M = U_M^T c, real (2L+1, nAA)."""
        c = np.asarray(c, dtype=np.float64)
        return np.stack([np.asarray(Um.T @ c).ravel() for Um in self.Usph])


def spherical_basis(L: int, maxorder: int, maxdeg: float, nR: int | None = None, maxL: int | None = None,
                    nspecies: int = 1, r0: float = 1.0, rcut: float = 5.0, rin: float | None = None,
                    pcut: int = 2, pin: int = 0, p: int = 2, zero_tol: float = 1e-12) -> SphericalSpec:
    """SymmetricBasis(SphericalVector(L), ...): AA tuples with sum(l) of the
    parity of L and |sum(m)| <= L (src/properties.jl:470-480), per class the
    coupling tree ended in L, permutation-symmetrised (``rpe_basis_L``),
    cleaned as ``symmetric_basis`` cleans.  Parity of U unpinned against the
    reference's SVD rotation, as for invariants."""
    from .coupling import mrange_L, rpe_basis_L
    if nR is None:
        nR = int(maxdeg)
    if maxL is None:
        maxL = int(maxdeg)
    radial = rn_basis(maxdeg=nR, r0=r0, rcut=rcut, rin=rin, pcut=pcut, pin=pin, p=p)
    aspec = init1pspec(nR, maxL, maxdeg, nspecies)
    nA0 = len(aspec)
    per_order = gensparse_ordered(aspec.degree.astype(np.float64), aspec.l, aspec.m, maxorder, maxdeg,
                                  prop=("spherical", L))
    rows, orders = [], []
    for k, tup in enumerate(per_order):
        if len(tup) == 0:
            continue
        r = -np.ones((len(tup), maxorder), dtype=np.int64)
        r[:, :k] = tup[:, ::-1]
        rows.append(r)
        orders.append(np.full(len(tup), k, dtype=np.int64))
    iAA2iA = np.concatenate(rows, axis=0)
    orders = np.concatenate(orders)
    nAA0 = len(orders)
    base = nA0 + 1
    keys = _encode(iAA2iA, base)
    korder = np.argsort(keys)
    skeys = keys[korder]
    aidx = -np.ones((nspecies, nR + 1, maxL + 1, 2 * maxL + 1), dtype=np.int64)
    aidx[aspec.mu, aspec.n, aspec.l, aspec.m + maxL] = np.arange(nA0)
    a_m = aspec.m
    refmask = np.all(np.where(iAA2iA >= 0, a_m[np.maximum(iAA2iA, 0)] == 0, True), axis=1)
    Irow, Jcol, vals, Bdeg, Bclass = [], [], [], [], []
    nB = 0
    nclass = 0
    for iAA in np.nonzero(refmask)[0]:
        k = int(orders[iAA])
        vs = iAA2iA[iAA, :k]
        if k == 0:
            if L != 0:
                continue
            Irow.append(np.array([nB])); Jcol.append(np.array([iAA])); vals.append(np.array([[1.0]]).T[:, :1].T)
            Bdeg.append(0.0); Bclass.append(nclass)
            nB += 1; nclass += 1
            continue
        ll = tuple(int(x) for x in aspec.l[vs])
        nn = tuple((int(a), int(b)) for a, b in zip(aspec.mu[vs], aspec.n[vs]))
        U = rpe_basis_L(ll, _nn_pattern(nn), L)                 # (nb, nM)
        if U.shape[0] == 0:
            continue
        mm = mrange_L(ll, L)
        M = mm.sum(axis=1)
        A = np.stack([aidx[aspec.mu[vs[t]], aspec.n[vs[t]], ll[t], mm[:, t] + maxL] for t in range(k)], axis=1)
        if np.any(A < 0):
            raise RuntimeError("m-tuple outside the 1p basis")
        A = -np.sort(-A, axis=1)
        r = -np.ones((len(A), maxorder), dtype=np.int64)
        r[:, :k] = A
        pk = _encode(r, base)
        pos = np.searchsorted(skeys, pk)
        if np.any(pos >= len(skeys)) or np.any(skeys[np.minimum(pos, len(skeys) - 1)] != pk):
            raise RuntimeError("bcol_ordered not in AA-spec")
        cols = korder[pos]
        ucols, inv = np.unique(cols, return_inverse=True)
        Uc = np.zeros((U.shape[0], 2 * L + 1, len(ucols)))
        for Mi in range(2 * L + 1):
            sel = M == Mi - L
            np.add.at(Uc[:, Mi, :].T, inv[sel], U[:, sel].T)
        rmax = np.abs(Uc).max(axis=(1, 2), keepdims=True)
        Uc[np.abs(Uc) <= zero_tol * rmax] = 0.0
        d = float(sum(aspec.degree[vs]))
        for irow in range(U.shape[0]):
            nzm = np.any(Uc[irow] != 0, axis=0)
            Irow.append(np.full(int(nzm.sum()), nB)); Jcol.append(ucols[nzm]); vals.append(Uc[irow][:, nzm])
            Bdeg.append(d); Bclass.append(nclass)
            nB += 1
        nclass += 1
    Irow = np.concatenate(Irow); Jcol = np.concatenate(Jcol); V = np.concatenate(vals, axis=1)
    Ufull = [sp.csr_matrix((V[i], (Irow, Jcol)), shape=(nB, nAA0)) for i in range(2 * L + 1)]
    colnorm = sum(np.asarray(abs(Ui).sum(axis=0)).ravel() for Ui in Ufull)
    Inz = np.nonzero(colnorm > 0.0)[0]
    Usph = tuple(Ui[:, Inz].tocsr() for Ui in Ufull)
    iAA2iA = iAA2iA[Inz]
    orders = orders[Inz]
    used = np.zeros(nA0, dtype=bool)
    used[iAA2iA[iAA2iA >= 0]] = True
    new_inds = -np.ones(nA0, dtype=np.int64)
    new_inds[used] = np.arange(used.sum())
    iAA2iA = np.where(iAA2iA >= 0, new_inds[np.maximum(iAA2iA, 0)], -1)
    aspec = OnePSpec(aspec.mu[used], aspec.n[used], aspec.l[used], aspec.m[used])
    info = dict(nA_pre=nA0, nAA_pre=nAA0, nclass=nclass, prop=f"spherical{L}",
                nAA_by_order={int(k): int((orders == k).sum()) for k in np.unique(orders)},
                maxorder=maxorder, maxdeg=maxdeg, nR=nR, maxL=maxL, nspecies=nspecies)
    return SphericalSpec(radial=radial, maxL=maxL, nspecies=nspecies, aspec=aspec, orders=orders, iAA2iA=iAA2iA,
                         U=sp.csr_matrix((0, len(orders))), Bdeg=np.array(Bdeg), Bclass=np.array(Bclass),
                         info=info, Usph=Usph, Lout=L)


def random_coefficients(spec: ACESpec, seed: int = 0) -> np.ndarray:
    """c_k ~ N(0,1) / (1 + deg_k)^2, deg_k = sum over the class of (n-1)+l."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal(spec.nB) / (1.0 + spec.Bdeg) ** 2
