"""Import (and export) linear ACE models in the dictionary shape of ACE.jl's
``write_dict``.

ACE.jl saves a model as nested dictionaries (JSON through ACEbase's
``save_json``), each tagged with ``"__id__"``.  The tags and field names below
are the ones ACE.jl's own ``write_dict`` methods produce:

* ``ACE_LinearACEModel`` {basis, c, evaluator}  (``src/linearmodel.jl:80-93``)
* ``ACE_SymmetricBasis`` {pibasis, A2Bmap, symgrp, isreal}
  (``src/symmbasis.jl:50-61``)
* ``ACE_PIBasis`` {basis1p, spec, real}, ``ACE_PIBasisSpec`` {orders,
  iAA2iA}  (``src/pibasis.jl:235-252``)
* ``ACE_Product1pBasis`` {bases, indices}  (``src/product_1pbasis.jl:57-66``)
* ``ACE_B1pComponent`` {syms, basis, fval, spec, degrees, label}
  (``src/b1pcomponent.jl:159-168``) around
  - the radial basis: ``ACE_SChain`` {F} (``src/chain.jl:75-77``) of
    ``ACE_Lambda`` "rr -> norm(rr)", the ``polytransform`` lambda
    "r -> ((1+r0)/(1+r))^p" (``src/transforms/distancetransforms.jl:16``,
    ``src/transforms/lambdas.jl:46-51``) and ``ACE_OrthPolyBasis``
    {pl, tl, pr, tr, A, B, C, tdf, ww} (``src/polynomials/orthpolys.jl:
    119-140``); spec entries {n}
  - the angular basis: ``ACE_SHBasis`` {maxL} (``src/polynomials/
    sphericalharmonics.jl:318-324``); spec entries {l, m}
* ``ACE_Categorical1pBasis`` {categories (``ACE_SList`` {T, list}), VSYM,
  ISYM, label}  (``src/discrete1pbasis.jl:42-51,134-143``)
* ``ACE_Invariant`` {val, T}  (``src/properties.jl:106-112``), the entries
  of A2Bmap.

Three leaf encodings come from ACEbase's FIO module, which is not part of the
reference tree (ACEbase 0.2.4 is a dependency, ``Project.toml``), so the
reader accepts each of the layouts such a file can reasonably hold and the
writer emits the first:

* a matrix (``iAA2iA``): ``{"size": [m, n], "data": [...]}`` with the data in
  Julia's column-major order (any ``"__id__"``), or a list of m rows;
* a sparse matrix (``A2Bmap``): ``{"m", "n", "colptr", "rowval", "nzval"}``,
  1-based CSC as Julia's ``SparseMatrixCSC`` stores it, nzval entries numbers
  or ``ACE_Invariant`` dictionaries (or nzval itself encoded as a vector);
* a vector (``c``, ``A``, ``tdf``, ...): a list of numbers, or a dictionary
  holding it under ``"data"`` or ``"vals"``.

Indices in the dictionary are 1-based as in Julia (``iAA2iA`` padded with 0);
the spec used by this library is 0-based (padded with -1).
"""
from __future__ import annotations

import re

import numpy as np
import scipy.sparse as sp

from .radial import OrthPolyBasis, PolyTransform, RadialBasis
from .spec import ACESpec, OnePSpec

_POLY = re.compile(r"r\s*->\s*\(\(\s*1\s*\+\s*([^)]+?)\s*\)\s*/\s*\(\s*1\s*\+\s*r\s*\)\s*\)\s*\^\s*(\d+)")


# ---------------------------------------------------------------- leaves

def _vector(x, dtype=np.float64) -> np.ndarray:
    if isinstance(x, dict):
        for k in ("data", "vals"):
            if k in x:
                return _vector(x[k], dtype)
        raise ValueError(f"unrecognised vector encoding: keys {sorted(x)}")
    return np.asarray(x, dtype=dtype)


def _matrix(x, dtype=np.int64) -> np.ndarray:
    if isinstance(x, dict):
        m, n = (int(v) for v in x["size"])
        return np.asarray(x["data"], dtype=dtype).reshape((n, m)).T.copy()   # column-major
    a = np.asarray(x, dtype=dtype)
    return a.reshape(len(x), -1) if a.ndim == 1 else a


def _scalar_value(v) -> float:
    if isinstance(v, dict):
        if v.get("__id__") == "ACE_Invariant" or "val" in v:
            return float(v["val"])
        raise ValueError(f"unsupported A2Bmap entry {v.get('__id__')}")
    return float(v)


def _sparse(x) -> sp.csr_matrix:
    """A SparseMatrixCSC (1-based CSC) -> scipy CSR (0-based)."""
    m, n = int(x["m"]), int(x["n"])
    colptr = np.asarray(_vector(x["colptr"], np.int64)) - 1
    rowval = np.asarray(_vector(x["rowval"], np.int64)) - 1
    nz = x["nzval"]
    if isinstance(nz, dict) and not ("val" in nz):
        nz = nz.get("data", nz.get("vals"))
    vals = np.array([_scalar_value(v) for v in nz], dtype=np.float64)
    return sp.csc_matrix((vals, rowval, colptr), shape=(m, n)).tocsr()


def _id(d) -> str:
    return d.get("__id__", "") if isinstance(d, dict) else ""


# ---------------------------------------------------------------- components

def _radial(comp: dict):
    """(OrthPolyBasis, PolyTransform) of the Rn component."""
    chain = comp["basis"]
    F = chain["F"] if _id(chain) == "ACE_SChain" else [chain]
    J = trans = None
    for f in F:
        if _id(f) == "ACE_OrthPolyBasis":
            J = f
        elif _id(f) == "ACE_Lambda":
            mt = _POLY.search(f["exstr"])
            if mt:
                trans = PolyTransform(int(mt.group(2)), float(mt.group(1)))
    if J is None:
        raise ValueError("radial component without an ACE_OrthPolyBasis")
    if trans is None:
        raise ValueError("radial component without a polytransform lambda 'r -> ((1+r0)/(1+r))^p'")
    opb = OrthPolyBasis(int(J["pl"]), float(J["tl"]), int(J["pr"]), float(J["tr"]),
                        _vector(J["A"]), _vector(J["B"]), _vector(J["C"]),
                        _vector(J.get("tdf", [])), _vector(J.get("ww", [])))
    return opb, trans


def _inv_poly(trans: PolyTransform, t: float) -> float:
    """r with ((1 + r0)/(1 + r))^p = t (the reference finds it numerically)."""
    return (1.0 + trans.r0) / t ** (1.0 / trans.p) - 1.0


def from_write_dict(D: dict):
    """(ACESpec, c) of a ``LinearACEModel`` dictionary (or (ACESpec, None) of
    a ``SymmetricBasis`` one)."""
    c = None
    if _id(D) == "ACE_LinearACEModel":
        c = _vector(D["c"])
        D = D["basis"]
    if _id(D) != "ACE_SymmetricBasis":
        raise ValueError(f"expected ACE_LinearACEModel or ACE_SymmetricBasis, got {_id(D)!r}")
    if "isreal" in D and not D["isreal"]:
        raise ValueError("complex-valued SymmetricBasis (isreal = false) is not an invariant model")
    pib = D["pibasis"]
    b1p = pib["basis1p"]
    if _id(b1p) != "ACE_Product1pBasis":
        raise ValueError(f"expected ACE_Product1pBasis, got {_id(b1p)!r}")
    bases = b1p["bases"]
    ind = np.asarray(b1p["indices"], dtype=np.int64).reshape(len(b1p["indices"]), len(bases))
    nA = ind.shape[0]
    n = np.zeros(nA, np.int64); l = np.zeros(nA, np.int64); m = np.zeros(nA, np.int64)
    mu = np.zeros(nA, np.int64)
    nspecies = 1
    radial = None
    have = set()
    for q, comp in enumerate(bases):
        col = ind[:, q] - 1
        if _id(comp) == "ACE_Categorical1pBasis":
            cats = comp["categories"]
            lst = cats["list"] if isinstance(cats, dict) else cats
            nspecies = len(lst)
            mu = col.copy()
            have.add("mu")
            continue
        if _id(comp) != "ACE_B1pComponent":
            raise ValueError(f"unsupported 1p component {_id(comp)!r}")
        spec = comp["spec"]
        inner = comp["basis"]
        if _id(inner) == "ACE_SHBasis":
            ls = np.array([s["l"] for s in spec]); ms = np.array([s["m"] for s in spec])
            l, m = ls[col], ms[col]
            have.add("lm")
        else:
            J, trans = _radial(comp)
            ns = np.array([s["n"] for s in spec])
            n = ns[col]
            tl, tr = J.tl, J.tr
            rr = sorted((_inv_poly(trans, tl), _inv_poly(trans, tr)))
            radial = RadialBasis(trans, J, float(rr[0]), float(rr[1]))
            have.add("n")
    if not {"n", "lm"} <= have:
        raise ValueError("the 1p basis needs a radial (Rn) and an angular (Ylm) component")
    pspec = pib["spec"]
    orders = _vector(pspec["orders"], np.int64)
    iAA = _matrix(pspec["iAA2iA"], np.int64)
    if iAA.shape[0] != len(orders):
        raise ValueError("iAA2iA rows != length(orders)")
    iAA2iA = np.where(iAA > 0, iAA - 1, -1)
    U = _sparse(D["A2Bmap"])
    if U.shape[1] != len(orders):
        raise ValueError("A2Bmap columns != number of AA functions")
    U.sort_indices()
    maxL = int(l.max()) if nA else 0
    for comp in bases:
        if _id(comp) == "ACE_B1pComponent" and _id(comp["basis"]) == "ACE_SHBasis":
            maxL = int(comp["basis"]["maxL"])
    aspec = OnePSpec(mu.astype(np.int64), n.astype(np.int64), l.astype(np.int64), m.astype(np.int64))
    deg = (n - 1) + l
    Bdeg = np.zeros(U.shape[0])
    Uc = U.tocsr()
    for b in range(U.shape[0]):
        cols = Uc.indices[Uc.indptr[b]:Uc.indptr[b + 1]]
        if len(cols):
            k = cols[0]
            Bdeg[b] = deg[iAA2iA[k][iAA2iA[k] >= 0]].sum()
    info = dict(nAA_by_order={int(k): int((orders == k).sum()) for k in np.unique(orders)},
                maxorder=int(iAA2iA.shape[1]), nspecies=nspecies, source="write_dict")
    spec = ACESpec(radial=radial, maxL=maxL, nspecies=nspecies, aspec=aspec, orders=orders,
                   iAA2iA=iAA2iA, U=U, Bdeg=Bdeg, Bclass=np.zeros(U.shape[0], np.int64), info=info)
    return spec, c


# ---------------------------------------------------------------- writer

def _t(name="Float64"):
    return {"__id__": "Type", "T": name}


def to_write_dict(spec: ACESpec, c=None) -> dict:
    """The dictionary ACE.jl's write_dict gives for this model (leaf encodings
    as listed in the module docstring)."""
    R = spec.radial
    J = R.J
    a = spec.aspec
    # component specs: distinct n, (l, m) and species in first-use order
    ns = list(range(1, len(J.A) + 1))
    L = int(spec.maxL)
    lm = [(ll, mm) for ll in range(L + 1) for mm in range(-ll, ll + 1)]
    lm_idx = {v: i for i, v in enumerate(lm)}
    trans = f"r -> ((1+{R.trans.r0!r})/(1+r))^{int(R.trans.p)}"
    rn = {"__id__": "ACE_B1pComponent", "syms": ["n"],
          "basis": {"__id__": "ACE_SChain", "F": [
              {"__id__": "ACE_Lambda", "exstr": "rr -> norm(rr)"},
              {"__id__": "ACE_Lambda", "exstr": trans},
              {"__id__": "ACE_OrthPolyBasis", "T": _t(), "pl": int(J.pl), "tl": float(J.tl), "pr": int(J.pr),
               "tr": float(J.tr), "A": [float(x) for x in J.A], "B": [float(x) for x in J.B],
               "C": [float(x) for x in J.C], "tdf": [float(x) for x in J.tdf], "ww": [float(x) for x in J.ww]}]},
          "fval": {"__id__": "ACE_StaticGet", "expr": "ACE.Transforms.GetVal{:rr}"},
          "spec": [{"n": k} for k in ns], "degrees": [k - 1 for k in ns], "label": "Rn"}
    ylm = {"__id__": "ACE_B1pComponent", "syms": ["l", "m"],
           "basis": {"__id__": "ACE_SHBasis", "T": _t(), "maxL": L},
           "fval": {"__id__": "ACE_StaticGet", "expr": "ACE.Transforms.GetVal{:rr}"},
           "spec": [{"l": ll, "m": mm} for ll, mm in lm], "degrees": [ll for ll, _ in lm], "label": "Ylm"}
    bases = [rn, ylm]
    idx = [[int(a.n[i]), lm_idx[(int(a.l[i]), int(a.m[i]))] + 1] for i in range(len(a))]
    if spec.nspecies > 1:
        cat = {"__id__": "ACE_Categorical1pBasis",
               "categories": {"__id__": "ACE_SList", "T": _t("Int64"), "list": list(range(spec.nspecies))},
               "VSYM": "mu", "ISYM": "mu", "label": "Cmu"}
        bases = [cat] + bases
        idx = [[int(a.mu[i]) + 1] + idx[i] for i in range(len(a))]
    nAA, K = spec.iAA2iA.shape
    iAA = np.where(spec.iAA2iA >= 0, spec.iAA2iA + 1, 0)
    U = spec.U.tocsc()
    U.sort_indices()
    A2B = {"__id__": "SparseMatrixCSC", "m": int(U.shape[0]), "n": int(U.shape[1]),
           "colptr": [int(x) + 1 for x in U.indptr], "rowval": [int(x) + 1 for x in U.indices],
           "nzval": [{"__id__": "ACE_Invariant", "val": float(v), "T": _t()} for v in U.data]}
    basis = {"__id__": "ACE_SymmetricBasis",
             "pibasis": {"__id__": "ACE_PIBasis",
                         "basis1p": {"__id__": "ACE_Product1pBasis", "bases": bases, "indices": idx},
                         "spec": {"__id__": "ACE_PIBasisSpec", "orders": [int(x) for x in spec.orders],
                                  "iAA2iA": {"__id__": "Matrix", "size": [int(nAA), int(K)],
                                             "data": [int(x) for x in iAA.T.ravel()]}},
                         "real": True},
             "A2Bmap": A2B, "symgrp": {"__id__": "ACE_O3", "lsym": "l", "msym": "m"}, "isreal": True}
    if c is None:
        return basis
    return {"__id__": "ACE_LinearACEModel", "basis": basis, "c": [float(x) for x in np.asarray(c)],
            "evaluator": {"__id__": "ACE_ProductEvaluator"}}
