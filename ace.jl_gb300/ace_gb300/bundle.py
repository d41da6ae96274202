"""Versioned spec-bundle files.

A bundle holds everything libace_b200 needs to rebuild a linear ACE model
without re-deriving the basis (in particular without recomputing the coupling
coefficients U, which is the expensive and LAPACK-dependent step of ACE.jl's
construction, ``src/symmbasis.jl:89-162``): the radial recursion, the A spec,
the AA spec, U and optionally the coefficients c.  It plays the role
ACE.jl's ``write_dict``/``read_dict`` of a ``LinearACEModel`` play
(``src/linearmodel.jl:80-93``, ``src/symmbasis.jl:50-61``,
``src/pibasis.jl:235-252``) for this library.

Format: one JSON document ``{"format": "ace-gb300-spec-bundle", "version": 1,
...}`` whose arrays are ``{"dtype", "shape", "data"}`` with little-endian
bytes in base64.
"""
from __future__ import annotations

import base64
import json

import numpy as np
import scipy.sparse as sp

from .radial import OrthPolyBasis, PolyTransform, RadialBasis
from .spec import ACESpec, OnePSpec

FORMAT = "ace-gb300-spec-bundle"
VERSION = 1


def _enc(a) -> dict:
    a = np.ascontiguousarray(a)
    dt = a.dtype.newbyteorder("<")
    return {"dtype": dt.str, "shape": list(a.shape), "data": base64.b64encode(a.astype(dt).tobytes()).decode()}


def _dec(d) -> np.ndarray:
    return np.frombuffer(base64.b64decode(d["data"]), dtype=np.dtype(d["dtype"])).reshape(d["shape"]).copy()


def to_dict(spec: ACESpec, c=None) -> dict:
    R = spec.radial
    U = spec.U.tocsr()
    U.sort_indices()
    d = {
        "format": FORMAT, "version": VERSION,
        "radial": {"p": R.trans.p, "r0": R.trans.r0, "rin": R.rin, "rcut": R.rcut,
                   "pl": R.J.pl, "tl": R.J.tl, "pr": R.J.pr, "tr": R.J.tr,
                   "A": _enc(R.J.A), "B": _enc(R.J.B), "C": _enc(R.J.C),
                   "tdf": _enc(R.J.tdf), "ww": _enc(R.J.ww)},
        "maxL": spec.maxL, "nspecies": spec.nspecies,
        "aspec": {"mu": _enc(spec.aspec.mu), "n": _enc(spec.aspec.n), "l": _enc(spec.aspec.l),
                  "m": _enc(spec.aspec.m)},
        "orders": _enc(spec.orders), "iAA2iA": _enc(spec.iAA2iA),
        "U": {"shape": list(U.shape), "indptr": _enc(U.indptr.astype(np.int64)),
              "indices": _enc(U.indices.astype(np.int32)), "data": _enc(U.data)},
        "Bdeg": _enc(spec.Bdeg), "Bclass": _enc(spec.Bclass),
        "info": {k: (v if not isinstance(v, dict) else {str(a): b for a, b in v.items()})
                 for k, v in spec.info.items()},
    }
    if c is not None:
        d["c"] = _enc(np.asarray(c, dtype=np.float64))
    return d


def from_dict(d: dict):
    if d.get("format") != FORMAT:
        raise ValueError("not an ace-gb300 spec bundle")
    if int(d.get("version", -1)) > VERSION:
        raise ValueError(f"bundle version {d.get('version')} is newer than this reader ({VERSION})")
    r = d["radial"]
    J = OrthPolyBasis(int(r["pl"]), float(r["tl"]), int(r["pr"]), float(r["tr"]),
                      _dec(r["A"]), _dec(r["B"]), _dec(r["C"]), _dec(r["tdf"]), _dec(r["ww"]))
    radial = RadialBasis(PolyTransform(int(r["p"]), float(r["r0"])), J, float(r["rin"]), float(r["rcut"]))
    a = d["aspec"]
    aspec = OnePSpec(_dec(a["mu"]), _dec(a["n"]), _dec(a["l"]), _dec(a["m"]))
    Ud = d["U"]
    U = sp.csr_matrix((_dec(Ud["data"]), _dec(Ud["indices"]), _dec(Ud["indptr"])), shape=tuple(Ud["shape"]))
    info = dict(d.get("info", {}))
    if "nAA_by_order" in info:
        info["nAA_by_order"] = {int(k): v for k, v in info["nAA_by_order"].items()}
    spec = ACESpec(radial=radial, maxL=int(d["maxL"]), nspecies=int(d["nspecies"]), aspec=aspec,
                   orders=_dec(d["orders"]), iAA2iA=_dec(d["iAA2iA"]), U=U,
                   Bdeg=_dec(d["Bdeg"]), Bclass=_dec(d["Bclass"]), info=info)
    c = _dec(d["c"]) if "c" in d else None
    return spec, c


def save(path: str, spec: ACESpec, c=None) -> None:
    with open(path, "w") as f:
        json.dump(to_dict(spec, c), f)


def load(path: str):
    with open(path) as f:
        return from_dict(json.load(f))
