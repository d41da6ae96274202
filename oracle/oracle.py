"""ctypes front-end of the FP64 CPU oracle (``ace_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline / reference arm, never by the product.

``Oracle(spec, c)`` holds one linear ACE model (spec + B-basis coefficients
c, with c~ = U^T c as ``src/evaluator.jl:30-31,59-60`` forms it) and exposes
the reference's evaluation entry points:

* ``evaluate``      -- site energies      (``src/evaluator.jl:121-147``)
* ``grad_config``   -- dE/drr_j           (``src/evaluator.jl:161-200``)
* ``basis``         -- B = real(U AA)     (``src/symmbasis.jl:297-316``)
* ``basis_d``       -- B and dB/drr_j     (``src/symmbasis.jl:322-334``)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build(force: bool = False) -> str:
    """Compile liboracle.so in place (gcc, OpenMP, no FMA contraction)."""
    so = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "ace_oracle.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src) or not _native(so):
        subprocess.run(["make", "-C", _HERE, "-B", "liboracle.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return so


def _native(path: str) -> bool:
    """True when the shared object is an ELF file for this host's CPU (one
    compiled on another machine is rebuilt)."""
    import platform
    import struct
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    with open(path, "rb") as f:
        head = f.read(20)
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return want is None or struct.unpack("<H" if head[5] == 1 else ">H", head[18:20])[0] == want


class _Spec(C.Structure):
    _fields_ = [
        ("nR", C.c_int), ("rA", C.c_void_p), ("rB", C.c_void_p), ("rC", C.c_void_p),
        ("pl", C.c_int), ("pr", C.c_int), ("tl", C.c_double), ("tr", C.c_double),
        ("tp", C.c_int), ("r0", C.c_double),
        ("L", C.c_int),
        ("nA", C.c_int), ("a_n", C.c_void_p), ("a_iy", C.c_void_p), ("a_mu", C.c_void_p),
        ("nAA", C.c_int64), ("maxord", C.c_int), ("orders", C.c_void_p), ("iAA2iA", C.c_void_p),
        ("ctilde", C.c_void_p),
        ("nB", C.c_int64), ("U_indptr", C.c_void_p), ("U_indices", C.c_void_p), ("U_data", C.c_void_p),
        ("Rext", C.c_void_p), ("dRext", C.c_void_p),
    ]


def _lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        P = C.c_void_p
        for name in ("oracle_energy", "oracle_grad_config", "oracle_A", "oracle_basis"):
            f = getattr(_LIB, name)
            f.restype = C.c_int
            f.argtypes = [P, C.c_int64, P, P, P, P, C.c_int]
        for name in ("oracle_energy_forces", "oracle_basis_d"):
            f = getattr(_LIB, name)
            f.restype = C.c_int
            f.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int]
        _LIB.oracle_radial_adjoint.restype = C.c_int
        _LIB.oracle_radial_adjoint.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int]
        _LIB.oracle_sh.restype = C.c_int
        _LIB.oracle_sh.argtypes = [C.c_int, P, P, P]
        _LIB.oracle_radial.restype = C.c_int
        _LIB.oracle_radial.argtypes = [P, C.c_int64, P, P, P]
    return _LIB


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Oracle:
    """With ``channels_per_l = K`` the model is the learned-radial form: the
    radial value of A entry (n, l, m) is channel (n-1) + K*l of externally
    supplied per-neighbour radials (``set_radial``), nR = K*(L+1)."""

    def __init__(self, spec, c=None, ctilde=None, channels_per_l=None):
        self.spec = spec
        self.K = channels_per_l
        if ctilde is None:
            if c is None:
                c = np.zeros(spec.nB)
            ctilde = spec.ctilde(c)
        self._keep = {}
        k = self._keep
        R = spec.radial
        k["rA"] = np.ascontiguousarray(R.J.A, dtype=np.float64)
        k["rB"] = np.ascontiguousarray(R.J.B, dtype=np.float64)
        k["rC"] = np.ascontiguousarray(R.J.C, dtype=np.float64)
        a = spec.aspec
        an = a.n - 1 if channels_per_l is None else (a.n - 1) + channels_per_l * a.l
        k["a_n"] = np.ascontiguousarray(an, dtype=np.int32)
        k["a_iy"] = np.ascontiguousarray(a.l * a.l + a.l + a.m, dtype=np.int32)
        k["a_mu"] = np.ascontiguousarray(a.mu, dtype=np.int32) if spec.nspecies > 1 else None
        k["orders"] = np.ascontiguousarray(spec.orders, dtype=np.int32)
        k["iAA2iA"] = np.ascontiguousarray(spec.iAA2iA, dtype=np.int32)
        k["ctilde"] = np.ascontiguousarray(ctilde, dtype=np.float64)
        U = spec.U.tocsr()
        U.sort_indices()
        k["U_indptr"] = np.ascontiguousarray(U.indptr, dtype=np.int64)
        k["U_indices"] = np.ascontiguousarray(U.indices, dtype=np.int32)
        k["U_data"] = np.ascontiguousarray(U.data, dtype=np.float64)
        s = _Spec()
        s.nR = len(R.J.A) if channels_per_l is None else channels_per_l * (spec.Leff + 1)
        s.rA, s.rB, s.rC = _p(k["rA"]), _p(k["rB"]), _p(k["rC"])
        s.pl, s.pr, s.tl, s.tr = R.J.pl, R.J.pr, R.J.tl, R.J.tr
        s.tp, s.r0 = R.trans.p, R.trans.r0
        s.L = spec.Leff
        s.nA = spec.nA
        s.a_n, s.a_iy, s.a_mu = _p(k["a_n"]), _p(k["a_iy"]), _p(k["a_mu"])
        s.nAA, s.maxord = spec.nAA, spec.maxorder
        s.orders, s.iAA2iA, s.ctilde = _p(k["orders"]), _p(k["iAA2iA"]), _p(k["ctilde"])
        s.nB = spec.nB
        s.U_indptr, s.U_indices, s.U_data = _p(k["U_indptr"]), _p(k["U_indices"]), _p(k["U_data"])
        self._s = s

    def set_radial(self, R, dR=None):
        """Per-neighbour radial channels (nNbr x nR) and their r-derivatives
        for the next calls (learned-radial form)."""
        assert self.K is not None
        self._keep["Rext"] = np.ascontiguousarray(R, dtype=np.float64)
        self._keep["dRext"] = np.ascontiguousarray(R * 0 if dR is None else dR, dtype=np.float64)
        assert self._keep["Rext"].shape[1] == self._s.nR
        self._s.Rext, self._s.dRext = _p(self._keep["Rext"]), _p(self._keep["dRext"])

    def radial_adjoint(self, offsets, rr, species=None, nthreads=0):
        """E and dE/dR_n(r_j) (nNbr x nR)."""
        offsets, rr, sp = self._inputs(offsets, rr, species)
        E = np.zeros(len(offsets) - 1)
        GR = np.zeros((len(rr), self._s.nR))
        rc = _lib().oracle_radial_adjoint(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp),
                                          _p(E), _p(GR), nthreads)
        assert rc == 0
        return E, GR

    def set_params(self, c):
        """``set_params!`` (src/linearmodel.jl:67-71): c~ = U^T c."""
        self._keep["ctilde"][:] = self.spec.ctilde(c)

    @staticmethod
    def _inputs(offsets, rr, species):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        rr = np.ascontiguousarray(rr, dtype=np.float64).reshape(-1, 3)
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        return offsets, rr, sp

    def evaluate(self, offsets, rr, species=None, nthreads=0):
        offsets, rr, sp = self._inputs(offsets, rr, species)
        E = np.zeros(len(offsets) - 1)
        rc = _lib().oracle_energy(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp), _p(E), nthreads)
        assert rc == 0
        return E

    def grad_config(self, offsets, rr, species=None, nthreads=0):
        offsets, rr, sp = self._inputs(offsets, rr, species)
        G = np.zeros_like(rr)
        rc = _lib().oracle_grad_config(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp), _p(G), nthreads)
        assert rc == 0
        return G

    def energy_forces(self, offsets, rr, species=None, nthreads=0):
        offsets, rr, sp = self._inputs(offsets, rr, species)
        E = np.zeros(len(offsets) - 1)
        G = np.zeros_like(rr)
        rc = _lib().oracle_energy_forces(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp),
                                         _p(E), _p(G), nthreads)
        assert rc == 0
        return E, G

    def A(self, offsets, rr, species=None, nthreads=0):
        offsets, rr, sp = self._inputs(offsets, rr, species)
        A = np.zeros((len(offsets) - 1, self.spec.nA, 2))
        rc = _lib().oracle_A(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp), _p(A), nthreads)
        assert rc == 0
        return A[..., 0] + 1j * A[..., 1]

    def basis(self, offsets, rr, species=None, nthreads=0):
        offsets, rr, sp = self._inputs(offsets, rr, species)
        B = np.zeros((len(offsets) - 1, self.spec.nB))
        rc = _lib().oracle_basis(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp), _p(B), nthreads)
        assert rc == 0
        return B

    def basis_d(self, offsets, rr, species=None, nthreads=0):
        offsets, rr, sp = self._inputs(offsets, rr, species)
        B = np.zeros((len(offsets) - 1, self.spec.nB))
        dB = np.zeros((len(rr), self.spec.nB, 3))
        rc = _lib().oracle_basis_d(C.byref(self._s), len(offsets) - 1, _p(offsets), _p(rr), _p(sp),
                                   _p(B), _p(dB), nthreads)
        assert rc == 0
        return B, dB

    def radial(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64).ravel()
        nR = self._s.nR
        R = np.zeros((len(r), nR)); dR = np.zeros((len(r), nR))
        assert _lib().oracle_radial(C.byref(self._s), len(r), _p(r), _p(R), _p(dR)) == 0
        return R, dR


def sh(L: int, x, grad: bool = False):
    """Complex Y_l^m (index_y order) at one point; with grad=True through the
    cYlm_ed! path, also returning the 3 Cartesian derivatives."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    nY = (L + 1) ** 2
    Y = np.zeros((nY, 2))
    dY = np.zeros((nY, 3, 2)) if grad else None
    assert _lib().oracle_sh(L, _p(x), _p(Y), _p(dY)) == 0
    Yc = Y[:, 0] + 1j * Y[:, 1]
    if grad:
        return Yc, dY[..., 0] + 1j * dY[..., 1]
    return Yc
