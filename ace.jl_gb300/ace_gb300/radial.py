"""Radial basis construction: transformed, enveloped orthonormal polynomials.

Host-side restatement of the construction half of ACE.jl's radial basis
(evaluation runs on the GPU and, for testing, in the oracle):

* ``polytransform(p, r0)``  -> t(r) = ((1+r0)/(1+r))^p
  (ACE.jl ``src/transforms/distancetransforms.jl:16``)
* ``discrete_jacobi``       -> uniform discrete measure on [tl, tr]
  (``src/polynomials/orthpolys.jl:340-349``)
* ``OrthPolyBasis`` Stieltjes recursion for A, B, C
  (``src/polynomials/orthpolys.jl:153-218``)
* ``Rn_basis`` defaults r0=1, rin=0.5*r0, pcut=2, pin=0
  (``src/utils/utils.jl:28-47``)

The polynomials are P_1 = A_1 fcut(t), P_2 = (A_2 t + B_2) P_1,
P_n = (A_n t + B_n) P_{n-1} + C_n P_{n-2}, with the envelope
fcut(t) = (t - tl)^pl (t - tr)^pr, zero when pl>0 and t<tl or pr>0 and t>tr
(``src/polynomials/orthpolys.jl:32-60,253-306``).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class PolyTransform:
    """t(r) = ((1 + r0) / (1 + r))^p  (distancetransforms.jl:16)."""
    p: int = 2
    r0: float = 1.0

    def __call__(self, r):
        x = (1.0 + self.r0) / (1.0 + np.asarray(r, dtype=np.float64))
        return _ipow(x, self.p)

    def deriv(self, r):
        r = np.asarray(r, dtype=np.float64)
        x = (1.0 + self.r0) / (1.0 + r)
        # d/dr x^p = p x^(p-1) * dx/dr, dx/dr = -(1+r0)/(1+r)^2
        return self.p * _ipow(x, self.p - 1) * (-(1.0 + self.r0) / ((1.0 + r) * (1.0 + r)))


def _ipow(x, p: int):
    """Integer power by repeated multiplication (Julia's literal_pow for the
    small literal exponents that polytransform strings contain)."""
    if p == 0:
        return np.ones_like(x)
    y = x
    for _ in range(p - 1):
        y = y * x
    return y


def fcut(pl, tl, pr, tr, t):
    """Envelope (orthpolys.jl:32,41-46)."""
    t = np.asarray(t, dtype=np.float64)
    v = (t - tl) ** pl * (t - tr) ** pr
    zero = np.zeros_like(t, dtype=bool)
    if pl > 0:
        zero |= t < tl
    if pr > 0:
        zero |= t > tr
    return np.where(zero, 0.0, v)


@dataclass
class OrthPolyBasis:
    """Recursion coefficients of an enveloped orthonormal polynomial basis
    (orthpolys.jl:82-99)."""
    pl: int
    tl: float
    pr: int
    tr: float
    A: np.ndarray
    B: np.ndarray
    C: np.ndarray
    tdf: np.ndarray = field(repr=False)
    ww: np.ndarray = field(repr=False)

    def __len__(self):
        return len(self.A)

    def evaluate(self, t):
        """P_n(t) for n = 1..N (orthpolys.jl:253-263); vectorised over t."""
        t = np.asarray(t, dtype=np.float64)
        N = len(self.A)
        P = np.zeros(t.shape + (N,))
        P[..., 0] = self.A[0] * fcut(self.pl, self.tl, self.pr, self.tr, t)
        if N > 1:
            P[..., 1] = (self.A[1] * t + self.B[1]) * P[..., 0]
        for n in range(2, N):
            P[..., n] = (self.A[n] * t + self.B[n]) * P[..., n - 1] + self.C[n] * P[..., n - 2]
        return P


def orth_poly_basis(N: int, pcut: int, tcut: float, pin: int, tin: float,
                    tdf: np.ndarray, ww: np.ndarray | None = None) -> OrthPolyBasis:
    """Discrete Stieltjes procedure (orthpolys.jl:153-218)."""
    assert pcut >= 0 and pin >= 0 and N > 0
    if tcut < tin:
        tl, tr, pl, pr = tcut, tin, pcut, pin
    else:
        tl, tr, pl, pr = tin, tcut, pin, pcut
    tdf = np.asarray(tdf, dtype=np.float64)
    if ww is None:
        ww = np.ones_like(tdf)
    ww = ww / ww.sum()
    A = np.zeros(N)
    B = np.zeros(N)
    C = np.zeros(N)

    def dotw(f1, f2):
        return float(np.dot(f1, ww * f2))

    J1_ = fcut(pl, tl, pr, tr, tdf)
    a = np.sqrt(dotw(J1_, J1_))
    A[0] = 1.0 / a
    J1 = A[0] * J1_
    if N > 1:
        b = dotw(tdf * J1, J1)
        J2_ = (tdf - b) * J1
        a = np.sqrt(dotw(J2_, J2_))
        A[1] = 1.0 / a
        B[1] = -b / a
        J2 = (A[1] * tdf + B[1]) * J1
        Jprev, Jpprev = J2, J1
    for n in range(2, N):
        b = dotw(tdf * Jprev, Jprev)
        c = dotw(tdf * Jprev, Jpprev)
        J_ = (tdf - b) * Jprev - c * Jpprev
        a = np.sqrt(dotw(J_, J_))
        A[n] = 1.0 / a
        B[n] = -b / a
        C[n] = -c / a
        Jprev, Jpprev = J_ / a, Jprev
    return OrthPolyBasis(pl, float(tl), pr, float(tr), A, B, C, tdf, ww)


def discrete_jacobi(N: int, pcut: int = 0, xcut: float = 1.0, pin: int = 0,
                    xin: float = -1.0, Nquad: int | None = None,
                    trans=lambda x: x) -> OrthPolyBasis:
    """orthpolys.jl:340-349: midpoint grid of Nquad points on [tl, tr] in the
    transformed variable."""
    if Nquad is None:
        Nquad = max(300, 3 * N)
    tcut = float(trans(xcut))
    tin = float(trans(xin))
    tl, tr = min(tin, tcut), max(tin, tcut)
    dt = (tr - tl) / Nquad
    tdf = np.linspace(tl + dt / 2, tr - dt / 2, Nquad)
    return orth_poly_basis(N, pcut, tcut, pin, tin, tdf)


@dataclass
class RadialBasis:
    """R_n(r) = P_n(t(r)), n = 1..maxdeg: ACE.jl's Rn1pBasis
    (b1pcomponents/Rn.jl:17-29) built by Rn_basis (utils/utils.jl:28-47)."""
    trans: PolyTransform
    J: OrthPolyBasis
    rin: float
    rcut: float

    def __len__(self):
        return len(self.J)

    def evaluate(self, r):
        return self.J.evaluate(self.trans(r))


def rn_basis(maxdeg: int = 6, r0: float = 1.0, rcut: float = 2.5,
             rin: float | None = None, pcut: int = 2, pin: int = 0,
             p: int = 2) -> RadialBasis:
    """Rn_basis with ACE.jl's defaults (utils/utils.jl:28-47)."""
    if rin is None:
        rin = 0.5 * r0
    trans = PolyTransform(p, r0)
    J = discrete_jacobi(maxdeg, pcut=pcut, xcut=rcut, pin=pin, xin=rin, trans=trans)
    return RadialBasis(trans, J, float(rin), float(rcut))
