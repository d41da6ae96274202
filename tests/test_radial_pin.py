"""Pins the radial recursion coefficients A, B, C of the restated Stieltjes
procedure (ace_gb300/radial.py, following src/polynomials/orthpolys.jl:
153-218 on the midpoint grid of :340-349) to values derived independently
in 60-digit arithmetic.

The independent route does not run the Stieltjes recursion: it forms the
Gram matrix of the enveloped monomials fcut(t) t^k under the same discrete
measure (the uniform weights on the midpoint grid that discrete_jacobi
builds), takes its Cholesky factor, and reads the three-term coefficients
off the orthonormal polynomials p_n so obtained:
A_n = k_n / k_{n-1} (ratio of leading coefficients),
B_n = -A_n <t p_{n-1}, p_{n-1}>, C_n = -A_n <t p_{n-1}, p_{n-2}>.
The grid, the envelope and the weights are fixed exactly by the reference's
definitions, so the coefficients are too; the float64 restatement must
reproduce them to round-off."""
import numpy as np
import pytest

from ace_gb300.radial import PolyTransform, rn_basis

mp = pytest.importorskip("mpmath")


def _mp_coefficients(N, r0=1.0, rcut=5.0, rin=None, pcut=2, pin=0, p=2, dps=60):
    mp.mp.dps = dps
    if rin is None:
        rin = 0.5 * r0
    tr_ = PolyTransform(p, r0)
    # the transform at the cutoffs, in high precision
    tcut = ((1 + mp.mpf(r0)) / (1 + mp.mpf(rcut))) ** p
    tin = ((1 + mp.mpf(r0)) / (1 + mp.mpf(rin))) ** p
    assert abs(float(tcut) - float(tr_(rcut))) < 1e-15 and abs(float(tin) - float(tr_(rin))) < 1e-15
    if tcut < tin:
        tl, tr, pl, pr = tcut, tin, pcut, pin
    else:
        tl, tr, pl, pr = tin, tcut, pin, pcut
    nq = max(300, 3 * N)
    dt = (tr - tl) / nq
    t = [tl + dt / 2 + (tr - tl - dt) * mp.mpf(i) / (nq - 1) for i in range(nq)]
    w = mp.mpf(1) / nq
    f = [((x - tl) ** pl) * ((x - tr) ** pr) for x in t]
    # Gram matrix of g_k = fcut(t) t^k, k < N
    G = mp.matrix(N, N)
    for i in range(N):
        for j in range(i, N):
            s = mp.fsum(w * f[q] * f[q] * t[q] ** (i + j) for q in range(nq))
            G[i, j] = G[j, i] = s
    Lc = mp.cholesky(G)
    Linv = Lc ** -1   # rows: coefficients of the orthonormal p_n in the g_k
    # values of p_n on the grid
    P = [[mp.fsum(Linv[n, k] * f[q] * t[q] ** k for k in range(n + 1)) for q in range(nq)] for n in range(N)]

    def ip(u, v):
        return mp.fsum(w * a * b for a, b in zip(u, v))
    A = [mp.mpf(0)] * N
    B = [mp.mpf(0)] * N
    C = [mp.mpf(0)] * N
    # P_1 = A_1 fcut: the leading coefficient of p_0 in the g_k is Linv[0, 0]
    A[0] = Linv[0, 0]
    for n in range(1, N):
        A[n] = Linv[n, n] / Linv[n - 1, n - 1]
        tp = [t[q] * P[n - 1][q] for q in range(nq)]
        B[n] = -A[n] * ip(tp, P[n - 1])
        if n >= 2:
            C[n] = -A[n] * ip(tp, P[n - 2])
    return np.array([float(x) for x in A]), np.array([float(x) for x in B]), np.array([float(x) for x in C])


@pytest.mark.parametrize("N", [8, 12, 16])
def test_recursion_coefficients_pinned(N):
    J = rn_basis(maxdeg=N, r0=1.0, rcut=5.0).J
    A, B, C = _mp_coefficients(N)
    # the signs: Cholesky makes every leading coefficient positive, as the
    # Stieltjes normalisation a = sqrt(<J, J>) > 0 does
    for name, x, y in (("A", J.A, A), ("B", J.B, B), ("C", J.C, C)):
        scale = np.max(np.abs(y))
        err = np.max(np.abs(x - y)) / scale
        assert err <= 5e-14, (name, N, err)
