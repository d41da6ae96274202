"""EuclideanVector basis (src/properties.jl:154-248) built on the host:
the basis functions B_b = Re(sum_k U[b,k] AA_k) in R^3 must transform as
vectors under O(3) (B(Q r) = Q B(r), including the inversion), be invariant
under permutations of the neighbours, and be linearly independent -- the
reference's own checks for equivariant bases (test/test_symmbasis.jl)."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import vector_basis


def _rotation(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def vector_B(oracle_mod, spec, offsets, rr, species=None):
    """B (nEnv, nB, 3) through the oracle's A and flat AA products."""
    orc = oracle_mod.Oracle(spec, ctilde=np.zeros(spec.nAA))
    A = orc.A(offsets, rr, species)                     # (nEnv, nA) complex
    AA = np.ones((A.shape[0], spec.nAA), dtype=complex)
    for t in range(spec.maxorder):
        v = spec.iAA2iA[:, t]
        AA = AA * np.where(v >= 0, A[:, np.maximum(v, 0)], 1.0)
    return np.stack([np.real(AA @ Ui.T.toarray()) for Ui in spec.Uvec], axis=2)


@pytest.fixture(scope="module")
def vspec():
    return vector_basis(3, 6, maxL=4)


def test_sizes(vspec):
    assert vspec.info["nAA_by_order"][1] == 18          # l = 1, n = 1..6, m = -1..1
    assert vspec.nB == 121
    assert not np.any(vspec.orders == 0)


def test_equivariance(oracle_mod, vspec):
    b = random_batch(6, 5, 9, seed=3)
    B = vector_B(oracle_mod, vspec, b.offsets, b.rr)
    assert np.max(np.abs(B)) > 1e-3
    for Q in (_rotation(1), _rotation(2), -np.eye(3), -_rotation(4)):
        BQ = vector_B(oracle_mod, vspec, b.offsets, b.rr @ Q.T)
        assert np.allclose(BQ, B @ Q.T, rtol=1e-10, atol=1e-10 * np.max(np.abs(B)))


def test_permutation_invariance(oracle_mod, vspec):
    b = random_batch(4, 6, 6, seed=5)
    rr = b.rr.copy()
    for e in range(b.nenv):
        o0, o1 = b.offsets[e], b.offsets[e + 1]
        rr[o0:o1] = rr[o0:o1][np.random.default_rng(e).permutation(o1 - o0)]
    assert np.allclose(vector_B(oracle_mod, vspec, b.offsets, rr), vector_B(oracle_mod, vspec, b.offsets, b.rr),
                       rtol=1e-11, atol=1e-12)


def test_linear_independence(oracle_mod, vspec):
    b = random_batch(400, 6, 12, seed=7)
    B = vector_B(oracle_mod, vspec, b.offsets, b.rr)              # (nEnv, nB, 3)
    M = B.transpose(0, 2, 1).reshape(-1, vspec.nB)
    s = np.linalg.svd(M, compute_uv=False)
    assert s[-1] / s[0] > 1e-10


# ---------------------------------------------------------------- SphericalVector{L}

def spherical_B(oracle_mod, spec, offsets, rr):
    orc = oracle_mod.Oracle(spec, ctilde=np.zeros(spec.nAA))
    A = orc.A(offsets, rr)
    AA = np.ones((A.shape[0], spec.nAA), dtype=complex)
    for t in range(spec.maxorder):
        v = spec.iAA2iA[:, t]
        AA = AA * np.where(v >= 0, A[:, np.maximum(v, 0)], 1.0)
    return np.stack([AA @ Um.T.toarray() for Um in spec.Usph], axis=2)   # (nEnv, nB, 2L+1)


def wigner_from_sh(oracle_mod, L, Q):
    """D with Y_L(Q x) = D Y_L(x), from the oracle's spherical harmonics."""
    rng = np.random.default_rng(0)
    X = rng.standard_normal((40, 3))
    def YL(x):
        return np.asarray(oracle_mod.sh(L, x))[L * L:(L + 1) ** 2]
    A = np.stack([YL(x) for x in X])                    # (n, 2L+1)
    Bq = np.stack([YL(Q @ x) for x in X])
    D, *_ = np.linalg.lstsq(A, Bq, rcond=None)
    return D.T


@pytest.mark.parametrize("L", [0, 1, 2])
def test_spherical_equivariance(oracle_mod, L):
    from ace_gb300.spec import spherical_basis
    spec = spherical_basis(L, 3, 6, maxL=4)
    b = random_batch(5, 5, 9, seed=11)
    B = spherical_B(oracle_mod, spec, b.offsets, b.rr)
    assert np.max(np.abs(B)) > 1e-3
    for Q in (_rotation(1), _rotation(6)):
        D = wigner_from_sh(oracle_mod, L, Q)
        BQ = spherical_B(oracle_mod, spec, b.offsets, b.rr @ Q.T)
        assert np.allclose(BQ, B @ D.T, rtol=1e-9, atol=1e-9 * np.max(np.abs(B)))
    # inversion: (-1)^L
    Bi = spherical_B(oracle_mod, spec, b.offsets, -b.rr)
    assert np.allclose(Bi, (-1) ** L * B, rtol=1e-10, atol=1e-10 * np.max(np.abs(B)))
    if L == 0:
        from ace_gb300.spec import symmetric_basis
        assert spec.nB == symmetric_basis(3, 6, maxL=4).nB
