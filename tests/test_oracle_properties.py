"""Reference property tests restated on the oracle:
A = sum_j phi(X_j) (test/test_1pbasis.jl:45-53), O(3) + permutation
invariance of B (test/test_symmbasis.jl:63-68), linear independence
(test/test_symmbasis.jl:102-110), :standard == :naive == sum(B .* c)
(test/test_linearmodel.jl:50-79), finite-difference gradients
(test/test_pibasis.jl:78-96) and categorical-species invariance
(test/test_discrete.jl:80-88)."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis


@pytest.fixture(scope="module")
def model(oracle_mod):
    spec = symmetric_basis(3, 6, maxL=6, rcut=2.5)
    c = random_coefficients(spec, 1)
    return spec, c, oracle_mod.Oracle(spec, c)


def _rot(seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    return q * np.sign(np.diag(r))


def test_A_is_sum_of_phi(model):
    spec, c, orc = model
    b = random_batch(3, 10, 10, rlo=0.5, rhi=2.5, seed=2)
    A = orc.A(b.offsets, b.rr)
    Asum = 0
    for j in range(10):
        Asum = Asum + orc.A(np.array([0, 1]), b.rr[j:j + 1])[0]
    assert np.allclose(A[0], Asum, rtol=1e-13, atol=1e-13)


def test_invariance(model):
    spec, c, orc = model
    b = random_batch(4, 10, 10, rlo=0.5, rhi=2.5, seed=3)
    B = orc.basis(b.offsets, b.rr)
    for k in range(5):
        Q = _rot(k) * (-1) ** k
        perm = np.random.default_rng(k).permutation(10)
        rr2 = np.concatenate([(b.rr[b.offsets[e]:b.offsets[e + 1]][perm]) @ Q.T for e in range(4)])
        B2 = orc.basis(b.offsets, rr2)
        assert np.allclose(B, B2, rtol=1e-10, atol=1e-12)


def test_linear_independence(model):
    spec, c, orc = model
    b = random_batch(3 * spec.nB, 10, 10, rlo=0.5, rhi=2.5, seed=4)
    B = orc.basis(b.offsets, b.rr)
    assert np.linalg.matrix_rank(B) == spec.nB


def test_standard_naive_reference_agree(model):
    spec, c, orc = model
    for k in range(10):
        b = random_batch(1, 10, 10, rlo=0.5, rhi=2.5, seed=10 + k)
        c = np.random.default_rng(k).random(spec.nB) - 0.5
        orc.set_params(c)
        E = orc.evaluate(b.offsets, b.rr)
        B, dB = orc.basis_d(b.offsets, b.rr)
        assert np.allclose(E, B @ c, rtol=1e-12)
        G = orc.grad_config(b.offsets, b.rr)
        assert np.allclose(G, np.einsum("jbx,b->jx", dB, c), rtol=1e-11, atol=1e-13)


def test_gradient_fd(model):
    spec, c, orc = model
    orc.set_params(c)
    b = random_batch(1, 8, 8, rlo=0.5, rhi=2.5, seed=5)
    G = orc.grad_config(b.offsets, b.rr)
    U = np.random.default_rng(1).standard_normal(b.rr.shape)
    F = lambda t: orc.evaluate(b.offsets, b.rr + t * U)[0]
    errs = []
    for h in (1e-2, 1e-3, 1e-4, 1e-5):
        errs.append(abs((F(h) - F(-h)) / (2 * h) - np.sum(G * U)))
    assert min(errs) < 1e-7 * max(1.0, abs(np.sum(G * U)))


def test_categorical_species_invariance(oracle_mod):
    # two species (test/test_discrete.jl:80-88): B is invariant under O(3)
    # and under permutations that move each neighbour's species with it, and
    # depends on which neighbour carries which species
    spec = symmetric_basis(3, 6, maxL=6, rcut=2.5, nspecies=2)
    orc = oracle_mod.Oracle(spec, random_coefficients(spec, 2))
    b = random_batch(1, 10, 10, rlo=0.5, rhi=2.5, nspecies=2, seed=5)
    B1 = orc.basis(b.offsets, b.rr, b.species)
    for k in range(10):
        Q = _rot(20 + k) * (-1) ** k
        perm = np.random.default_rng(k).permutation(10)
        B2 = orc.basis(b.offsets, b.rr[perm] @ Q.T, b.species[perm])
        assert np.allclose(B1, B2, rtol=1e-10, atol=1e-12)
    flipped = (1 - b.species).astype(b.species.dtype)
    assert not np.allclose(B1, orc.basis(b.offsets, b.rr, flipped), rtol=1e-6)
