"""GPU evaluation of EuclideanVector models (complex AA coefficients through
ace_set_ctilde_complex / ace_energy_forces_multi) against the host
evaluation Re(sum_k c~_k AA_k) from the oracle's A, O(3) covariance and
finite differences of the gradient.  Tolerances: FP64 1e-12 (values) and
1e-7 (gradients vs central differences); fp32x2 1e-6; FP32 3e-5."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.model import LinearVectorModel
from ace_gb300.spec import random_coefficients, vector_basis

pytestmark = pytest.mark.gpu


def _rotation(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


@pytest.fixture(scope="module")
def lib():
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    build()
    return L


@pytest.fixture(scope="module")
def vmodel_inputs():
    spec = vector_basis(3, 8, maxL=6)
    c = random_coefficients(spec, seed=6)
    return spec, c


def host_vector(oracle_mod, spec, c, b):
    orc = oracle_mod.Oracle(spec, ctilde=np.zeros(spec.nAA))
    A = orc.A(b.offsets, b.rr, b.species)
    AA = np.ones((A.shape[0], spec.nAA), dtype=complex)
    for t in range(spec.maxorder):
        v = spec.iAA2iA[:, t]
        AA = AA * np.where(v >= 0, A[:, np.maximum(v, 0)], 1.0)
    return np.real(AA @ spec.ctilde_vector(c).T)          # (nEnv, 3)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32x2", 1e-6), ("fp32", 3e-5)])
def test_vector_model_values(lib, oracle_mod, vmodel_inputs, prec, tol):
    spec, c = vmodel_inputs
    b = random_batch(120, 8, 24, seed=9)
    model = LinearVectorModel(spec, c, precision=prec)
    V = model.evaluate([b.rr[b.offsets[e]:b.offsets[e + 1]] for e in range(b.nenv)])
    Vref = host_vector(oracle_mod, spec, c, b)
    err = np.max(np.abs(V - Vref)) / np.max(np.abs(Vref))
    print(prec, "vector relerr", err)
    assert err <= tol


def test_vector_model_covariance_and_gradient(lib, vmodel_inputs):
    spec, c = vmodel_inputs
    model = LinearVectorModel(spec, c, precision="fp64")
    b = random_batch(30, 8, 16, seed=12)
    cfgs = [b.rr[b.offsets[e]:b.offsets[e + 1]] for e in range(b.nenv)]
    V = model.evaluate(cfgs)
    for Q in (_rotation(3), -np.eye(3), -_rotation(5)):
        VQ = model.evaluate([x @ Q.T for x in cfgs])
        assert np.allclose(VQ, V @ Q.T, rtol=1e-10, atol=1e-10 * np.max(np.abs(V)))
    G = model.grad_config(cfgs)
    h = 1e-5
    for e in (0, 7, 29):
        x = cfgs[e]
        for j in (0, len(x) - 1):
            for a in range(3):
                xp = x.copy(); xp[j, a] += h
                xm = x.copy(); xm[j, a] -= h
                fd = (model.evaluate(xp) - model.evaluate(xm)) / (2 * h)
                assert np.allclose(G[e][j, :, a], fd, rtol=1e-6, atol=1e-7 * np.max(np.abs(V)))


def test_vector_model_after_autotune_to_trie(lib, vmodel_inputs, monkeypatch):
    """Complex coefficients run the item kernels whatever schedule the
    context's real-coefficient calls use."""
    monkeypatch.setenv("ACE_B200_KERNEL", "trie")
    spec, c = vmodel_inputs
    model = LinearVectorModel(spec, c, precision="fp64")
    monkeypatch.delenv("ACE_B200_KERNEL")
    ref = LinearVectorModel(spec, c, precision="fp64")
    b = random_batch(20, 8, 16, seed=2)
    cfgs = [b.rr[b.offsets[e]:b.offsets[e + 1]] for e in range(b.nenv)]
    assert np.allclose(model.evaluate(cfgs), ref.evaluate(cfgs), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("L", [1, 2])
def test_spherical_model(lib, oracle_mod, L):
    """SphericalVector{L} models (complex components) against the host
    evaluation sum_b c_b B_b^M from the oracle's A, and finite differences."""
    from ace_gb300.model import LinearSphericalModel
    from ace_gb300.spec import spherical_basis
    spec = spherical_basis(L, 3, 7, maxL=5)
    c = random_coefficients(spec, seed=3)
    model = LinearSphericalModel(spec, c, precision="fp64")
    b = random_batch(40, 6, 18, seed=4)
    cfgs = [b.rr[b.offsets[e]:b.offsets[e + 1]] for e in range(b.nenv)]
    V = model.evaluate(cfgs)                                   # (nEnv, 2L+1) complex
    orc = oracle_mod.Oracle(spec, ctilde=np.zeros(spec.nAA))
    A = orc.A(b.offsets, b.rr)
    AA = np.ones((A.shape[0], spec.nAA), dtype=complex)
    for t in range(spec.maxorder):
        v = spec.iAA2iA[:, t]
        AA = AA * np.where(v >= 0, A[:, np.maximum(v, 0)], 1.0)
    Vref = AA @ spec.ctilde_spherical(c).T
    assert np.max(np.abs(V - Vref)) <= 1e-12 * np.max(np.abs(Vref))
    G = model.grad_config(cfgs)
    h = 1e-5
    x = cfgs[3]
    for j in (0, len(x) - 1):
        for a in range(3):
            xp = x.copy(); xp[j, a] += h
            xm = x.copy(); xm[j, a] -= h
            fd = (model.evaluate(xp) - model.evaluate(xm)) / (2 * h)
            assert np.allclose(G[3][j, :, a], fd, rtol=1e-6, atol=1e-7 * np.max(np.abs(V)))
