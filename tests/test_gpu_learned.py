"""GPU checks of the learned radial form through the C ABI.

* the MLP forward (R, dR/dr) and backward (parameter gradient) kernels
  against the FP64 numpy restatement (oracle/mlp_oracle.py): 2e-5 and 1e-4
  relative to the largest magnitude; the tensor-core (BF16) inference kernel
  within 2e-2 (R) and 4e-2 (dR/dr);
* energies, forces and the radial adjoint dE/dR of the learned form (FP32)
  against the FP64 C oracle fed the same radial channels: 3e-5 (E), 1e-4
  (dE/drr, dE/dR);
* one Adam step against its formula;
* distillation from a plain 3-species model: the trained network beats the
  same student before training and the method without the network (the
  student spec's species-blind polynomial radials, coefficients fitted the
  same way);
* the force-loss gradient (a Hessian-vector product formed from two exact
  energy gradients) against central differences of the force loss in the
  MLP parameters: 3e-2 relative;
* the plain-model fallback for environments outside the training radii.
"""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.learned import (LearnedRadialModel, RadialMLP, distill, energy_error, fit_coefficients,
                               force_loss_gradient, learned_context, pretrain_radial, student_spec)
from ace_gb300.spec import random_coefficients, symmetric_basis

pytestmark = pytest.mark.gpu

K, NS = 4, 3


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def lib():
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    build()
    return L


@pytest.fixture(scope="module")
def student():
    spec = student_spec(3, 6, K, 4)
    mlp = RadialMLP.init(spec, K=K, nspecies=NS, Q=6, seed=1)
    rng = np.random.default_rng(2)
    mlp.params = (mlp.params + 0.05 * rng.standard_normal(len(mlp.params))).astype(np.float32)
    return spec, mlp


def _torch():
    return pytest.importorskip("torch")


def test_mlp_forward_backward(lib, student):
    import mlp_oracle
    torch = _torch()
    spec, mlp = student
    ctx = learned_context(spec, mlp)
    b = random_batch(40, 3, 30, nspecies=NS, seed=3, rlo=0.5, rhi=5.5)
    n = b.nnbr
    dev = torch.device("cuda", 0)
    rr = torch.from_numpy(b.rr).to(dev)
    sp = torch.from_numpy(b.species).to(dev)
    R = torch.empty((n, 2 * mlp.C), dtype=torch.float32, device=dev)
    ctx.radial_mlp_forward(rr, sp, R)
    torch.cuda.synchronize()
    r = np.linalg.norm(b.rr, axis=1)
    cfg = mlp.feature_config(spec)
    Rref, dRref = mlp_oracle.forward(mlp.params.astype(np.float64), r, b.species, cfg, mlp.C)
    Rg = R.cpu().numpy()
    assert relerr(Rg[:, :mlp.C], Rref) <= 2e-5
    assert relerr(Rg[:, mlp.C:], dRref) <= 1e-4
    rng = np.random.default_rng(4)
    gR = rng.standard_normal((n, mlp.C)).astype(np.float32)
    wj = rng.random(n).astype(np.float32)
    g = torch.zeros(len(mlp.params), dtype=torch.float32, device=dev)
    ctx.radial_mlp_backward(rr, sp, torch.from_numpy(gR).to(dev), torch.from_numpy(wj).to(dev), g)
    torch.cuda.synchronize()
    gref = mlp_oracle.backward(mlp.params.astype(np.float64), r, b.species, gR, wj, cfg, mlp.C)
    assert relerr(g.cpu().numpy(), gref) <= 1e-4
    # inference radials on the tensor cores (BF16 operands, FP32 accumulation)
    Rt = torch.empty_like(R)
    ctx.radial_mlp_infer(rr, sp, Rt)
    torch.cuda.synchronize()
    Rt = Rt.cpu().numpy()
    print("tensor-core inference: R", relerr(Rt[:, :mlp.C], Rref), "dR", relerr(Rt[:, mlp.C:], dRref))
    assert relerr(Rt[:, :mlp.C], Rref) <= 2e-2
    assert relerr(Rt[:, mlp.C:], dRref) <= 4e-2


def _oracle_inputs(spec, mlp, b):
    import mlp_oracle
    r = np.linalg.norm(b.rr, axis=1)
    return mlp_oracle.forward(mlp.params.astype(np.float64), r, b.species, mlp.feature_config(spec), mlp.C)


def test_learned_energy_forces_and_radial_adjoint(lib, oracle_mod, student, monkeypatch):
    torch = _torch()
    monkeypatch.setenv("ACE_B200_MLP", "fp32")   # FP32 radials for oracle parity
    spec, mlp = student
    c = random_coefficients(spec, seed=5)
    ctx = learned_context(spec, mlp)
    ctx.set_params(c)
    b = random_batch(60, 5, 25, nspecies=NS, seed=6)
    E, G = ctx.energy_forces(b.offsets, b.rr, b.species)
    orc = oracle_mod.Oracle(spec, c, channels_per_l=K)
    R, dR = _oracle_inputs(spec, mlp, b)
    orc.set_radial(R, dR)
    Eref, Gref = orc.energy_forces(b.offsets, b.rr, b.species)
    scale = np.maximum(np.abs(Eref), np.sqrt(np.mean(Eref ** 2)))
    assert np.max(np.abs(E - Eref) / scale) <= 3e-5
    assert relerr(G, Gref) <= 1e-4
    # dE/dR_c(r_j) through the device entry point
    dev = torch.device("cuda", 0)
    off = torch.from_numpy(b.offsets).to(dev)
    rr = torch.from_numpy(b.rr).to(dev)
    sp = torch.from_numpy(b.species).to(dev)
    Ed = torch.empty(b.nenv, dtype=torch.float64, device=dev)
    GR = torch.empty((b.nnbr, mlp.C), dtype=torch.float32, device=dev)
    ctx.energy_radial_adjoint(off, rr, sp, Ed, None, GR)
    ctx.sync()
    E2, GRref = orc.radial_adjoint(b.offsets, b.rr, b.species)
    assert np.max(np.abs(Ed.cpu().numpy() - E2) / scale) <= 3e-5
    assert relerr(GR.cpu().numpy(), GRref) <= 1e-4


def test_adam_step(lib, student):
    torch = _torch()
    spec, mlp = student
    ctx = learned_context(spec, mlp)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(7)
    n = 1000
    w0, g, m0, v0 = (rng.standard_normal(n).astype(np.float32) for _ in range(4))
    v0 = np.abs(v0)
    w, m, v = (torch.from_numpy(x.copy()).to(dev) for x in (w0, m0, v0))
    ctx.adam_step(w, torch.from_numpy(g).to(dev), m, v, 1e-2, 3)
    torch.cuda.synchronize()
    b1, b2, eps = 0.9, 0.999, 1e-8
    mr = b1 * m0 + (1 - b1) * g
    vr = b2 * v0 + (1 - b2) * g * g
    wr = w0 - 1e-2 * (mr / (1 - b1 ** 3)) / (np.sqrt(vr / (1 - b2 ** 3)) + eps)
    assert np.allclose(w.cpu().numpy(), wr, rtol=1e-5, atol=1e-6)
    assert np.allclose(m.cpu().numpy(), mr, rtol=1e-6, atol=1e-7)


def test_distillation_gain_and_fallback(lib):
    """Teacher: plain 3-species order-3 / degree-6 model.  Student: K = 4
    learned channels per l.  Training must beat the untrained student."""
    _torch()
    teacher_spec = symmetric_basis(3, 6, maxL=4, nspecies=NS)
    ct = random_coefficients(teacher_spec, seed=8)
    teacher = lib.Context(teacher_spec, "fp64")
    teacher.set_params(ct)
    train = random_batch(3000, 8, 24, nspecies=NS, seed=9)
    test = random_batch(800, 8, 24, nspecies=NS, seed=10)
    Etr, _ = teacher.energy_forces(train.offsets, train.rr, train.species)
    Ete, _ = teacher.energy_forces(test.offsets, test.rr, test.species)
    spec = student_spec(3, 6, K, 4)
    mlp = RadialMLP.init(spec, K=K, nspecies=NS, Q=6, seed=3)
    ctx = learned_context(spec, mlp)
    pretrain_radial(ctx, mlp, spec, nsamples=200_000, steps=400, batch=16384)
    c0 = fit_coefficients(ctx, spec, train, Etr)
    ctx.set_params(c0)
    err0 = energy_error(ctx.energy_forces(test.offsets, test.rr, test.species)[0], Ete)
    c1, hist = distill(ctx, mlp, spec, train, Etr, c0, steps=600, batch_envs=256, lr=2e-3, refit_every=200,
                       refit_envs=3000)
    err1 = energy_error(ctx.energy_forces(test.offsets, test.rr, test.species)[0], Ete)
    # the method without the network: the student spec's own polynomial
    # radials (species-blind, width K), coefficients fitted the same way
    plain = lib.Context(spec, "fp32")
    cp = fit_coefficients(plain, spec, train, Etr)
    plain.set_params(cp)
    err_plain = energy_error(plain.energy_forces(test.offsets, test.rr, test.species)[0], Ete)
    plain.close()
    print("untrained", err0, "trained", err1, "without network", err_plain, "loss", hist[0], hist[-1])
    assert err1["rel_rmse"] < 0.8 * err0["rel_rmse"]
    assert err1["rel_rmse"] < 0.8 * err_plain["rel_rmse"]
    # fallback: an environment with a neighbour inside the training radii's
    # lower bound goes to the plain model, whose energy it reproduces exactly
    model = LearnedRadialModel(spec, mlp, c1, teacher, r_envelope=(0.8, 5.0))
    rr = test.rr.copy()
    rr[test.offsets[2]] *= 0.5 / np.linalg.norm(rr[test.offsets[2]])
    from ace_gb300.configs import Batch
    bt = Batch(test.offsets, rr, test.species)
    E, G, ok = model.energy_forces(bt)
    assert not ok[2] and ok.sum() == test.nenv - 1
    Et2, Gt2 = teacher.energy_forces(test.offsets, rr, test.species)
    assert E[2] == Et2[2]
    o0, o1 = test.offsets[2], test.offsets[3]
    assert np.allclose(G[o0:o1], Gt2[o0:o1], rtol=1e-10, atol=1e-14)
    Es, _ = model.ctx.energy_forces(test.offsets, rr, test.species)
    assert np.allclose(E[ok], Es[ok], rtol=1e-12, atol=0)


def test_learned_basis_and_derivative(lib, oracle_mod, student, monkeypatch):
    """B and dB of the learned form (FP32) against the oracle fed the same
    radial channels: 1e-5 (B) and 1e-4 (dB) relative to the largest
    magnitude."""
    monkeypatch.setenv("ACE_B200_MLP", "fp32")
    spec, mlp = student
    ctx = learned_context(spec, mlp)
    b = random_batch(20, 5, 15, nspecies=NS, seed=12)
    B, dB = ctx.basis(b.offsets, b.rr, b.species, grad=True)
    orc = oracle_mod.Oracle(spec, np.zeros(spec.nB), channels_per_l=K)
    R, dR = _oracle_inputs(spec, mlp, b)
    orc.set_radial(R, dR)
    Bref, dBref = orc.basis_d(b.offsets, b.rr, b.species)
    assert relerr(B, Bref) <= 1e-5
    assert relerr(dB, dBref) <= 1e-4


def test_force_loss_gradient(lib, student, monkeypatch):
    torch = _torch()
    spec, mlp = student
    # the loss below is evaluated with the FP32 MLP that training uses (the
    # inference calls would otherwise take the BF16 tensor-core radials)
    monkeypatch.setenv("ACE_B200_MLP", "fp32")
    ctx = learned_context(spec, mlp, precision="fp64")
    ctx.set_params(random_coefficients(spec, seed=5))
    b = random_batch(8, 8, 20, nspecies=NS, seed=21)
    dev = torch.device("cuda", 0)
    off = torch.from_numpy(b.offsets).to(dev)
    rr = torch.from_numpy(b.rr).to(dev)
    sp = torch.from_numpy(b.species).to(dev)
    E = torch.empty(b.nenv, dtype=torch.float64, device=dev)
    G = torch.empty_like(rr)
    GR = torch.empty((b.nnbr, mlp.C), dtype=torch.float32, device=dev)
    ctx.energy_radial_adjoint(off, rr, sp, E, G, GR)
    rng = np.random.default_rng(22)
    Gt = G + 0.3 * float(G.abs().mean()) * torch.from_numpy(rng.standard_normal((b.nnbr, 3))).to(dev)
    g = torch.zeros(len(mlp.params), dtype=torch.float32, device=dev)
    loss = force_loss_gradient(ctx, g, off, rr, sp, G, Gt, 1.0, E, GR)
    torch.cuda.synchronize()
    g = g.cpu().numpy()

    def loss_at(params):
        ctx.set_radial_mlp(params, mlp.K, mlp.Q, mlp.nspecies, mlp.tmax)
        _, Gp = ctx.energy_forces(b.offsets, b.rr, b.species)
        Gth = Gt.cpu().numpy()
        return float(np.mean((Gp - Gth) ** 2) / np.mean(Gth ** 2))
    assert abs(loss_at(mlp.params) - loss) <= 1e-6 * loss
    for k in np.argsort(-np.abs(g))[:4]:
        d = 2e-3
        p1, p0 = mlp.params.copy(), mlp.params.copy()
        p1[k] += d
        p0[k] -= d
        num = (loss_at(p1) - loss_at(p0)) / (2 * d)
        assert abs(num - g[k]) <= 3e-2 * abs(num), (k, num, g[k])
    ctx.close()
