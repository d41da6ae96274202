"""GPU parity: libace_b200 (through its C ABI) against the FP64 CPU oracle.

Tolerances (relative to the largest magnitude of the compared quantity):
  FP64 mode: energies 1e-12, gradients 1e-10, basis 1e-12
  FP32 mode (plain FP32 products, no compensation): energies 3e-5, gradients 1e-4
  FP32X2 mode (double-float energy path, FP32 adjoint): energies 1e-6 (the bar
  for the chosen form), gradients 1e-5
  FP32C mode (double-float A, FP32 products and adjoint, first-order energy
  correction): energies 1e-6, gradients 1e-5; its basis path is FP32X2's
"""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

pytestmark = pytest.mark.gpu

TOL = {"fp64": dict(E=1e-12, G=1e-10, B=1e-12), "fp32": dict(E=3e-5, G=1e-4, B=1e-5),
       "fp32x2": dict(E=1e-6, G=1e-5, B=1e-11), "fp32c": dict(E=1e-6, G=1e-5, B=1e-11)}


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def energy_relerr(E, Eref):
    # per-environment relative error, normalised by |E| (floored at the rms energy)
    scale = np.maximum(np.abs(Eref), np.sqrt(np.mean(Eref ** 2)))
    return float(np.max(np.abs(E - Eref) / scale))


@pytest.fixture(scope="module")
def lib():
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    build()
    return L


SPECS = {
    "test": dict(maxorder=3, maxdeg=6, maxL=6, rcut=5.0),
    "cfg1": dict(maxorder=3, maxdeg=8, maxL=6),
    "cfg2": dict(maxorder=4, maxdeg=12, maxL=12),
    "ord5": dict(maxorder=5, maxdeg=10, maxL=10),
    # order 5 / degree 16 / L 16: 1,310,316 AA functions, 55,420 B functions
    "ord5_deg16": dict(maxorder=5, maxdeg=16, maxL=16),
    # 4 species, order 4 / degree 10 / L 10: 1,830,429 AA functions
    "ord4_deg10_4sp": dict(maxorder=4, maxdeg=10, maxL=10, nspecies=4),
}
_spec_cache = {}


def get_spec(name):
    if name not in _spec_cache:
        _spec_cache[name] = symmetric_basis(**SPECS[name])
    return _spec_cache[name]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
@pytest.mark.parametrize("name,nenv,jlo,jhi", [("test", 64, 10, 10), ("cfg1", 1000, 12, 24),
                                               ("cfg2", 200, 20, 60), ("ord5", 100, 20, 40)])
def test_energy_forces(lib, oracle_mod, prec, name, nenv, jlo, jhi):
    spec = get_spec(name)
    c = random_coefficients(spec, seed=11)
    b = random_batch(nenv, jlo, jhi, seed=5)
    orc = oracle_mod.Oracle(spec, c)
    Eref, Gref = orc.energy_forces(b.offsets, b.rr)
    ctx = lib.Context(spec, prec)
    ctx.set_params(c)
    E, G = ctx.energy_forces(b.offsets, b.rr)
    print(f"{name} {prec}: E relerr {energy_relerr(E, Eref):.3g}  G relerr {relerr(G, Gref):.3g}")
    assert energy_relerr(E, Eref) <= TOL[prec]["E"], energy_relerr(E, Eref)
    assert relerr(G, Gref) <= TOL[prec]["G"], relerr(G, Gref)
    # energy-only entry point
    E2 = ctx.energy_forces(b.offsets, b.rr, forces=False)
    assert energy_relerr(E2, Eref) <= TOL[prec]["E"]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
def test_multispecies(lib, oracle_mod, prec):
    spec = symmetric_basis(3, 6, maxL=6, nspecies=3)
    c = random_coefficients(spec, seed=2)
    b = random_batch(50, 8, 30, nspecies=3, seed=9)
    orc = oracle_mod.Oracle(spec, c)
    Eref, Gref = orc.energy_forces(b.offsets, b.rr, b.species)
    ctx = lib.Context(spec, prec)
    ctx.set_params(c)
    E, G = ctx.energy_forces(b.offsets, b.rr, b.species)
    assert energy_relerr(E, Eref) <= TOL[prec]["E"]
    assert relerr(G, Gref) <= TOL[prec]["G"]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
@pytest.mark.parametrize("path", ["fused", "materialised"])
@pytest.mark.parametrize("name,nenv,ns", [("cfg1", 300, 1), ("cfg2", 40, 1), ("species", 30, 3)])
def test_basis(lib, oracle_mod, prec, path, name, nenv, ns, monkeypatch):
    """B = U real(AA): the fused kernel (AA never in memory) and the
    AA-scratch path, against the oracle."""
    monkeypatch.setenv("ACE_B200_BASIS", path)
    spec = symmetric_basis(3, 6, maxL=6, nspecies=3) if name == "species" else get_spec(name)
    b = random_batch(nenv, 12, 24, nspecies=ns, seed=4)
    orc = oracle_mod.Oracle(spec)
    Bref = orc.basis(b.offsets, b.rr, b.species)
    ctx = lib.Context(spec, prec)
    B = ctx.basis(b.offsets, b.rr, b.species)
    assert relerr(B, Bref) <= TOL[prec]["B"]


def test_edge_cases(lib, oracle_mod):
    spec = get_spec("test")
    c = random_coefficients(spec, seed=1)
    ctx = lib.Context(spec, "fp64")
    ctx.set_params(c)
    ct = spec.ctilde(c)
    # empty environments (the reference raises; here E = c~_0), ragged sizes, J = 1
    offsets = np.array([0, 0, 1, 1, 4, 4], dtype=np.int64)
    rr = np.random.default_rng(0).standard_normal((4, 3)) + 1.0
    E, G = ctx.energy_forces(offsets, rr)
    orc = oracle_mod.Oracle(spec, c)
    for e in (1, 3):
        o = slice(offsets[e], offsets[e + 1])
        Er, Gr = orc.energy_forces(np.array([0, offsets[e + 1] - offsets[e]]), rr[o])
        assert abs(E[e] - Er[0]) <= 1e-12 * max(1, abs(Er[0]))
        assert np.allclose(G[o], Gr, rtol=1e-10, atol=1e-14)
    for e in (0, 2, 4):
        assert E[e] == ct[0]
    # zero environments
    E0, G0 = ctx.energy_forces(np.zeros(1, dtype=np.int64), np.zeros((0, 3)))
    assert E0.shape == (0,)
    # beyond the cutoff: R vanishes, only the constant remains
    far = np.array([[6.0, 0.0, 0.0], [0.0, 7.0, 0.0]])
    E1, G1 = ctx.energy_forces(np.array([0, 2]), far)
    assert abs(E1[0] - ct[0]) < 1e-14 and np.all(G1 == 0)


def test_invalid_inputs_rejected(lib):
    spec = get_spec("test")
    ctx = lib.Context(spec, "fp64")
    rr = np.ones((3, 3))
    with pytest.raises(lib.AceError):
        ctx.energy_forces(np.array([0, 2, 1]), rr)          # non-monotone offsets
    with pytest.raises(lib.AceError):
        ctx.energy_forces(np.array([1, 3]), rr)             # offsets[0] != 0
    bad = rr.copy(); bad[1, 0] = np.nan
    with pytest.raises(lib.AceError):
        ctx.energy_forces(np.array([0, 3]), bad)            # non-finite position
    bad = rr.copy(); bad[2] = 0
    with pytest.raises(lib.AceError):
        ctx.energy_forces(np.array([0, 3]), bad)            # r == 0
    with pytest.raises(lib.AceError):
        ctx.set_params(np.zeros(spec.nB + 1))               # wrong length
    spec3 = symmetric_basis(2, 4, maxL=4, nspecies=2)
    ctx3 = lib.Context(spec3, "fp64")
    with pytest.raises(lib.AceError):
        ctx3.energy_forces(np.array([0, 3]), rr, np.array([0, 1, 2]))  # species out of range


def test_device_pointer_path(lib, oracle_mod):
    torch = pytest.importorskip("torch")
    spec = get_spec("cfg1")
    c = random_coefficients(spec, seed=3)
    b = random_batch(500, 12, 24, seed=8)
    orc = oracle_mod.Oracle(spec, c)
    Eref, Gref = orc.energy_forces(b.offsets, b.rr)
    ctx = lib.Context(spec, "fp64")
    ctx.set_params(c)
    off = torch.from_numpy(b.offsets).cuda()
    rr = torch.from_numpy(b.rr).cuda()
    E = torch.empty(b.nenv, dtype=torch.float64, device="cuda")
    G = torch.empty_like(rr)
    stream = torch.cuda.current_stream().cuda_stream
    ctx.energy_forces_device(off, rr, None, E, G, stream=stream, sync=False)
    ctx.sync()
    assert energy_relerr(E.cpu().numpy(), Eref) <= 1e-12
    assert relerr(G.cpu().numpy(), Gref) <= 1e-10


def test_model_api_gradients(lib, oracle_mod):
    from ace_gb300.model import LinearACEModel, SymmetricBasis
    basis = SymmetricBasis(spec=get_spec("test"))
    c = random_coefficients(basis.spec, seed=5)
    model = LinearACEModel(basis, c)
    b = random_batch(4, 10, 10, seed=6)
    cfgs = [b.env(e)[0] for e in range(4)]
    dB = model.grad_params_config(cfgs)              # list of (nB, J, 3)
    g = model.grad_config(cfgs)
    for e in range(4):
        assert np.allclose(np.einsum("bjx,b->jx", dB[e], c), g[e], rtol=1e-10, atol=1e-13)


def test_model_api(lib, oracle_mod):
    from ace_gb300.model import LinearACEModel, SymmetricBasis
    basis = SymmetricBasis(spec=get_spec("test"))
    c = random_coefficients(basis.spec, seed=5)
    model = LinearACEModel(basis, c)
    b = random_batch(5, 10, 10, seed=6)
    cfgs = [b.env(e)[0] for e in range(5)]
    E = model.evaluate(cfgs)
    orc = oracle_mod.Oracle(basis.spec, c)
    assert np.allclose(E, orc.evaluate(b.offsets, b.rr), rtol=1e-12)
    assert np.isclose(model.evaluate(cfgs[0]), E[0], rtol=1e-14)
    g = model.grad_config(cfgs)
    assert np.allclose(np.concatenate(g), orc.grad_config(b.offsets, b.rr), rtol=1e-10, atol=1e-14)
    B = model.grad_params(cfgs)
    assert np.allclose(B @ c, E, rtol=1e-12)
    c2 = random_coefficients(basis.spec, seed=7)
    model.set_params(c2)
    assert np.allclose(model.evaluate(cfgs), B @ c2, rtol=1e-11)


@pytest.mark.parametrize("prec", ["fp64", "fp32x2", "fp32"])
@pytest.mark.parametrize("name,nenv,ns", [("test", 20, 1), ("cfg1", 40, 1), ("species", 15, 3)])
def test_basis_derivative(lib, oracle_mod, prec, name, nenv, ns):
    """evaluate_ed / grad_params_config: dB_b/drr_j against the oracle."""
    spec = get_spec(name) if name != "species" else symmetric_basis(3, 6, maxL=6, nspecies=3)
    b = random_batch(nenv, 8, 20, nspecies=ns, seed=12)
    orc = oracle_mod.Oracle(spec)
    Bref, dBref = orc.basis_d(b.offsets, b.rr, b.species)
    ctx = lib.Context(spec, prec)
    B, dB = ctx.basis(b.offsets, b.rr, b.species, grad=True)
    tol = {"fp64": 1e-11, "fp32x2": 1e-11, "fp32": 1e-4}[prec]
    assert relerr(B, Bref) <= tol * 10
    assert relerr(dB, dBref) <= tol, relerr(dB, dBref)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_adjoint_eval_d(lib, oracle_mod, prec):
    """adjoint_EVAL_D (src/evaluator.jl:204-244): sum_j w_j . dB/drr_j."""
    spec = get_spec("cfg1")
    b = random_batch(30, 12, 24, seed=21)
    w = np.random.default_rng(2).standard_normal(b.rr.shape)
    orc = oracle_mod.Oracle(spec)
    _, dBref = orc.basis_d(b.offsets, b.rr)
    ref = np.stack([np.einsum("jbx,jx->b", dBref[b.offsets[e]:b.offsets[e + 1]], w[b.offsets[e]:b.offsets[e + 1]])
                    for e in range(b.nenv)])
    ctx = lib.Context(spec, prec)
    out = ctx.adjoint_eval_d(b.offsets, b.rr, w)
    tol = {"fp64": 1e-11, "fp32": 1e-4}[prec]
    assert relerr(out, ref) <= tol, relerr(out, ref)


@pytest.mark.parametrize("prec", ["fp64", "fp32x2", "fp32c"])
def test_multi_property(lib, oracle_mod, prec):
    """Multi-property model (c::Vector{SVector{N}}): each property equals the
    single-property evaluation with that column of coefficients."""
    from ace_gb300.model import LinearACEModel, SymmetricBasis
    spec = get_spec("cfg1")
    rng = np.random.default_rng(8)
    C3 = np.stack([random_coefficients(spec, seed=s) for s in (1, 2, 3)], axis=1)   # (nB, 3)
    b = random_batch(50, 12, 24, seed=13)
    ctx = lib.Context(spec, prec)
    ctx.set_params_multi(C3)
    E, G = ctx.energy_forces_multi(b.offsets, b.rr)
    assert E.shape == (50, 3) and G.shape == (len(b.rr), 3, 3)
    for p in range(3):
        Eref, Gref = oracle_mod.Oracle(spec, C3[:, p]).energy_forces(b.offsets, b.rr)
        assert energy_relerr(E[:, p], Eref) <= TOL[prec]["E"]
        assert relerr(G[:, p], Gref) <= TOL[prec]["G"]
    model = LinearACEModel(SymmetricBasis(spec=spec, precision=prec), C3)
    Em = model.evaluate([b.env(e)[0] for e in range(3)])
    assert Em.shape == (3, 3) and np.allclose(Em, E[:3], rtol=1e-12)


@pytest.mark.parametrize("prec", ["fp32x2", "fp32c"])
def test_autotune_keeps_results(lib, oracle_mod, prec):
    torch = pytest.importorskip("torch")
    spec = get_spec("cfg1")
    c = random_coefficients(spec, seed=3)
    b = random_batch(2000, 12, 24, seed=8)
    Eref, Gref = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr)
    ctx = lib.Context(spec, prec)
    ctx.set_params(c)
    off = torch.from_numpy(b.offsets).cuda(); rr = torch.from_numpy(b.rr).cuda()
    E = torch.empty(b.nenv, dtype=torch.float64, device="cuda"); G = torch.empty_like(rr)
    choice = ctx.autotune(off, rr, None, E, G, reps=1)
    assert choice % 1000 in (16, 24, 32, 40, 48, 64)
    if prec == "fp32c":
        assert choice >= 1000  # the compensated form runs on the item schedule only
    E2, G2 = ctx.energy_forces(b.offsets, b.rr)
    assert energy_relerr(E2, Eref) <= TOL[prec]["E"]
    assert relerr(G2, Gref) <= TOL[prec]["G"]


def test_cuda_graph_capture(lib, oracle_mod):
    """The device-pointer call (no synchronisation, no allocation) can be
    captured into a CUDA graph and replayed on new positions."""
    torch = pytest.importorskip("torch")
    spec = get_spec("cfg1")
    c = random_coefficients(spec, seed=3)
    b = random_batch(500, 12, 24, seed=8)
    ctx = lib.Context(spec, "fp64")
    ctx.set_params(c)
    off = torch.from_numpy(b.offsets).cuda(); rr = torch.from_numpy(b.rr).cuda()
    E = torch.empty(b.nenv, dtype=torch.float64, device="cuda"); G = torch.empty_like(rr)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.energy_forces_device(off, rr, None, E, G, stream=s.cuda_stream, sync=False)  # warm-up, outside capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ctx.energy_forces_device(off, rr, None, E, G, stream=s.cuda_stream, sync=False)
    b2 = random_batch(500, 12, 24, seed=9)
    # same neighbour counts are required for a replay: reuse the offsets, move the positions
    rr2 = b2.rr[:len(b.rr)] if len(b2.rr) >= len(b.rr) else np.resize(b2.rr, b.rr.shape)
    rr.copy_(torch.from_numpy(np.ascontiguousarray(rr2)))
    g.replay()
    torch.cuda.synchronize()
    ctx.sync()
    Eref, Gref = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, rr2)
    assert energy_relerr(E.cpu().numpy(), Eref) <= 1e-12
    assert relerr(G.cpu().numpy(), Gref) <= 1e-10


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
def test_order5_degree16(lib, oracle_mod, prec):
    """The order-5 / degree-16 basis (J = 30) against the oracle."""
    spec = get_spec("ord5_deg16")
    c = random_coefficients(spec, seed=4)
    b = random_batch(12, 30, 30, seed=21)
    orc = oracle_mod.Oracle(spec, c)
    Eref, Gref = orc.energy_forces(b.offsets, b.rr)
    ctx = lib.Context(spec, prec)
    ctx.set_params(c)
    E, G = ctx.energy_forces(b.offsets, b.rr)
    print(f"ord5_deg16 {prec}: E relerr {energy_relerr(E, Eref):.3g}  G relerr {relerr(G, Gref):.3g}")
    assert energy_relerr(E, Eref) <= TOL[prec]["E"]
    assert relerr(G, Gref) <= TOL[prec]["G"]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
def test_four_species_bimodal(lib, oracle_mod, prec):
    """4 species, order 4 / degree 10, neighbour counts 60 % U{40..80} and
    40 % U{8..20}, against the oracle."""
    spec = get_spec("ord4_deg10_4sp")
    c = random_coefficients(spec, seed=8)
    b = random_batch(16, 8, 80, nspecies=4, seed=13, bimodal=(0.6, (40, 80), (8, 20)))
    orc = oracle_mod.Oracle(spec, c)
    Eref, Gref = orc.energy_forces(b.offsets, b.rr, b.species)
    ctx = lib.Context(spec, prec)
    ctx.set_params(c)
    E, G = ctx.energy_forces(b.offsets, b.rr, b.species)
    print(f"ord4_deg10_4sp {prec}: E relerr {energy_relerr(E, Eref):.3g}  G relerr {relerr(G, Gref):.3g}")
    assert energy_relerr(E, Eref) <= TOL[prec]["E"]
    assert relerr(G, Gref) <= TOL[prec]["G"]


def _rotation(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def test_full_size_order4_degree12(lib, oracle_mod):
    """The full order-4 / degree-12 workload (100,000 environments, J in
    U{20..60}): the chosen fp32x2 form against the FP64 form on every
    environment, the FP64 form against the oracle on a sample, O(3)
    invariance of the energies and covariance of the gradients under a
    rotation and a reflection, and invariance under a permutation of each
    environment's neighbours."""
    spec = get_spec("cfg2")
    c = random_coefficients(spec, seed=2024)
    b = random_batch(100_000, 20, 60, seed=2024)
    c64 = lib.Context(spec, "fp64"); c64.set_params(c)
    cx2 = lib.Context(spec, "fp32x2"); cx2.set_params(c)
    E64, G64 = c64.energy_forces(b.offsets, b.rr)
    E, G = cx2.energy_forces(b.offsets, b.rr)
    assert energy_relerr(E, E64) <= 1e-6
    assert relerr(G, G64) <= TOL["fp32x2"]["G"]
    # oracle on a sample of 300 environments spread over the batch
    idx = np.random.default_rng(0).choice(b.nenv, 300, replace=False)
    off = np.concatenate([[0], np.cumsum(np.diff(b.offsets)[idx])])
    rr = np.concatenate([b.rr[b.offsets[e]:b.offsets[e + 1]] for e in idx])
    Eo, Go = oracle_mod.Oracle(spec, c).energy_forces(off, rr)
    assert energy_relerr(E64[idx], Eo) <= 1e-12
    Gs = np.concatenate([G64[b.offsets[e]:b.offsets[e + 1]] for e in idx])
    assert relerr(Gs, Go) <= 1e-10
    # O(3): E(Q r) = E(r), G(Q r) = Q G(r)
    for Q in (_rotation(1), -_rotation(2)):
        Er, Gr = cx2.energy_forces(b.offsets, b.rr @ Q.T)
        assert energy_relerr(Er, E) <= 1e-6
        assert relerr(Gr, G @ Q.T) <= 2 * TOL["fp32x2"]["G"]
    # permutation of the neighbours inside every environment
    rng = np.random.default_rng(3)
    perm = np.concatenate([b.offsets[e] + rng.permutation(b.offsets[e + 1] - b.offsets[e])
                           for e in range(b.nenv)])
    Ep, Gp = cx2.energy_forces(b.offsets, b.rr[perm])
    assert energy_relerr(Ep, E) <= 1e-6
    assert relerr(Gp, G[perm]) <= 2 * TOL["fp32x2"]["G"]


def test_host_pipeline(lib, oracle_mod):
    """Large host-buffer calls run as a chunked copy/compute pipeline: the
    results equal the device-pointer call, and an invalid position in a late
    chunk is still reported."""
    torch = pytest.importorskip("torch")
    spec = get_spec("test")
    c = random_coefficients(spec, seed=3)
    ctx = lib.Context(spec, "fp64")
    ctx.set_params(c)
    b = random_batch(20000, 4, 12, seed=17)
    E, G = ctx.energy_forces(b.offsets, b.rr)
    dev = torch.device("cuda", 0)
    off_d = torch.from_numpy(b.offsets).to(dev)
    rr_d = torch.from_numpy(b.rr).to(dev)
    Ed = torch.empty(b.nenv, dtype=torch.float64, device=dev)
    Gd = torch.empty_like(rr_d)
    ctx.energy_forces_device(off_d, rr_d, None, Ed, Gd)
    assert np.array_equal(E, Ed.cpu().numpy())
    assert np.allclose(G, Gd.cpu().numpy(), rtol=1e-12, atol=1e-15)
    idx = np.random.default_rng(0).choice(b.nenv, 50, replace=False)
    off = np.concatenate([[0], np.cumsum(np.diff(b.offsets)[idx])])
    rr = np.concatenate([b.rr[b.offsets[e]:b.offsets[e + 1]] for e in idx])
    Eo, Go = oracle_mod.Oracle(spec, c).energy_forces(off, rr)
    assert energy_relerr(E[idx], Eo) <= 1e-12
    bad = b.rr.copy()
    bad[b.offsets[19990]] = np.nan
    with pytest.raises(lib.AceError):
        ctx.energy_forces(b.offsets, bad)
    # the context stays usable
    E2, _ = ctx.energy_forces(b.offsets, b.rr)
    assert np.array_equal(E2, E)


def test_host_pipeline_species(lib):
    """The host pipeline with a multi-species spec and species arrays."""
    torch = pytest.importorskip("torch")
    spec = symmetric_basis(3, 6, maxL=6, nspecies=3)
    c = random_coefficients(spec, seed=7)
    ctx = lib.Context(spec, "fp32x2")
    ctx.set_params(c)
    b = random_batch(12000, 4, 16, nspecies=3, seed=19)
    E, G = ctx.energy_forces(b.offsets, b.rr, b.species)
    dev = torch.device("cuda", 0)
    Ed = torch.empty(b.nenv, dtype=torch.float64, device=dev)
    Gd = torch.empty((b.nnbr, 3), dtype=torch.float64, device=dev)
    ctx.energy_forces_device(torch.from_numpy(b.offsets).to(dev), torch.from_numpy(b.rr).to(dev),
                             torch.from_numpy(b.species).to(dev), Ed, Gd)
    assert np.array_equal(E, Ed.cpu().numpy())
    # FP32 adjoint accumulated with shared-memory atomics: order-dependent rounding
    assert relerr(G, Gd.cpu().numpy()) <= 1e-6
    bad = b.species.copy()
    bad[b.offsets[11000]] = 5
    with pytest.raises(lib.AceError):
        ctx.energy_forces(b.offsets, b.rr, bad)


def test_contexts_of_different_sizes_interleave(lib, oracle_mod):
    """Contexts of one precision with different spec sizes (so different
    shared-memory needs) can be created and used in any order."""
    big = get_spec("cfg2")
    small = get_spec("test")
    cb = lib.Context(big, "fp32x2"); cb.set_params(random_coefficients(big, seed=1))
    cs = lib.Context(small, "fp32x2"); cs.set_params(random_coefficients(small, seed=1))
    b = random_batch(20, 10, 30, seed=4)
    Eb1, _ = cb.energy_forces(b.offsets, b.rr)
    Bb1 = cb.basis(b.offsets, b.rr)
    cs.energy_forces(b.offsets, b.rr)
    cs.basis(b.offsets, b.rr)
    Eb2, _ = cb.energy_forces(b.offsets, b.rr)        # after the smaller context's set-up
    Bb2 = cb.basis(b.offsets, b.rr)
    assert np.array_equal(Eb1, Eb2) and np.array_equal(Bb1, Bb2)


@pytest.mark.parametrize("kernel", ["items", "trie"])
@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp32x2", "fp32c"])
def test_other_schedules(lib, oracle_mod, prec, kernel, monkeypatch):
    """The task schedule is the default correlation walk for orders >= 3;
    the per-thread item runs and the trie walk (ACE_B200_KERNEL, read at
    context creation) stay selectable and give the same results (the
    compensated form has no trie walk and keeps its item runs)."""
    monkeypatch.setenv("ACE_B200_KERNEL", kernel)
    spec = get_spec("cfg2")
    c = random_coefficients(spec, seed=11)
    b = random_batch(100, 20, 60, seed=5)
    Eref, Gref = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr)
    ctx = lib.Context(spec, prec)
    ctx.set_params(c)
    E, G = ctx.energy_forces(b.offsets, b.rr)
    assert energy_relerr(E, Eref) <= TOL[prec]["E"]
    assert relerr(G, Gref) <= TOL[prec]["G"]
