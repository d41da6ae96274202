"""Failure detection on the GPU, exercised without a GPU fault.

The reference only asserts on bad input (an empty configuration,
src/product_1pbasis.jl:124).  Here host inputs are validated before any
launch, and device inputs are checked inside the kernels, which set bits of
the context's status word and skip the bad environment; the host reads the
word back and returns ACE_ERR_KERNEL with a message.  These tests feed device
inputs that the kernels must reject -- a NaN position, a neighbour at the
centre (r = 0), non-monotone offsets, a species out of range -- and check
the status, that the good environments of the same launch are still right,
and that the context evaluates correctly afterwards.

The tensor-core radial MLP waits for each MMA on an mbarrier with a bounded
number of polls; ACE_B200_TC_WAIT_LIMIT=0 makes every wait give up at once.
The kernel must then record ACE_STATUS_TIMEOUT, wait (bounded) for its MMAs
still in flight, free its tensor memory and return; a second context then
runs the same kernel normally, which needs the tensor memory freed."""
import ctypes as C

import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

pytestmark = pytest.mark.gpu

ACE_ERR_KERNEL = 4
IN_OUT_DEVICE = 1 | 2
ASYNC = 4


@pytest.fixture(scope="module")
def L():
    from ace_gb300 import lib
    from ace_gb300.build import build
    build()
    return lib


def _run(ctx, L, torch, b, flags=IN_OUT_DEVICE):
    off = torch.from_numpy(b.offsets).cuda()
    rr = torch.from_numpy(b.rr).cuda()
    sp = None if b.species is None else torch.from_numpy(b.species).cuda()
    E = torch.zeros(b.nenv, dtype=torch.float64, device="cuda")
    G = torch.zeros_like(rr)
    rc = ctx.lib.ace_energy_forces(ctx.h, b.nenv, L._ptr(off), L._ptr(rr), None if sp is None else L._ptr(sp),
                                   L._ptr(E), L._ptr(G), flags, None)
    return rc, E.cpu().numpy(), G.cpu().numpy()


def _message(ctx):
    return ctx.lib.ace_last_error_string(ctx.h).decode()


@pytest.mark.parametrize("prec", ["fp64", "fp32x2", "fp32c"])
@pytest.mark.parametrize("defect", ["nan", "centre"])
def test_bad_position_on_device(L, oracle_mod, prec, defect):
    torch = pytest.importorskip("torch")
    spec = symmetric_basis(3, 6, maxL=6)
    c = random_coefficients(spec, seed=1)
    b = random_batch(40, 10, 20, seed=2)
    Eref, Gref = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr)
    ctx = L.Context(spec, prec)
    ctx.set_params(c)
    bad = random_batch(40, 10, 20, seed=2)
    j = int(bad.offsets[7]) + 3                      # a neighbour of environment 7
    bad.rr[j] = np.nan if defect == "nan" else 0.0
    rc, E, _ = _run(ctx, L, torch, bad)
    assert rc == ACE_ERR_KERNEL
    assert "bad position" in _message(ctx)
    keep = np.arange(bad.nenv) != 7                  # the other environments are unaffected
    assert np.max(np.abs(E[keep] - Eref[keep])) <= 1e-6 * np.max(np.abs(Eref))
    # the status word was cleared and the context still evaluates correctly
    rc, E, G = _run(ctx, L, torch, b)
    assert rc == 0, _message(ctx)
    assert np.max(np.abs(E - Eref)) <= 1e-6 * np.max(np.abs(Eref))
    assert np.max(np.abs(G - Gref)) <= 1e-5 * np.max(np.abs(Gref))
    ctx.close()


def test_bad_offsets_on_device(L, oracle_mod):
    torch = pytest.importorskip("torch")
    spec = symmetric_basis(3, 6, maxL=6)
    c = random_coefficients(spec, seed=1)
    b = random_batch(6, 10, 20, seed=4)
    Eref, _ = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr)
    ctx = L.Context(spec, "fp64")
    ctx.set_params(c)
    bad = random_batch(6, 10, 20, seed=4)
    # environment 2 ends before it starts; every offset stays inside the
    # neighbour array, so no read leaves the caller's buffers
    bad.offsets = b.offsets.copy()
    bad.offsets[3] = bad.offsets[2] - 5
    rc, E, _ = _run(ctx, L, torch, bad)
    assert rc == ACE_ERR_KERNEL
    assert "bad offsets" in _message(ctx)
    assert np.isnan(E[2])
    for e in (0, 1, 4, 5):                           # environments with valid ranges
        assert abs(E[e] - Eref[e]) <= 1e-12 * np.max(np.abs(Eref))
    rc, E, _ = _run(ctx, L, torch, b)
    assert rc == 0, _message(ctx)
    assert np.max(np.abs(E - Eref)) <= 1e-12 * np.max(np.abs(Eref))
    ctx.close()


def test_bad_species_on_device_async(L, oracle_mod):
    """The asynchronous device call returns at once; ace_sync reports."""
    torch = pytest.importorskip("torch")
    spec = symmetric_basis(3, 6, maxL=6, nspecies=3)
    c = random_coefficients(spec, seed=1)
    b = random_batch(20, 8, 20, nspecies=3, seed=5)
    Eref, _ = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr, b.species)
    ctx = L.Context(spec, "fp32x2")
    ctx.set_params(c)
    bad = random_batch(20, 8, 20, nspecies=3, seed=5)
    bad.species[int(bad.offsets[4])] = 7
    rc, _, _ = _run(ctx, L, torch, bad, flags=IN_OUT_DEVICE | ASYNC)
    assert rc == 0
    assert ctx.lib.ace_sync(ctx.h) == ACE_ERR_KERNEL
    assert "species out of range" in _message(ctx)
    rc, E, _ = _run(ctx, L, torch, b)
    assert rc == 0, _message(ctx)
    assert np.max(np.abs(E - Eref)) <= 1e-6 * np.max(np.abs(Eref))
    ctx.close()


def test_tensor_core_wait_gives_up(L, monkeypatch):
    torch = pytest.importorskip("torch")
    import mlp_oracle
    from ace_gb300.learned import RadialMLP, learned_context, student_spec
    spec = student_spec(3, 6, 4, 4)
    mlp = RadialMLP.init(spec, K=4, nspecies=3, Q=6, seed=1)
    b = random_batch(200, 10, 30, nspecies=3, seed=6)
    rr = torch.from_numpy(b.rr).cuda()
    sp = torch.from_numpy(b.species).cuda()
    R = torch.zeros((b.nnbr, 2 * mlp.C), dtype=torch.float32, device="cuda")
    monkeypatch.setenv("ACE_B200_TC_WAIT_LIMIT", "0")
    ctx = learned_context(spec, mlp)                 # the limit is read here
    monkeypatch.delenv("ACE_B200_TC_WAIT_LIMIT")
    rc = ctx.lib.ace_radial_mlp_infer(ctx.h, b.nnbr, L._ptr(rr), L._ptr(sp), L._ptr(R), None)
    assert rc == 0                                   # asynchronous: the status comes with ace_sync
    assert ctx.lib.ace_sync(ctx.h) == ACE_ERR_KERNEL
    assert "tensor-core wait timed out" in _message(ctx)
    ctx.close()
    # tensor memory was freed: the same kernel runs to completion in a new context
    ctx2 = learned_context(spec, mlp)
    ctx2.radial_mlp_infer(rr, sp, R)
    ctx2.sync()
    Rref, _ = mlp_oracle.forward(mlp.params.astype(np.float64), np.linalg.norm(b.rr, axis=1), b.species,
                                 mlp.feature_config(spec), mlp.C)
    Rg = R.cpu().numpy()[:, :mlp.C]
    assert np.max(np.abs(Rg - Rref)) <= 2e-2 * np.max(np.abs(Rref))
    ctx2.close()
