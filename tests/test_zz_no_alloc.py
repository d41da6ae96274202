"""ace_basis_noalloc: the symmetric basis for callers that must not allocate
device memory while they run -- an MD engine that reserves the device memory
pool at start-up and owns it afterwards, or a service that keeps a fixed
footprint.  Such a caller creates its context during set-up (which
allocates) and then evaluates through this entry point, which allocates
nothing, not even on its first call.

Each case calls the entry point through the C ABI with device buffers, twice
in a row with different inputs (the static scratch is shared by all calls and
keeps the previous call's contents), and checks B against the FP64 CPU oracle
and against ace_basis, and that free device memory is unchanged across every
call, the first one after context creation included.

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

pytestmark = pytest.mark.gpu

# relative to max |B| of the oracle
TOL = {"fp64": 1e-12, "fp32x2": 1e-11, "fp32": 1e-5}


@pytest.fixture(scope="module")
def L():
    from ace_gb300 import lib
    from ace_gb300.build import build
    build()
    return lib


def _noalloc_case(L, oracle_mod, spec, prec, nspecies, jlo, jhi, nenv):
    torch = pytest.importorskip("torch")
    orc = oracle_mod.Oracle(spec, random_coefficients(spec, seed=3))
    ctx = L.Context(spec, prec)
    lib = ctx.lib
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (1, 2):  # two calls in a row, different inputs
        b = random_batch(nenv, jlo, jhi, nspecies=nspecies, seed=seed)
        Bref = orc.basis(b.offsets, b.rr, b.species)
        Bapi = ctx.basis(b.offsets, b.rr, b.species)       # the allocating entry point
        off = torch.from_numpy(b.offsets).cuda()
        rr = torch.from_numpy(b.rr).cuda()
        sp = None if b.species is None else torch.from_numpy(b.species).cuda()
        B = torch.full((b.nenv, spec.nB), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = lib.ace_basis_noalloc(ctx.h, b.nenv, L._ptr(off), L._ptr(rr), None if sp is None else L._ptr(sp),
                                   L._ptr(B), C.c_void_p(stream))
        assert rc == 0, lib.ace_last_error_string(ctx.h)
        assert lib.ace_sync(ctx.h) == 0
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, "ace_basis_noalloc changed the free device memory"
        Bn = B.cpu().numpy()
        scale = np.max(np.abs(Bref))
        err = np.max(np.abs(Bn - Bref)) / scale
        assert err <= TOL[prec], (prec, seed, err)
        assert np.max(np.abs(Bn - Bapi)) / scale <= TOL[prec]
    ctx.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32x2", "fp32"])
def test_basis_noalloc_single_species(L, oracle_mod, prec):
    _noalloc_case(L, oracle_mod, symmetric_basis(3, 8, maxL=6), prec, 1, 12, 24, 2000)


@pytest.mark.parametrize("prec", ["fp64", "fp32x2"])
def test_basis_noalloc_species(L, oracle_mod, prec):
    """Three species: the device species array selects each neighbour's
    categorical factor."""
    _noalloc_case(L, oracle_mod, symmetric_basis(3, 6, maxL=6, nspecies=3), prec, 3, 8, 30, 500)


def test_basis_noalloc_rejects_learned_form(L):
    torch = pytest.importorskip("torch")
    from ace_gb300.learned import RadialMLP, learned_context, student_spec
    sspec = student_spec(3, 6, 4, 4)
    mlp = RadialMLP.init(sspec, K=4, nspecies=3, Q=6, seed=1)
    ctx = learned_context(sspec, mlp)
    b = random_batch(8, 8, 12, nspecies=3, seed=1)
    off = torch.from_numpy(b.offsets).cuda()
    rr = torch.from_numpy(b.rr).cuda()
    sp = torch.from_numpy(b.species).cuda()
    B = torch.empty((b.nenv, sspec.nB), dtype=torch.float64, device="cuda")
    rc = ctx.lib.ace_basis_noalloc(ctx.h, b.nenv, L._ptr(off), L._ptr(rr), L._ptr(sp), L._ptr(B), None)
    assert rc == 5  # ACE_ERR_UNSUPPORTED
    assert b"learned" in ctx.lib.ace_last_error_string(ctx.h)
    ctx.close()


def test_basis_noalloc_rejects_large_specs(L):
    """A spec whose per-environment AA vector exceeds the 16 MiB static
    scratch (4 species, order 4, degree 11: 3.7M AA functions, 29.6 MB in
    FP64) is rejected with ACE_ERR_UNSUPPORTED before any launch."""
    torch = pytest.importorskip("torch")
    spec = symmetric_basis(4, 11, maxL=11, nspecies=4)
    assert spec.nAA * 8 > 16 << 20
    ctx = L.Context(spec, "fp64")
    b = random_batch(4, 8, 12, nspecies=4, seed=1)
    off = torch.from_numpy(b.offsets).cuda()
    rr = torch.from_numpy(b.rr).cuda()
    sp = torch.from_numpy(b.species).cuda()
    B = torch.empty((b.nenv, spec.nB), dtype=torch.float64, device="cuda")
    rc = ctx.lib.ace_basis_noalloc(ctx.h, b.nenv, L._ptr(off), L._ptr(rr), L._ptr(sp), L._ptr(B), None)
    assert rc == 5  # ACE_ERR_UNSUPPORTED
    assert b"16 MiB" in ctx.lib.ace_last_error_string(ctx.h)
    ctx.close()
