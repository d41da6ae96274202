"""ace_basis_noalloc: the symmetric basis for callers that must not allocate
device memory while they run (an MD engine that owns the device memory pool
after start-up, a service with a fixed footprint).  The entry point is called
through the C ABI with device buffers and must reproduce ace_basis, twice in a
row (the static scratch is shared by all calls and keeps the previous call's
contents), without taking device memory on the second call.

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import symmetric_basis

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "fp32x2", "fp32"])
def test_basis_noalloc_matches_basis(prec):
    torch = pytest.importorskip("torch")
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    build()
    tol = {"fp64": 1e-12, "fp32x2": 1e-12, "fp32": 1e-6}[prec]
    spec = symmetric_basis(3, 8, maxL=6)
    ctx = L.Context(spec, prec)
    lib = ctx.lib
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (1, 2):  # two calls in a row, different inputs
        b = random_batch(3000, 12, 24, seed=seed)
        Bref = ctx.basis(b.offsets, b.rr)                      # existing entry point
        off = torch.from_numpy(b.offsets).cuda()
        rr = torch.from_numpy(b.rr).cuda()
        B = torch.full((b.nenv, spec.nB), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = lib.ace_basis_noalloc(ctx.h, b.nenv, L._ptr(off), L._ptr(rr), None, L._ptr(B), C.c_void_p(stream))
        assert rc == 0, lib.ace_last_error_string(ctx.h)
        assert lib.ace_sync(ctx.h) == 0
        torch.cuda.synchronize()
        if seed == 2:  # the first call on a device may load the library's device code
            assert torch.cuda.mem_get_info()[0] == free0
        Bn = B.cpu().numpy()
        err = np.max(np.abs(Bn - Bref)) / np.max(np.abs(Bref))
        assert err <= tol, err
    ctx.close()
