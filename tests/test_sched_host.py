"""Host logic of the correlation schedules (ace.jl_gb300/csrc/ace_sched.h):
the trie walk, the item schedule and the task schedule, replayed
in double precision by tests/host/sched_check.cpp, must reproduce the flat
products of the reference evaluator (energy, and the adjoint along
conjugation-symmetric directions, which is what the forces contract with)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("sched")
    exe = str(d / "sched_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "ace.jl_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "host", "sched_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("args", [(2, 6, 6, 1), (3, 6, 6, 1), (3, 8, 6, 1), (4, 10, 10, 1), (5, 8, 8, 1),
                                  (3, 6, 6, 3), (4, 8, 8, 2), (6, 7, 7, 1)])
def test_schedules_match_flat_products(checker, oracle_mod, tmp_path, args):
    o, deg, L, ns = args
    spec = symmetric_basis(o, deg, maxL=L, nspecies=ns)
    c = random_coefficients(spec, seed=3)
    b = random_batch(1, 30, 30, nspecies=ns, seed=1)
    A = oracle_mod.Oracle(spec, c).A(b.offsets, b.rr, b.species)[0]
    a = spec.aspec
    # a conjugation-symmetric direction: W_{n,l,-m} = (-1)^m conj(W_{n,l,m})
    rng = np.random.default_rng(0)
    W = np.zeros(spec.nA, complex)
    idx = {(int(mu), int(n), int(l), int(m)): i for i, (mu, n, l, m) in enumerate(zip(a.mu, a.n, a.l, a.m))}
    for i, (mu, n, l, m) in enumerate(zip(a.mu, a.n, a.l, a.m)):
        if m > 0:
            W[i] = rng.standard_normal() + 1j * rng.standard_normal()
            W[idx[(int(mu), int(n), int(l), -int(m))]] = (-1) ** int(m) * np.conj(W[i])
        elif m == 0:
            W[i] = rng.standard_normal()
    U = spec.U.tocsr()
    U.sort_indices()
    for name, arr, dt in [("an", a.n - 1, np.int32), ("al", a.l, np.int32), ("am", a.m, np.int32),
                          ("amu", a.mu, np.int32), ("ord", spec.orders, np.int32), ("iaa", spec.iAA2iA, np.int32),
                          ("Up", U.indptr, np.int64), ("Ui", U.indices, np.int32), ("Ud", U.data, np.float64),
                          ("ct", spec.ctilde(c), np.float64), ("A", np.stack([A.real, A.imag], 1), np.float64),
                          ("W", np.stack([W.real, W.imag], 1), np.float64)]:
        np.ascontiguousarray(arr, dtype=dt).tofile(str(tmp_path / f"{name}.bin"))
    out = subprocess.run([checker, str(tmp_path)], capture_output=True, text=True, check=True).stdout.split()
    halved, n, nitems = int(out[0]), int(out[1]), int(out[2])
    eT, eI, gT, gI, eK, gK = map(float, out[3:9])
    assert halved == 1
    assert eT < 1e-12 and eI < 1e-12 and eK < 1e-12
    assert gT < 1e-11 and gI < 1e-11 and gK < 1e-11
