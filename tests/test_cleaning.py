"""The AA cleaning rule against the reference's.

clean_pibasis! (src/symmbasis.jl:225-236) keeps every AA column of U whose
norm exceeds atol = 0, i.e. it drops exact zeros only.  The spec builder
here first sets U entries below 1e-12 of their row maximum to zero (round-off
of the coupling arithmetic) and then applies the same exact-zero rule.  These
checks build the spec both ways (zero_tol = 1e-12, the default, and
zero_tol = 0, the reference's rule applied to this U) and show that

* the default AA list is the exact-zero list with some functions removed,
  order preserved;
* every removed function's U column is round-off: at most 1e-12 of the
  largest |U| of each of its rows, so its coefficient c~ = U^T c is
  round-off too;
* the FP64 oracle gives the same energies and forces on both specs
  (relative 1e-13), so the removed functions change no result."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis


def _tuples(spec):
    A = spec.aspec
    key = np.stack([A.mu, A.n, A.l, A.m], axis=1)
    out = []
    for k in range(spec.nAA):
        t = spec.iAA2iA[k]
        out.append(tuple(tuple(key[i]) for i in t if i >= 0))
    return out


@pytest.mark.parametrize("args", [(4, 10, 10, 1), (3, 8, 6, 2)])
def test_cleaning_drops_only_roundoff(oracle_mod, args):
    order, deg, L, ns = args
    s1 = symmetric_basis(order, deg, maxL=L, nspecies=ns)
    s0 = symmetric_basis(order, deg, maxL=L, nspecies=ns, zero_tol=0.0)
    assert s1.nB == s0.nB
    t1, t0 = _tuples(s1), _tuples(s0)
    pos = {t: i for i, t in enumerate(t0)}
    idx = np.array([pos[t] for t in t1])                 # every kept function is in the exact-zero list
    assert np.all(np.diff(idx) > 0)                      # in the same order
    dropped = np.setdiff1d(np.arange(s0.nAA), idx)
    U0 = s0.U.tocsr()
    rowmax = np.asarray(abs(U0).max(axis=1).todense()).ravel()
    Ud = abs(U0[:, dropped]).tocoo()
    if Ud.nnz:
        assert np.all(Ud.data <= 1e-12 * rowmax[Ud.row])
    c = random_coefficients(s1, seed=4)
    b = random_batch(50, 10, 30, nspecies=ns, seed=5)
    E1, G1 = oracle_mod.Oracle(s1, c).energy_forces(b.offsets, b.rr, b.species)
    E0, G0 = oracle_mod.Oracle(s0, c).energy_forces(b.offsets, b.rr, b.species)
    assert np.max(np.abs(E1 - E0)) <= 1e-13 * np.max(np.abs(E0))
    assert np.max(np.abs(G1 - G0)) <= 1e-13 * np.max(np.abs(G0))
