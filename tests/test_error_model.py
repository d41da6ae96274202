"""The compensated form's error estimate, checked on a numpy model of its
arithmetic (CPU).

The compensated kernel (ACE_PREC_FP32_COMP, task schedule) evaluates the
correlation products in FP32 on A rounded to FP32 (A's own rounding is
corrected to first order through the adjoint): per task the prefix product
Q_t = A_t0 A_t1 ..., per item Q = Q_t A_mid, H = c_own + sum_g c_g A_leaf_g,
the two real products p1 = Q.re H.re and p2 = Q.im H.im, the term p1 - p2,
the task's terms summed in FP32 and added to a double-float total.  Its
estimate of an environment's energy rounding error is
k sqrt(sum_tasks S^2 + sum_shorts t^2) 2^-24, S = sum over the task's items
of |p1| + |p2|, k = 5 (ace_set_energy_tolerance).

This test restates that arithmetic in numpy with the same rounding sites
(FP32 products and sums, without fused multiply-adds), on seeded
environments of an order-4 and an order-5 basis, and checks that the
rounding error of every environment -- against the same products in FP64 on
the same FP32 inputs -- is within the estimate, and that the estimate is not
vacuous (the errors reach a fair fraction of it)."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

K_TASKS = 5.0
U32 = 2.0 ** -24


def _structure(spec):
    """Tasks, items and short functions of the spec, as the task schedule
    groups them: a task is a (K-2)-prefix of the descending index rows of the
    functions of order >= K-1; its items are (mid, up to two leaves) with the
    coefficient of the prefix function (task, mid) on the first item."""
    K = spec.maxorder
    KT = K - 2
    iaa, ords = spec.iAA2iA, spec.orders
    rows = []
    for k in np.flatnonzero(ords >= K - 1):
        rows.append((tuple(iaa[k, :KT]), int(iaa[k, KT]), int(iaa[k, K - 1]) if ords[k] == K else -1, int(k)))
    rows.sort()
    tasks = []  # (prefix, [(mid, own_k, [(leaf, k), ...]), ...])
    for pre, mid, leaf, k in rows:
        if not tasks or tasks[-1][0] != pre:
            tasks.append((pre, []))
        items = tasks[-1][1]
        if not items or items[-1][0] != mid or (leaf >= 0 and len(items[-1][2]) == 2):
            items.append((mid, -1, []))
        m, own, leaves = items[-1]
        if leaf < 0:
            items[-1] = (m, k, leaves)
        else:
            leaves.append((leaf, k))
    shorts = np.flatnonzero(ords < K - 1)
    return tasks, shorts


def _cmul32(a, b):
    re = np.float32(a.real) * np.float32(b.real) - np.float32(a.imag) * np.float32(b.imag)
    im = np.float32(a.real) * np.float32(b.imag) + np.float32(a.imag) * np.float32(b.real)
    return np.complex64(complex(re, im))


def _model(Ahi, c32, spec, tasks, shorts):
    """(energy of the FP32 arithmetic, the same products in FP64, s_e)."""
    iaa, ords = spec.iAA2iA, spec.orders
    A64 = Ahi.astype(np.complex128)
    e_model = 0.0
    e_exact = 0.0
    s2 = 0.0
    for pre, items in tasks:
        qt = Ahi[pre[0]]
        qt64 = A64[pre[0]]
        for v in pre[1:]:
            qt = _cmul32(qt, Ahi[v])
            qt64 = qt64 * A64[v]
        eterm = np.float32(0.0)
        size = 0.0
        for mid, own, leaves in items:
            h = np.complex64(complex(c32[own] if own >= 0 else 0.0, 0.0))
            h64 = complex(float(c32[own]) if own >= 0 else 0.0, 0.0)
            for leaf, k in leaves:
                h = np.complex64(complex(np.float32(h.real) + np.float32(c32[k]) * np.float32(Ahi[leaf].real),
                                         np.float32(h.imag) + np.float32(c32[k]) * np.float32(Ahi[leaf].imag)))
                h64 += float(c32[k]) * A64[leaf]
            q = _cmul32(qt, Ahi[mid])
            p1 = np.float32(q.real) * np.float32(h.real)
            p2 = np.float32(q.imag) * np.float32(h.imag)
            eterm = np.float32(eterm + np.float32(p1 - p2))
            size += abs(float(p1)) + abs(float(p2))
            e_exact += (qt64 * A64[mid] * h64).real
        e_model += float(eterm)
        s2 += size * size
    for k in shorts:
        o = int(ords[k])
        if o == 0:
            e_model += float(c32[k])
            e_exact += float(c32[k])
            continue
        p = Ahi[iaa[k, 0]]
        p64 = A64[iaa[k, 0]]
        for t in range(1, o):
            p = _cmul32(p, Ahi[iaa[k, t]])
            p64 = p64 * A64[iaa[k, t]]
        t32 = np.float32(c32[k]) * np.float32(p.real)
        e_model += float(t32)
        e_exact += float(c32[k]) * p64.real
        s2 += float(t32) ** 2
    return e_model, e_exact, np.sqrt(s2) * U32


@pytest.mark.parametrize("order,deg,nenv", [(4, 8, 60), (5, 8, 30)])
def test_estimate_bounds_model_error(oracle_mod, order, deg, nenv):
    spec = symmetric_basis(order, deg, maxL=deg)
    c = random_coefficients(spec, seed=7)
    ct = spec.ctilde(c)
    c32 = ct.astype(np.float32)
    b = random_batch(nenv, 20, 40, seed=8)
    A = oracle_mod.Oracle(spec, c).A(b.offsets, b.rr)
    tasks, shorts = _structure(spec)
    ratios = []
    for e in range(nenv):
        Ahi = A[e].astype(np.complex64)
        em, ex, s = _model(Ahi, c32, spec, tasks, shorts)
        assert abs(em - ex) <= K_TASKS * s, (e, abs(em - ex) / s)
        ratios.append(abs(em - ex) / s)
    # the estimate is not vacuous: the largest errors reach a fair fraction of it
    assert max(ratios) >= 0.3
