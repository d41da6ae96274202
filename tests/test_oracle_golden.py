"""The oracle pinned against known answers: closed-form Y_l^m
(reference test/polynomials/test_ylm.jl:14-66), sympy Clebsch-Gordan values
(test/test_cg.jl:21-38) and the SH product expansion (test/test_cg.jl:56-76)."""
import json
import os

import numpy as np

from ace_gb300.coupling import clebschgordan

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_ylm_closed_form(oracle_mod):
    rows = json.load(open(os.path.join(GOLD, "ylm_closed_form.json")))
    for row in rows:
        Yex = np.array(row["re"]) + 1j * np.array(row["im"])
        Y = oracle_mod.sh(3, row["x"])
        assert np.allclose(Y, Yex, rtol=1e-12, atol=1e-12)
        # the gradient path (cYlm_ed!) must give the same values
        Y2, _ = oracle_mod.sh(3, row["x"], grad=True)
        assert np.allclose(Y2, Yex, rtol=1e-12, atol=1e-12)


def test_cg_vs_sympy():
    rows = json.load(open(os.path.join(GOLD, "cg_sympy.json")))
    assert len(rows) >= 200
    for j1, m1, j2, m2, J, M, val in rows:
        assert abs(clebschgordan(j1, m1, j2, m2, J, M) - val) <= 1e-14 * max(1.0, abs(val))


def test_sh_product_expansion(oracle_mod):
    rng = np.random.default_rng(7)
    for _ in range(100):
        l1, l2 = rng.integers(1, 7, size=2)
        m1, m2 = rng.integers(-l1, l1 + 1), rng.integers(-l2, l2 + 1)
        th, ph = rng.random() * np.pi, (rng.random() - 0.5) * 2 * np.pi
        R = [np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)]
        Y = oracle_mod.sh(int(l1 + l2), R)
        iy = lambda l, m: m + l + l * l
        p = Y[iy(l1, m1)] * Y[iy(l2, m2)]
        M = m1 + m2
        p2 = 0.0
        for L in range(abs(M), l1 + l2 + 1):
            p2 += np.sqrt((2 * l1 + 1) * (2 * l2 + 1) / (4 * np.pi * (2 * L + 1))) * \
                clebschgordan(int(l1), 0, int(l2), 0, L, 0) * \
                clebschgordan(int(l1), int(m1), int(l2), int(m2), L, int(M)) * Y[iy(L, M)]
        assert abs(p - p2) < 1e-13


def test_sh_gradient_fd(oracle_mod):
    rng = np.random.default_rng(3)
    for _ in range(10):
        x = rng.standard_normal(3)
        _, dY = oracle_mod.sh(6, x, grad=True)
        h = 1e-6
        for a in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a] += h; xm[a] -= h
            fd = (oracle_mod.sh(6, xp) - oracle_mod.sh(6, xm)) / (2 * h)
            assert np.allclose(dY[:, a], fd, atol=1e-7)
