"""Generates the committed golden fixtures under tests/golden/.

* cg_sympy.json -- Clebsch-Gordan coefficients from sympy's
  ``sympy.physics.quantum.spin.CG`` for the random index sets the reference's
  ``test/test_cg.jl:21-38`` draws (j1, j2 in 0:10, J up to 10), seeded.
* ylm_closed_form.json -- complex Y_l^m, l <= 3, from the closed-form
  expressions the reference's ``test/polynomials/test_ylm.jl:14-32`` checks
  against (textbook formulas written out here), at seeded random directions,
  including directions within 1e-9 of the pole.

Run:  python tests/golden/make_golden.py   (needs sympy; the GPU host does not)
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def cg_fixture(ntest=300, seed=0):
    from sympy.physics.quantum.spin import CG
    rng = np.random.default_rng(seed)
    rows = []
    while len(rows) < ntest:
        j1 = int(rng.integers(0, 11)); j2 = int(rng.integers(0, 11))
        J = int(rng.integers(abs(j1 - j2), min(10, j1 + j2) + 1))
        m1 = int(rng.integers(-j1, j1 + 1))
        for m2 in range(-j2, j2 + 1):
            M = m1 + m2
            if abs(M) <= J:
                val = float(CG(j1, m1, j2, m2, J, M).doit().evalf(30))
                rows.append([j1, m1, j2, m2, J, M, val])
    return rows


def ylm_closed(theta, phi):
    s, c = np.sin(theta), np.cos(theta)
    e = lambda m: np.exp(1j * m * phi)
    pi = np.pi
    return [
        0.5 * np.sqrt(1 / pi),
        0.5 * np.sqrt(3 / (2 * pi)) * s * e(-1),
        0.5 * np.sqrt(3 / pi) * c,
        -0.5 * np.sqrt(3 / (2 * pi)) * s * e(1),
        0.25 * np.sqrt(15 / (2 * pi)) * s ** 2 * e(-2),
        0.5 * np.sqrt(15 / (2 * pi)) * s * c * e(-1),
        0.25 * np.sqrt(5 / pi) * (3 * c ** 2 - 1),
        -0.5 * np.sqrt(15 / (2 * pi)) * s * c * e(1),
        0.25 * np.sqrt(15 / (2 * pi)) * s ** 2 * e(2),
        1 / 8 * e(-3) * np.sqrt(35 / pi) * s ** 3,
        1 / 4 * e(-2) * np.sqrt(105 / (2 * pi)) * c * s ** 2,
        1 / 8 * e(-1) * np.sqrt(21 / pi) * (-1 + 5 * c ** 2) * s,
        1 / 4 * np.sqrt(7 / pi) * (-3 * c + 5 * c ** 3),
        -(1 / 8) * e(1) * np.sqrt(21 / pi) * (-1 + 5 * c ** 2) * s,
        1 / 4 * e(2) * np.sqrt(105 / (2 * pi)) * c * s ** 2,
        -(1 / 8) * e(3) * np.sqrt(35 / pi) * s ** 3,
    ]


def ylm_fixture(n=30, seed=1):
    rng = np.random.default_rng(seed)
    rows = []
    for k in range(2 * n):
        if k < n:
            theta = rng.random() * np.pi
        else:
            theta = rng.random() * 1e-9
            if theta < 1e-10:
                theta = 0.0
        phi = (rng.random() - 0.5) * 2 * np.pi
        r = 0.1 + rng.random()
        x = [r * np.sin(theta) * np.cos(phi), r * np.sin(theta) * np.sin(phi), r * np.cos(theta)]
        Y = ylm_closed(theta, phi)
        rows.append(dict(x=x, re=[float(np.real(y)) for y in Y], im=[float(np.imag(y)) for y in Y]))
    return rows


if __name__ == "__main__":
    with open(os.path.join(HERE, "cg_sympy.json"), "w") as f:
        json.dump(cg_fixture(), f)
    with open(os.path.join(HERE, "ylm_closed_form.json"), "w") as f:
        json.dump(ylm_fixture(), f)
    print("wrote fixtures to", HERE)
