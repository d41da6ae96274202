"""Host-side checks of the learned radial form: the numpy MLP oracle against
finite differences, the parameter layout shared with the CUDA kernels, and
the training-envelope split of LearnedRadialModel."""
import numpy as np
import pytest

from ace_gb300.configs import Batch, random_batch
from ace_gb300.learned import LearnedRadialModel, RadialMLP, student_spec


@pytest.fixture(scope="module")
def setup():
    import mlp_oracle
    spec = student_spec(3, 6, 4, 4)
    mlp = RadialMLP.init(spec, K=4, nspecies=3, Q=6, seed=1)
    mlp.params = (mlp.params + 0.05 * np.random.default_rng(2).standard_normal(len(mlp.params))).astype(np.float32)
    return mlp_oracle, spec, mlp


def test_layout_matches(setup):
    mo, spec, mlp = setup
    _, n = mo.layout(mlp.D, mlp.C)
    assert n == len(mlp.params) == RadialMLP.nparams_for(mlp.K, mlp.Q, mlp.nspecies, mlp.L)
    assert mlp.C == mlp.K * (spec.Leff + 1)


def test_oracle_radial_derivative(setup):
    mo, spec, mlp = setup
    cfg = mlp.feature_config(spec)
    r = np.linspace(0.6, 4.9, 37)
    s = np.arange(37) % 3
    _, dR = mo.forward(mlp.params, r, s, cfg, mlp.C)
    h = 1e-6
    Rp, _ = mo.forward(mlp.params, r + h, s, cfg, mlp.C)
    Rm, _ = mo.forward(mlp.params, r - h, s, cfg, mlp.C)
    fd = (Rp - Rm) / (2 * h)
    assert np.max(np.abs(fd - dR)) <= 1e-6 * max(1.0, np.max(np.abs(dR)))


def test_oracle_radial_vanishes_beyond_cutoff(setup):
    mo, spec, mlp = setup
    R, dR = mo.forward(mlp.params, np.array([5.0, 5.5, 9.0]), np.zeros(3, int), mlp.feature_config(spec), mlp.C)
    assert np.max(np.abs(R)) < 1e-12 and np.max(np.abs(dR[1:])) == 0.0


def test_oracle_backward_finite_difference(setup):
    mo, spec, mlp = setup
    cfg = mlp.feature_config(spec)
    rng = np.random.default_rng(3)
    r = 0.8 + 4.0 * rng.random(25)
    s = rng.integers(0, 3, 25)
    gR = rng.standard_normal((25, mlp.C))
    wj = rng.random(25)
    p = mlp.params.astype(np.float64)
    g = mo.backward(p, r, s, gR, wj, cfg, mlp.C)

    def L(q):
        R, _ = mo.forward(q, r, s, cfg, mlp.C)
        return float(np.sum(wj[:, None] * gR * R))
    idx = rng.choice(len(p), 40, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (L(p + e) - L(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_envelope_split():
    class Stub:
        rlo, rhi = 0.8, 5.0

        class mlp:
            nspecies = 2
    b = random_batch(6, 3, 5, nspecies=2, seed=4)
    rr = b.rr.copy()
    sp = b.species.copy()
    rr[b.offsets[1]] *= 0.5 / np.linalg.norm(rr[b.offsets[1]])     # env 1: a neighbour at r = 0.5
    sp[b.offsets[3]] = 7                                            # env 3: a species outside the MLP's
    nb = Batch(np.concatenate([b.offsets[:5], [b.offsets[4]], b.offsets[5:]]), rr, sp)  # env 5 empty
    ok = LearnedRadialModel.inside(Stub, nb)
    assert ok.tolist() == [True, False, True, False, True, True, True]


def test_oracle_external_radials(setup, oracle_mod):
    """The oracle's learned-form path: with every channel (k, l) set to the
    spec's own polynomial R_k it reproduces the plain evaluation, and its
    radial adjoint matches finite differences of the energy."""
    from ace_gb300.spec import random_coefficients
    _, spec, _ = setup
    c = random_coefficients(spec, seed=3)
    b = random_batch(5, 4, 9, seed=6)
    plain = oracle_mod.Oracle(spec, c)
    E0, G0 = plain.energy_forces(b.offsets, b.rr)
    r = np.linalg.norm(b.rr, axis=1)
    Rk, dRk = plain.radial(r)
    L1 = spec.Leff + 1
    lo = oracle_mod.Oracle(spec, c, channels_per_l=len(Rk[0]))
    lo.set_radial(np.tile(Rk, (1, L1)), np.tile(dRk, (1, L1)))
    E1, G1 = lo.energy_forces(b.offsets, b.rr)
    assert np.allclose(E1, E0, rtol=1e-13, atol=1e-13)
    assert np.allclose(G1, G0, rtol=1e-11, atol=1e-12)
    rng = np.random.default_rng(1)
    R = np.tile(Rk, (1, L1)) + 0.1 * rng.standard_normal((len(r), Rk.shape[1] * L1))
    lo.set_radial(R)
    E, GR = lo.radial_adjoint(b.offsets, b.rr)
    env = np.searchsorted(b.offsets, np.arange(len(r)), side="right") - 1
    h = 1e-6
    for j, cch in [(0, 0), (3, 5), (len(r) - 1, R.shape[1] - 1), (7, 2)]:
        Rp = R.copy(); Rp[j, cch] += h
        Rm = R.copy(); Rm[j, cch] -= h
        lo.set_radial(Rp); Ep = lo.evaluate(b.offsets, b.rr)
        lo.set_radial(Rm); Em = lo.evaluate(b.offsets, b.rr)
        fd = (Ep[env[j]] - Em[env[j]]) / (2 * h)
        assert abs(fd - GR[j, cch]) <= 1e-6 * max(1.0, abs(fd))
