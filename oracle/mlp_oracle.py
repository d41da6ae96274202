"""FP64 numpy restatement of the learned radial MLP of libace_b200
(``ace.jl_gb300/csrc/ace_mlp.cu``): forward values, r-derivatives and the
parameter gradient.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` to check the CUDA kernels,
never by the product.  The learned radial form has no counterpart in ACE.jl;
its definition is the one written in ``include/ace_b200.h``:

  t = ((1 + r0)/(1 + r))^p, fe(t) = (t - tl)^pl (t - tr)^pr (0 outside)
  x = 2 (t - tl)/(tmax - tl) - 1,  f = [T_0(x) .. T_{Q-1}(x), onehot(s)]
  h1 = silu(W1 f + b1), h2 = silu(W2 h1 + b2), R = fe(t) (W3 h2 + b3)
"""
from __future__ import annotations

import numpy as np

H = 64


def layout(D: int, C: int):
    o, n = {}, 0
    for name, size in (("W1", H * D), ("b1", H), ("W2", H * H), ("b2", H), ("W3", C * H), ("b3", C)):
        o[name] = (n, size)
        n += size
    return o, n


def unpack(params, D, C):
    o, _ = layout(D, C)
    p = np.asarray(params, dtype=np.float64)
    W1 = p[o["W1"][0]:o["W1"][0] + H * D].reshape(H, D)
    b1 = p[o["b1"][0]:o["b1"][0] + H]
    W2 = p[o["W2"][0]:o["W2"][0] + H * H].reshape(H, H)
    b2 = p[o["b2"][0]:o["b2"][0] + H]
    W3 = p[o["W3"][0]:o["W3"][0] + C * H].reshape(C, H)
    b3 = p[o["b3"][0]:o["b3"][0] + C]
    return W1, b1, W2, b2, W3, b3


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def features(r, species, *, p, r0, tl, tr, pl, pr, tmax, Q, S):
    r = np.asarray(r, dtype=np.float64)
    u = 1.0 + r
    x = (1.0 + r0) / u
    t = x ** p
    dtdr = p * x ** (p - 1) * (-(1.0 + r0) / (u * u))
    outside = np.zeros_like(t, dtype=bool)
    if pl > 0:
        outside |= t < tl
    if pr > 0:
        outside |= t > tr
    fe = np.where(outside, 0.0, (t - tl) ** pl * (t - tr) ** pr)
    dfe = np.zeros_like(t)
    if pl > 0:
        dfe += pl * (t - tl) ** (pl - 1) * (t - tr) ** pr
    if pr > 0:
        dfe += (t - tl) ** pl * pr * (t - tr) ** (pr - 1)
    dfe = np.where(outside, 0.0, dfe)
    xs = 2.0 / (tmax - tl)
    z = xs * (t - tl) - 1.0
    T = np.zeros((len(r), Q))
    dT = np.zeros((len(r), Q))
    T[:, 0] = 1.0
    if Q > 1:
        T[:, 1] = z
        dT[:, 1] = 1.0
    for q in range(2, Q):
        T[:, q] = 2 * z * T[:, q - 1] - T[:, q - 2]
        dT[:, q] = 2 * T[:, q - 1] + 2 * z * dT[:, q - 1] - dT[:, q - 2]
    s = np.zeros(len(r), dtype=np.int64) if species is None else np.asarray(species, dtype=np.int64)
    oh = np.zeros((len(r), S))
    oh[np.arange(len(r)), s] = 1.0
    f = np.concatenate([T, oh], axis=1)
    df = np.concatenate([dT * xs, np.zeros((len(r), S))], axis=1)
    return f, df, fe, dfe, dtdr


def forward(params, r, species, cfg, C):
    """R (n, C) and dR/dr (n, C)."""
    f, df, fe, dfe, dtdr = features(r, species, **cfg)
    W1, b1, W2, b2, W3, b3 = unpack(params, f.shape[1], C)
    z1 = f @ W1.T + b1
    s1 = _sig(z1)
    h1 = z1 * s1
    dh1 = s1 * (1 + z1 * (1 - s1)) * (df @ W1.T)
    z2 = h1 @ W2.T + b2
    s2 = _sig(z2)
    h2 = z2 * s2
    dh2 = s2 * (1 + z2 * (1 - s2)) * (dh1 @ W2.T)
    o = h2 @ W3.T + b3
    do = dh2 @ W3.T
    R = fe[:, None] * o
    dR = (dfe[:, None] * o + fe[:, None] * do) * dtdr[:, None]
    return R, dR


def backward(params, r, species, gR, wj, cfg, C):
    """d/dparams of sum_j wj sum_c gR[j, c] R_c(r_j)."""
    f, _, fe, _, _ = features(r, species, **cfg)
    D = f.shape[1]
    W1, b1, W2, b2, W3, b3 = unpack(params, D, C)
    z1 = f @ W1.T + b1
    s1 = _sig(z1)
    h1 = z1 * s1
    z2 = h1 @ W2.T + b2
    s2 = _sig(z2)
    h2 = z2 * s2
    w = fe * (np.ones(len(r)) if wj is None else np.asarray(wj, dtype=np.float64))
    go = np.asarray(gR, dtype=np.float64) * w[:, None]
    gW3 = go.T @ h2
    gb3 = go.sum(0)
    gz2 = (go @ W3) * (s2 * (1 + z2 * (1 - s2)))
    gW2 = gz2.T @ h1
    gb2 = gz2.sum(0)
    gz1 = (gz2 @ W2) * (s1 * (1 + z1 * (1 - s1)))
    gW1 = gz1.T @ f
    gb1 = gz1.sum(0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
