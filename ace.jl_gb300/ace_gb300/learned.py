"""Learned radial compression of a multi-species ACE model.

A plain multi-species model (the teacher) has one-particle functions
R_n(r) [species = s] Y_l^m (src/b1pcomponents/Rn.jl:17-29 times
src/discrete1pbasis.jl:78-123): nR x nspecies radial channels per l.  The
learned form (the student) replaces them by K channels per l computed by a
small MLP of (transformed distance, neighbour species) -- its definition is in
``include/ace_b200.h`` -- over a single-species spec with nR = K, so the A and
AA widths shrink with K instead of nR x nspecies.  The student is fitted to
the teacher by distillation:

1. ``pretrain_radial``: the MLP is regressed on seeded neighbour samples onto
   the student spec's own polynomial radials R_k(r), the same for every l
   and species.  The pretrained student is the method without the network:
   a species-blind radial basis of width K.
2. ``fit_coefficients``: the student's basis coefficients c by ridge least
   squares on teacher energies of seeded environments and, optionally, on
   the teacher's per-neighbour gradients (c enters both linearly; the
   student basis B and its derivative dB are evaluated on the GPU).
3. ``distill``: Adam on the MLP parameters against the teacher energies and,
   optionally, the teacher's per-neighbour gradients, with c re-fitted every
   few hundred steps.  The energy loss gradient is exact: dL/dR_c(r_j) comes
   from the energy kernel's adjoint (``ace_energy_radial_adjoint``) and is
   pushed through the MLP by ``ace_radial_mlp_backward``.  The force loss
   L_F = sum_j |G_j - G*_j|^2 (G_j = dE/drr_j) has the gradient
   d/dtheta sum_j W_j . G_j with W_j = dL_F/dG_j held fixed, and
   sum_j W_j . G_j is the derivative of sum_e E_e(rr + eps W) at eps = 0: a
   Hessian-vector product, formed as the central difference in eps of two
   exact energy gradients (``force_loss_gradient``, truncation O(eps^2)).

``LearnedRadialModel`` evaluates the student and sends every environment
with a neighbour outside the training radii (or a species the MLP was not
trained on) to the teacher, the plain model, against which the student's
error is also measured.

Training runs on the GPU through the library's kernels; torch only holds the
device buffers and forms the elementwise loss residuals.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .configs import Batch
from .lib import Context
from .spec import ACESpec, symmetric_basis

H = 64


@dataclass
class RadialMLP:
    K: int
    Q: int
    nspecies: int
    L: int
    tmax: float
    params: np.ndarray = field(repr=False)

    @property
    def D(self):
        return self.Q + self.nspecies

    @property
    def C(self):
        return self.K * (self.L + 1)

    @staticmethod
    def nparams_for(K, Q, nspecies, L):
        D, C = Q + nspecies, K * (L + 1)
        return H * D + H + H * H + H + C * H + C

    @classmethod
    def init(cls, spec: ACESpec, K: int, nspecies: int, Q: int = 8, seed: int = 0) -> "RadialMLP":
        """Weights N(0, 1/fan_in), zero biases.  tmax = t(0): the feature
        x = 2 (t - tl)/(tmax - tl) - 1 spans [-1, 1] on [0, rcut]."""
        rng = np.random.default_rng(seed)
        L = spec.Leff
        D, C = Q + nspecies, K * (L + 1)
        W1 = rng.standard_normal((H, D)) / np.sqrt(D)
        W2 = rng.standard_normal((H, H)) / np.sqrt(H)
        W3 = rng.standard_normal((C, H)) / np.sqrt(H)
        p = np.concatenate([W1.ravel(), np.zeros(H), W2.ravel(), np.zeros(H), W3.ravel(), np.zeros(C)])
        tmax = float(spec.radial.trans(0.0))
        return cls(K, Q, nspecies, L, tmax, p.astype(np.float32))

    def feature_config(self, spec: ACESpec) -> dict:
        R = spec.radial
        return dict(p=R.trans.p, r0=R.trans.r0, tl=R.J.tl, tr=R.J.tr, pl=R.J.pl, pr=R.J.pr, tmax=self.tmax,
                    Q=self.Q, S=self.nspecies)

    def to_dict(self):
        return {"K": self.K, "Q": self.Q, "nspecies": self.nspecies, "L": self.L, "tmax": self.tmax,
                "params": self.params.astype(float).tolist()}

    @classmethod
    def from_dict(cls, d):
        return cls(int(d["K"]), int(d["Q"]), int(d["nspecies"]), int(d["L"]), float(d["tmax"]),
                   np.asarray(d["params"], dtype=np.float32))


def student_spec(maxorder: int, maxdeg: int, K: int, maxL: int, **kw) -> ACESpec:
    """Single-species spec whose radial index n <= K is the MLP channel k."""
    return symmetric_basis(maxorder, maxdeg, nR=K, maxL=maxL, **kw)


def learned_context(spec: ACESpec, mlp: RadialMLP, device: int = 0, precision: str = "fp32") -> Context:
    ctx = Context(spec, precision, device)
    ctx.set_radial_mlp(mlp.params, mlp.K, mlp.Q, mlp.nspecies, mlp.tmax)
    return ctx


def _torch():
    import torch
    return torch


class _Trainer:
    """Device buffers for the MLP parameters' gradient and Adam moments."""

    def __init__(self, ctx: Context, mlp: RadialMLP, device):
        torch = _torch()
        self.ctx = ctx
        self.mlp = mlp
        self.dev = device
        self.w_ptr, self.n = ctx.radial_mlp_params()
        self.g = torch.zeros(self.n, dtype=torch.float32, device=device)
        self.m = torch.zeros_like(self.g)
        self.v = torch.zeros_like(self.g)
        self.step = 0

    def adam(self, lr):
        self.step += 1
        self.ctx.adam_step(self.w_ptr, self.g, self.m, self.v, lr, self.step)

    def params_to_host(self):
        self.mlp.params = self.ctx.radial_mlp_get_params()
        return self.mlp.params


def pca_radial_targets(teacher: ACESpec, K: int, L: int, r: np.ndarray, sp: np.ndarray, chunk: int = 200_000):
    """Species-aware radial targets: for every l, the K leading principal
    directions (over the samples) of the teacher's radial x species channels
    R_n(r) [s = s'] with (n-1) + l <= maxdeg -- the best K-dimensional linear
    compression of the channels the teacher's A entries of that l use -- each
    scaled to unit RMS.  Returns (N, K (L+1)) float32, channel k + K l."""
    S = teacher.nspecies
    deg = float(teacher.info.get("maxdeg", len(teacher.radial.J.A)))
    nR = len(teacher.radial.J.A)
    N = len(r)
    out = np.zeros((N, K * (L + 1)), dtype=np.float32)
    for l in range(L + 1):
        nl = int(min(nR, np.floor(deg - l + 1e-9) + 1))
        if nl <= 0:
            continue
        G = np.zeros((nl * S, nl * S))
        for i0 in range(0, N, chunk):
            R = teacher.radial.evaluate(r[i0:i0 + chunk])[:, :nl]
            X = np.zeros((len(R), nl * S))
            for s_ in range(S):
                m = sp[i0:i0 + chunk] == s_
                X[m, s_ * nl:(s_ + 1) * nl] = R[m]
            G += X.T @ X
        w, V = np.linalg.eigh(G / N)
        V = V[:, ::-1][:, :K]
        w = np.maximum(w[::-1][:K], 1e-30)
        kk = V.shape[1]
        for i0 in range(0, N, chunk):
            R = teacher.radial.evaluate(r[i0:i0 + chunk])[:, :nl]
            X = np.zeros((len(R), nl * S))
            for s_ in range(S):
                m = sp[i0:i0 + chunk] == s_
                X[m, s_ * nl:(s_ + 1) * nl] = R[m]
            out[i0:i0 + chunk, K * l:K * l + kk] = (X @ V) / np.sqrt(w)
    return out


def pretrain_radial(ctx: Context, mlp: RadialMLP, spec: ACESpec, nsamples: int = 2_000_000, steps: int = 1500,
                    batch: int = 32768, lr: float = 2e-3, rlo: float = 0.8, rhi: float = 5.0, seed: int = 7,
                    teacher: ACESpec | None = None, log=None):
    """Regress the MLP's channels (k, l) on seeded neighbour samples r ~
    U[rlo, rhi], species uniform, onto either the teacher's compressed
    radial x species channels (``pca_radial_targets``, when a teacher spec is
    given) or the student spec's own polynomial R_k(r) for every l and
    species (the species-blind radial basis of width K); returns the loss
    history."""
    torch = _torch()
    dev = torch.device("cuda", ctx.device)
    rng = np.random.default_rng(seed)
    r = rlo + (rhi - rlo) * rng.random(nsamples)
    sp = rng.integers(0, mlp.nspecies, nsamples).astype(np.int32)
    rr = np.zeros((nsamples, 3))
    rr[:, 0] = r
    rr_d = torch.from_numpy(rr).to(dev)
    sp_d = torch.from_numpy(sp).to(dev)
    C = mlp.C
    if teacher is not None:
        T_d = torch.from_numpy(pca_radial_targets(teacher, mlp.K, mlp.L, r, sp)).to(dev)
    else:
        T_d = torch.from_numpy(spec.radial.evaluate(r)[:, :mlp.K].astype(np.float32)).to(dev)
    out = torch.empty((batch, 2 * C), dtype=torch.float32, device=dev)
    tr = _Trainer(ctx, mlp, dev)
    hist = []
    perm = torch.randperm(nsamples, device=dev, generator=torch.Generator(device=dev).manual_seed(seed))
    pos = 0
    for it in range(steps):
        if pos + batch > nsamples:
            perm = perm[torch.randperm(nsamples, device=dev)]
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        rb, sb = rr_d[idx].contiguous(), sp_d[idx].contiguous()
        ctx.radial_mlp_forward(rb, sb, out)
        R = out[:, :C]
        T = T_d[idx] if teacher is not None else T_d[idx].repeat(1, mlp.L + 1)
        diff = R - T
        gR = (2.0 / (batch * C)) * diff
        tr.g.zero_()
        ctx.radial_mlp_backward(rb, sb, gR.contiguous(), None, tr.g)
        tr.adam(lr if it < 0.7 * steps else lr * 0.1)
        if it % 100 == 0 or it == steps - 1:
            loss = float((diff * diff).mean())
            hist.append((it, loss))
            if log:
                log(f"pretrain {it}: mse {loss:.3e}")
    tr.params_to_host()
    return hist


def fit_coefficients(ctx: Context, spec: ACESpec, b: Batch, E_target: np.ndarray, ridge: float = 1e-8,
                     forces=None):
    """Ridge least squares for the student's basis coefficients c: energy
    rows B c = E over the environments of b and, with forces = (bf, G, w),
    gradient rows dB c = dE/drr over the neighbours of bf (weight w), each
    block normalised by its target variance; the basis and its derivative
    come from the GPU basis path (learned radials included)."""
    torch = _torch()
    dev = torch.device("cuda", ctx.device)
    nB = spec.nB
    B = torch.empty((b.nenv, nB), dtype=torch.float64, device=dev)
    ctx.basis_to_device(b.offsets, b.rr, b.species, B)
    Et = torch.from_numpy(np.asarray(E_target, dtype=np.float64)).to(dev)
    se = float(Et.var()) or 1.0
    G = (B.T @ B) / (b.nenv * se)
    rhs = (B.T @ Et) / (b.nenv * se)
    del B
    if forces is not None:
        bf, Gt, w = forces
        Bf = torch.empty((bf.nenv, nB), dtype=torch.float64, device=dev)
        dB = torch.empty((bf.nnbr, nB, 3), dtype=torch.float64, device=dev)
        ctx.basis_to_device(bf.offsets, bf.rr, bf.species, Bf, dB)
        D = dB.permute(0, 2, 1).reshape(-1, nB)
        del dB, Bf
        g = torch.from_numpy(np.ascontiguousarray(Gt, dtype=np.float64).reshape(-1)).to(dev)
        sf = float((g * g).mean()) or 1.0
        G += w * (D.T @ D) / (len(g) * sf)
        rhs += w * (D.T @ g) / (len(g) * sf)
        del D
    # the normal equations are nB x nB: solved on the host
    Gh, rh = G.cpu().numpy(), rhs.cpu().numpy()
    Gh[np.diag_indices(nB)] += ridge * np.trace(Gh) / nB
    return np.linalg.solve(Gh, rh)


def force_loss_gradient(ctx: Context, g, off, rr, sp, G, Gt, weight, E_buf, GR_buf, disp: float = 1e-2):
    """Adds to the parameter gradient g the gradient of the force loss
    weight * mean_j |G_j - Gt_j|^2 / mean |Gt|^2 over one batch (device
    tensors; G = dE/drr of the learned form at the current parameters).

    With W_j = dL_F/dG_j held fixed, dL_F/dtheta = d/dtheta sum_j W_j . G_j,
    and sum_j W_j . G_j = d/deps sum_e E_e(rr + eps W) at eps = 0, so the
    gradient is d/deps of the parameter gradient of the energies summed over
    the batch: the central difference of the exact energy gradients at
    rr +- h W, with h chosen so that the largest displacement is `disp`
    (Angstrom).  Returns the loss value."""
    torch = _torch()
    res = G - Gt
    n3 = res.numel()
    sf = float((Gt * Gt).mean()) or 1.0
    W = (2.0 * weight / (n3 * sf)) * res
    wmax = float(W.abs().max())
    loss = weight * float((res * res).mean()) / sf
    if wmax == 0.0:
        return loss
    h = disp / wmax
    n = rr.shape[0]
    for sgn in (1.0, -1.0):
        rs = (rr + (sgn * h) * W).contiguous()
        ctx.energy_radial_adjoint(off, rs, sp, E_buf, None, GR_buf[:n])
        wj = torch.full((n,), sgn / (2.0 * h), dtype=torch.float32, device=rr.device)
        ctx.radial_mlp_backward(rs, sp, GR_buf[:n], wj, g)
    return loss


def sub_batch(b: Batch, e0: int, e1: int) -> Batch:
    o0, o1 = int(b.offsets[e0]), int(b.offsets[e1])
    return Batch(b.offsets[e0:e1 + 1] - o0, b.rr[o0:o1], None if b.species is None else b.species[o0:o1])


def distill(ctx: Context, mlp: RadialMLP, spec: ACESpec, train: Batch, E_train: np.ndarray, c: np.ndarray,
            steps: int = 2000, batch_envs: int = 512, lr: float = 1e-3, refit_every: int = 500,
            refit_envs: int = 20000, forces=None, force_loss=None, log=None):
    """Adam on the MLP parameters against teacher energies (c fixed between
    ridge re-fits, which also use the teacher gradients `forces` when
    given, see fit_coefficients); returns (c, history).

    force_loss = (bf, Gt, weight, batch_envs): each step also adds the
    gradient of weight * the relative mean-square force error on a batch of
    the environments of bf (teacher gradients Gt), see force_loss_gradient."""
    torch = _torch()
    dev = torch.device("cuda", ctx.device)
    off_d = torch.from_numpy(train.offsets).to(dev)
    rr_d = torch.from_numpy(train.rr).to(dev)
    sp_d = None if train.species is None else torch.from_numpy(train.species).to(dev)
    Et_d = torch.from_numpy(np.asarray(E_train, dtype=np.float64)).to(dev)
    J = torch.from_numpy(np.diff(train.offsets)).to(dev)
    var = float(np.var(E_train))
    nEnv = train.nenv
    maxn = int(np.max(train.offsets[batch_envs:] - train.offsets[:-batch_envs])) if nEnv > batch_envs else \
        int(train.offsets[-1])
    E_b = torch.empty(batch_envs, dtype=torch.float64, device=dev)
    GR = torch.empty((maxn, mlp.C), dtype=torch.float32, device=dev)
    tr = _Trainer(ctx, mlp, dev)
    ctx.set_params(c)
    hist = []
    rng = np.random.default_rng(11)
    refit = sub_batch(train, 0, min(refit_envs, nEnv))
    if force_loss is not None:
        fb, fG, fw, fbe = force_loss
        f_off = torch.from_numpy(fb.offsets).to(dev)
        f_rr = torch.from_numpy(fb.rr).to(dev)
        f_sp = None if fb.species is None else torch.from_numpy(fb.species).to(dev)
        f_Gt = torch.from_numpy(np.ascontiguousarray(fG, dtype=np.float64).reshape(-1, 3)).to(dev)
        fbe = min(fbe, fb.nenv)
        fmax = int(np.max(fb.offsets[fbe:] - fb.offsets[:-fbe])) if fb.nenv > fbe else int(fb.offsets[-1])
        f_E = torch.empty(fbe, dtype=torch.float64, device=dev)
        f_G = torch.empty((fmax, 3), dtype=torch.float64, device=dev)
        if fmax > GR.shape[0]:
            GR = torch.empty((fmax, mlp.C), dtype=torch.float32, device=dev)
    for it in range(steps):
        e0 = int(rng.integers(0, max(1, nEnv - batch_envs)))
        e1 = min(nEnv, e0 + batch_envs)
        ne = e1 - e0
        o0, o1 = int(train.offsets[e0]), int(train.offsets[e1])
        off_b = (off_d[e0:e1 + 1] - o0).contiguous()
        rr_b = rr_d[o0:o1]
        sp_b = None if sp_d is None else sp_d[o0:o1]
        Eb = E_b[:ne]
        ctx.energy_radial_adjoint(off_b, rr_b, sp_b, Eb, None, GR[:o1 - o0])
        res = Eb - Et_d[e0:e1]
        w = (2.0 / (ne * var)) * res
        wj = torch.repeat_interleave(w, J[e0:e1]).to(torch.float32)
        tr.g.zero_()
        ctx.radial_mlp_backward(rr_b, sp_b, GR[:o1 - o0], wj, tr.g)
        floss = 0.0
        if force_loss is not None:
            q0 = int(rng.integers(0, max(1, fb.nenv - fbe)))
            q1 = min(fb.nenv, q0 + fbe)
            p0, p1 = int(fb.offsets[q0]), int(fb.offsets[q1])
            fo = (f_off[q0:q1 + 1] - p0).contiguous()
            fr = f_rr[p0:p1]
            fs = None if f_sp is None else f_sp[p0:p1]
            ctx.energy_radial_adjoint(fo, fr, fs, f_E[:q1 - q0], f_G[:p1 - p0], GR[:p1 - p0])
            floss = force_loss_gradient(ctx, tr.g, fo, fr, fs, f_G[:p1 - p0], f_Gt[p0:p1], fw, f_E[:q1 - q0], GR)
        step_lr = lr * (0.1 if it >= 0.8 * steps else 1.0)
        tr.adam(step_lr)
        if it % 100 == 0 or it == steps - 1:
            loss = float((res * res).mean()) / var
            hist.append((it, loss, floss) if force_loss is not None else (it, loss))
            if log:
                log(f"distill {it}: rel mse {loss:.3e} force {floss:.3e}")
        if refit_every and (it + 1) % refit_every == 0 and it + 1 < steps:
            torch.cuda.synchronize()
            c = fit_coefficients(ctx, spec, refit, E_train[:refit.nenv], forces=forces)
            ctx.set_params(c)
    tr.params_to_host()
    c = fit_coefficients(ctx, spec, refit, E_train[:refit.nenv], forces=forces)
    ctx.set_params(c)
    return c, hist


def energy_error(E, Eref):
    """Relative RMS error and max per-environment error normalised by
    max(|E|, rms E) of the reference."""
    E, Eref = np.asarray(E), np.asarray(Eref)
    rms = np.sqrt(np.mean(Eref ** 2))
    return {"rel_rmse": float(np.sqrt(np.mean((E - Eref) ** 2)) / rms),
            "rel_max": float(np.max(np.abs(E - Eref) / np.maximum(np.abs(Eref), rms)))}


class LearnedRadialModel:
    """The student (learned radials) with the teacher (plain basis) as its
    fallback for environments outside the training envelope."""

    def __init__(self, spec: ACESpec, mlp: RadialMLP, c: np.ndarray, fallback: Context,
                 r_envelope=(0.8, 5.0), device: int = 0):
        self.spec = spec
        self.mlp = mlp
        self.ctx = learned_context(spec, mlp, device)
        self.ctx.set_params(c)
        self.fallback = fallback
        self.rlo, self.rhi = r_envelope

    def inside(self, b: Batch) -> np.ndarray:
        """Environments whose neighbours all lie in the training radii and
        species range."""
        r = np.linalg.norm(b.rr, axis=1)
        bad = (r < self.rlo) | (r > self.rhi)
        if b.species is not None:
            bad |= (b.species < 0) | (b.species >= self.mlp.nspecies)
        cs = np.concatenate([[0], np.cumsum(bad, dtype=np.int64)])
        return (cs[b.offsets[1:]] - cs[b.offsets[:-1]]) == 0

    def energy_forces(self, b: Batch):
        """E, dE/drr and the mask of environments the student evaluated."""
        ok = self.inside(b)
        E = np.empty(b.nenv)
        G = np.empty_like(b.rr)
        J_all = np.diff(b.offsets)
        for mask, ctx in ((ok, self.ctx), (~ok, self.fallback)):
            idx = np.nonzero(mask)[0]
            if len(idx) == 0:
                continue
            J = J_all[idx]
            off = np.concatenate([[0], np.cumsum(J)])
            nb = np.repeat(b.offsets[idx] - off[:-1], J) + np.arange(off[-1])
            sp = None if b.species is None else b.species[nb]
            Es, Gs = ctx.energy_forces(off, b.rr[nb], sp)
            E[idx] = Es
            G[nb] = Gs
        return E, G, ok
