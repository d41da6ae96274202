"""Host-side mirror of ACE.jl's model API, evaluated by libace_b200.

Same names and argument meaning as the reference:

* ``SymmetricBasis(maxorder, maxdeg, ...)``       -- src/symmbasis.jl:74-82
  (``evaluate``, ``evaluate_d``, ``evaluate_ed``  -- :297-336)
* ``LinearACEModel(basis, c, evaluator="gpu")``   -- src/linearmodel.jl:44-56
  (``evaluate``, ``grad_config``, ``grad_params``, ``grad_params_config``,
  ``set_params``, ``params``                      -- :63-71,107-128)
* ``ACEConfig`` / a list of positions            -- src/states.jl:422-430,
  src/ACE.jl:157-170

A configuration is an (J, 3) array of neighbour positions rr_j (and, for a
multi-species basis, a species index per neighbour).  Passing a list of
configurations evaluates them in one batched call; results come back per
configuration.  ACE.jl raises on an empty configuration
(src/product_1pbasis.jl:124); here an empty configuration is accepted and
gives E = c~_0 (the order-0 coefficient) and an empty gradient.

There is no CPU fallback: the library must be built, and a GPU present.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .lib import Context
from .spec import ACESpec, random_coefficients, symmetric_basis


@dataclass
class ACEConfig:
    rr: np.ndarray
    species: np.ndarray | None = None

    def __len__(self):
        return len(self.rr)


def _pack(cfgs):
    single = isinstance(cfgs, (ACEConfig, np.ndarray))
    if single:
        cfgs = [cfgs]
    cfgs = [c if isinstance(c, ACEConfig) else ACEConfig(np.asarray(c, dtype=np.float64).reshape(-1, 3))
            for c in cfgs]
    offsets = np.zeros(len(cfgs) + 1, dtype=np.int64)
    np.cumsum([len(c) for c in cfgs], out=offsets[1:])
    rr = np.concatenate([np.asarray(c.rr, dtype=np.float64).reshape(-1, 3) for c in cfgs]) if cfgs else \
        np.zeros((0, 3))
    if any(c.species is not None for c in cfgs):
        sp = np.concatenate([np.asarray(c.species, dtype=np.int32) for c in cfgs])
    else:
        sp = None
    return single, offsets, rr, sp


class SymmetricBasis:
    """Rotation-invariant ACE basis (Invariant property, O3 group,
    SimpleSparseBasis selector) over an Rn x Ylm [x species] 1p basis."""

    def __init__(self, maxorder: int | None = None, maxdeg: float | None = None, spec: ACESpec | None = None,
                 precision: str = "fp64", device: int = 0, **kw):
        self.spec = spec if spec is not None else symmetric_basis(maxorder, maxdeg, **kw)
        self.precision = precision
        self.device = device
        self._ctx = None

    def __len__(self):
        return self.spec.nB

    @property
    def ctx(self) -> Context:
        if self._ctx is None:
            self._ctx = Context(self.spec, self.precision, self.device)
        return self._ctx

    def evaluate(self, cfgs):
        single, off, rr, sp = _pack(cfgs)
        B = self.ctx.basis(off, rr, sp)
        return B[0] if single else B

    def evaluate_ed(self, cfgs):
        single, off, rr, sp = _pack(cfgs)
        B, dB = self.ctx.basis(off, rr, sp, grad=True)
        parts = [dB[off[e]:off[e + 1]].transpose(1, 0, 2) for e in range(len(off) - 1)]
        return (B[0], parts[0]) if single else (B, parts)

    def evaluate_d(self, cfgs):
        return self.evaluate_ed(cfgs)[1]


class LinearACEModel:
    """E(cfg) = sum_b c_b B_b(cfg), evaluated through c~ = U^T c.

    With a 2-D c of shape (nB, nprop) the model has nprop properties
    (ACE.jl's c::Vector{SVector{N}}, src/linearmodel.jl:28-35): energies come
    back as (..., nprop) and gradients as (J, nprop, 3)."""

    def __init__(self, basis: SymmetricBasis, c=None, evaluator: str = "gpu"):
        if evaluator not in ("gpu", "standard"):
            raise ValueError("unknown evaluator")
        self.basis = basis
        self.c = np.zeros(len(basis)) if c is None else np.array(c, dtype=np.float64)
        self.ctx = Context(basis.spec, basis.precision, basis.device)
        self._push()

    @property
    def multi(self):
        return self.c.ndim == 2

    def _push(self):
        if self.multi:
            self.ctx.set_params_multi(self.c)
        else:
            self.ctx.set_params(self.c)

    def _ef(self, off, rr, sp, forces=True):
        if self.multi:
            return self.ctx.energy_forces_multi(off, rr, sp)
        return self.ctx.energy_forces(off, rr, sp, forces=forces)

    def params(self):
        return self.c.copy()

    def nparams(self):
        return len(self.c)

    def set_params(self, c):
        self.c[...] = c
        self._push()
        return self

    def evaluate(self, cfgs):
        single, off, rr, sp = _pack(cfgs)
        E = self._ef(off, rr, sp, forces=False)
        if self.multi:
            E = E[0]
        return E[0] if single else E

    def grad_config(self, cfgs):
        single, off, rr, sp = _pack(cfgs)
        _, G = self._ef(off, rr, sp)
        parts = [G[off[e]:off[e + 1]] for e in range(len(off) - 1)]
        return parts[0] if single else parts

    def energy_forces(self, cfgs):
        """Energies and forces F_j = -dE/drr_j in one pass."""
        single, off, rr, sp = _pack(cfgs)
        E, G = self._ef(off, rr, sp)
        F = [-G[off[e]:off[e + 1]] for e in range(len(off) - 1)]
        return (E[0], F[0]) if single else (E, F)

    def grad_params(self, cfgs):
        return self.basis.evaluate(cfgs)

    def grad_params_config(self, cfgs):
        return self.basis.evaluate_d(cfgs)


class LinearVectorModel:
    """A linear model over an EuclideanVector basis (``spec.vector_basis``):
    V(cfg) = sum_b c_b B_b(cfg) in R^3 (src/properties.jl:154-248 with
    src/linearmodel.jl's evaluate / grad_config).  Evaluated as three
    complex-coefficient properties (x, y, z) on the GPU."""

    def __init__(self, spec, c, precision: str = "fp64", device: int = 0):
        self.spec = spec
        self.c = np.array(c, dtype=np.float64)
        self.ctx = Context(spec, precision, device)
        self.set_params(self.c)

    def set_params(self, c):
        self.c[...] = c
        self.ctx.set_ctilde_complex(self.spec.ctilde_vector(self.c))
        return self

    def evaluate(self, cfgs):
        """V (3,) per configuration."""
        single, off, rr, sp = _pack(cfgs)
        E, _ = self.ctx.energy_forces_multi(off, rr, sp)      # (nEnv, 3)
        return E[0] if single else E

    def grad_config(self, cfgs):
        """dV_i/drr_j[a] as (J, 3, 3) (i = component, a = coordinate) per configuration."""
        single, off, rr, sp = _pack(cfgs)
        _, G = self.ctx.energy_forces_multi(off, rr, sp)      # (nNbr, 3, 3)
        parts = [G[off[e]:off[e + 1]] for e in range(len(off) - 1)]
        return parts[0] if single else parts


class LinearSphericalModel:
    """A linear model over a SphericalVector{L} basis (``spec.spherical_basis``):
    V_M(cfg) = sum_b c_b B_b^M(cfg), complex, M = -L..L.  Evaluated as
    2 (2L+1) complex-coefficient properties: Re V_M with c~^M and
    Im V_M = Re(-i c~^M . AA)."""

    def __init__(self, spec, c, precision: str = "fp64", device: int = 0):
        self.spec = spec
        self.L = spec.Lout
        self.c = np.array(c, dtype=np.float64)
        self.ctx = Context(spec, precision, device)
        self.set_params(self.c)

    def set_params(self, c):
        self.c[...] = c
        ct = self.spec.ctilde_spherical(self.c).astype(np.complex128)
        self.ctx.set_ctilde_complex(np.concatenate([ct, -1j * ct]))
        return self

    def _eval(self, cfgs):
        single, off, rr, sp = _pack(cfgs)
        E, G = self.ctx.energy_forces_multi(off, rr, sp)      # (nEnv, 2n), (nNbr, 2n, 3)
        n = 2 * self.L + 1
        return single, off, E[:, :n] + 1j * E[:, n:], G[:, :n] + 1j * G[:, n:]

    def evaluate(self, cfgs):
        """V (2L+1,) complex per configuration."""
        single, _, V, _ = self._eval(cfgs)
        return V[0] if single else V

    def grad_config(self, cfgs):
        """dV_M/drr_j[a] as (J, 2L+1, 3) complex per configuration."""
        single, off, _, G = self._eval(cfgs)
        parts = [G[off[e]:off[e + 1]] for e in range(len(off) - 1)]
        return parts[0] if single else parts


__all__ = ["ACEConfig", "SymmetricBasis", "LinearACEModel", "LinearVectorModel", "LinearSphericalModel",
           "random_coefficients", "symmetric_basis"]
