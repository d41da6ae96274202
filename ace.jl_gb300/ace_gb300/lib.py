"""ctypes binding of libace_b200 (the C ABI declared in include/ace_b200.h)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

ACE_OK = 0
ACE_ERR_INVALID = 1
ACE_ERR_CUDA = 2
ACE_ERR_ALLOC = 3
ACE_ERR_KERNEL = 4
ACE_ERR_UNSUPPORTED = 5

PREC = {"fp64": 0, "fp32": 1, "fp32_bf16x3": 2, "fp32x2": 4, "fp32c": 5}

ACE_INPUTS_ON_DEVICE = 1
ACE_OUTPUTS_ON_DEVICE = 2
ACE_ASYNC = 4

EXPORTED = ("ace_ctx_create", "ace_ctx_destroy", "ace_set_params", "ace_set_ctilde",
            "ace_energy_forces", "ace_energy", "ace_basis", "ace_sync", "ace_get_spec_sizes",
            "ace_last_error_string", "ace_launch_count", "ace_basis_noalloc", "ace_adjoint_eval_d",
            "ace_set_params_multi", "ace_energy_forces_multi", "ace_autotune", "ace_set_radial_mlp",
            "ace_radial_mlp_params", "ace_radial_mlp_forward", "ace_radial_mlp_backward",
            "ace_energy_radial_adjoint", "ace_adam_step", "ace_radial_mlp_get_params", "ace_radial_mlp_infer",
            "ace_set_ctilde_complex", "ace_set_energy_tolerance", "ace_energy_error_estimates")


class AceError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libace_b200 error {code}: {msg}")
        self.code = code


class SpecBundle(C.Structure):
    _fields_ = [
        ("version", C.c_int32), ("nR", C.c_int32),
        ("rA", C.c_void_p), ("rB", C.c_void_p), ("rC", C.c_void_p),
        ("pl", C.c_int32), ("pr", C.c_int32), ("tl", C.c_double), ("tr", C.c_double),
        ("tp", C.c_int32), ("r0", C.c_double),
        ("nA", C.c_int32), ("a_n", C.c_void_p), ("a_l", C.c_void_p), ("a_m", C.c_void_p), ("a_mu", C.c_void_p),
        ("nspecies", C.c_int32),
        ("nAA", C.c_int64), ("maxord", C.c_int32), ("orders", C.c_void_p), ("iAA2iA", C.c_void_p),
        ("nB", C.c_int64), ("U_indptr", C.c_void_p), ("U_indices", C.c_void_p), ("U_data", C.c_void_p),
    ]


class RadialMLPDesc(C.Structure):
    _fields_ = [("version", C.c_int32), ("K", C.c_int32), ("Q", C.c_int32), ("nspecies", C.c_int32),
                ("H", C.c_int32), ("tmax", C.c_double), ("params", C.c_void_p), ("nparams", C.c_int64)]


_lib = None


def load(path: str | None = None):
    """Load libace_b200.so (it must have been built; the product has no
    fallback when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libace_b200.so not built at {path}; run __graft_entry__.build()")
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.ace_ctx_create.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]
    lib.ace_ctx_destroy.argtypes = [P]
    lib.ace_set_params.argtypes = [P, P, C.c_int64]
    lib.ace_set_ctilde.argtypes = [P, P, C.c_int64]
    lib.ace_energy_forces.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int32, P]
    lib.ace_energy.argtypes = [P, C.c_int64, P, P, P, P, C.c_int32, P]
    lib.ace_basis.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int32, P]
    lib.ace_basis_noalloc.argtypes = [P, C.c_int64, P, P, P, P, P]
    lib.ace_adjoint_eval_d.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int32, P]
    lib.ace_set_params_multi.argtypes = [P, P, C.c_int64, C.c_int32]
    lib.ace_autotune.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int32, P, P]
    lib.ace_energy_forces_multi.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int32, P]
    lib.ace_set_radial_mlp.argtypes = [P, P]
    lib.ace_radial_mlp_params.argtypes = [P, P, P]
    lib.ace_radial_mlp_forward.argtypes = [P, C.c_int64, P, P, P, P]
    lib.ace_radial_mlp_get_params.argtypes = [P, P, C.c_int32]
    lib.ace_radial_mlp_infer.argtypes = [P, C.c_int64, P, P, P, P]
    lib.ace_set_ctilde_complex.argtypes = [P, P, C.c_int64, C.c_int32]
    lib.ace_radial_mlp_backward.argtypes = [P, C.c_int64, P, P, P, P, P, P]
    lib.ace_energy_radial_adjoint.argtypes = [P, C.c_int64, P, P, P, P, P, P, P]
    lib.ace_adam_step.argtypes = [C.c_int64, P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32, P]
    lib.ace_sync.argtypes = [P]
    lib.ace_get_spec_sizes.argtypes = [P, P]
    lib.ace_last_error_string.argtypes = [P]
    lib.ace_last_error_string.restype = C.c_char_p
    lib.ace_launch_count.argtypes = [P]
    lib.ace_launch_count.restype = C.c_int64
    lib.ace_set_energy_tolerance.argtypes = [P, C.c_double]
    lib.ace_energy_error_estimates.argtypes = [P, C.c_int64, P, P]
    for name in ("ace_ctx_create", "ace_ctx_destroy", "ace_set_params", "ace_set_ctilde",
                 "ace_energy_forces", "ace_energy", "ace_basis", "ace_sync", "ace_get_spec_sizes",
                 "ace_basis_noalloc", "ace_adjoint_eval_d",
            "ace_set_params_multi", "ace_energy_forces_multi", "ace_autotune", "ace_set_radial_mlp",
                 "ace_radial_mlp_params", "ace_radial_mlp_forward", "ace_radial_mlp_backward",
                 "ace_energy_radial_adjoint", "ace_adam_step", "ace_radial_mlp_get_params",
                 "ace_radial_mlp_infer", "ace_set_ctilde_complex", "ace_set_energy_tolerance",
                 "ace_energy_error_estimates"):
        getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a.data_ptr()))  # torch tensor


def make_bundle(spec):
    """SpecBundle (+ the arrays it points to, which must stay alive)."""
    keep = {}
    R = spec.radial
    keep["rA"] = np.ascontiguousarray(R.J.A, dtype=np.float64)
    keep["rB"] = np.ascontiguousarray(R.J.B, dtype=np.float64)
    keep["rC"] = np.ascontiguousarray(R.J.C, dtype=np.float64)
    a = spec.aspec
    keep["a_n"] = np.ascontiguousarray(a.n - 1, dtype=np.int32)
    keep["a_l"] = np.ascontiguousarray(a.l, dtype=np.int32)
    keep["a_m"] = np.ascontiguousarray(a.m, dtype=np.int32)
    keep["a_mu"] = np.ascontiguousarray(a.mu, dtype=np.int32)
    keep["orders"] = np.ascontiguousarray(spec.orders, dtype=np.int32)
    keep["iAA2iA"] = np.ascontiguousarray(spec.iAA2iA, dtype=np.int32)
    U = spec.U.tocsr()
    U.sort_indices()
    keep["U_indptr"] = np.ascontiguousarray(U.indptr, dtype=np.int64)
    keep["U_indices"] = np.ascontiguousarray(U.indices, dtype=np.int32)
    keep["U_data"] = np.ascontiguousarray(U.data, dtype=np.float64)
    b = SpecBundle()
    b.version = 1
    b.nR = len(keep["rA"])
    b.rA, b.rB, b.rC = _ptr(keep["rA"]), _ptr(keep["rB"]), _ptr(keep["rC"])
    b.pl, b.pr, b.tl, b.tr = R.J.pl, R.J.pr, R.J.tl, R.J.tr
    b.tp, b.r0 = R.trans.p, R.trans.r0
    b.nA = spec.nA
    b.a_n, b.a_l, b.a_m = _ptr(keep["a_n"]), _ptr(keep["a_l"]), _ptr(keep["a_m"])
    b.a_mu = _ptr(keep["a_mu"])
    b.nspecies = spec.nspecies
    b.nAA, b.maxord = spec.nAA, spec.maxorder
    b.orders, b.iAA2iA = _ptr(keep["orders"]), _ptr(keep["iAA2iA"])
    b.nB = U.shape[0]
    b.U_indptr, b.U_indices, b.U_data = _ptr(keep["U_indptr"]), _ptr(keep["U_indices"]), _ptr(keep["U_data"])
    return b, keep


class Context:
    """One libace_b200 context: the spec on one device, in one precision."""

    def __init__(self, spec, precision: str = "fp64", device: int = 0):
        self.lib = load()
        self.spec = spec
        self.precision = precision
        self.device = device
        bundle, self._keep = make_bundle(spec)
        h = C.c_void_p()
        rc = self.lib.ace_ctx_create(C.byref(bundle), PREC[precision], device, C.byref(h))
        if rc != ACE_OK:
            raise AceError(rc, self.lib.ace_last_error_string(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.ace_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != ACE_OK:
            raise AceError(rc, self.lib.ace_last_error_string(self.h).decode())

    def set_params(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64)
        self._check(self.lib.ace_set_params(self.h, _ptr(c), len(c)))

    def set_ctilde(self, ct):
        ct = np.ascontiguousarray(ct, dtype=np.float64)
        self._check(self.lib.ace_set_ctilde(self.h, _ptr(ct), len(ct)))

    def launch_count(self) -> int:
        return int(self.lib.ace_launch_count(self.h))

    # host-buffer entry points (numpy in, numpy out)
    def energy_forces(self, offsets, rr, species=None, forces=True):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        rr = np.ascontiguousarray(rr, dtype=np.float64).reshape(-1, 3)
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        nenv = len(offsets) - 1
        E = np.empty(nenv)
        G = np.empty_like(rr) if forces else None
        self._check(self.lib.ace_energy_forces(self.h, nenv, _ptr(offsets), _ptr(rr), _ptr(sp),
                                               _ptr(E), _ptr(G), 0, None))
        return (E, G) if forces else E

    def basis(self, offsets, rr, species=None, grad=False):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        rr = np.ascontiguousarray(rr, dtype=np.float64).reshape(-1, 3)
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        nenv = len(offsets) - 1
        B = np.empty((nenv, self.spec.nB))
        dB = np.empty((len(rr), self.spec.nB, 3)) if grad else None
        self._check(self.lib.ace_basis(self.h, nenv, _ptr(offsets), _ptr(rr), _ptr(sp),
                                       _ptr(B), _ptr(dB), 0, None))
        return (B, dB) if grad else B

    def basis_device(self, offsets, rr, species, B, stream=None, sync=True):
        """B (nEnv, nB) of device inputs into a device tensor."""
        flags = ACE_INPUTS_ON_DEVICE | ACE_OUTPUTS_ON_DEVICE | (0 if sync else ACE_ASYNC)
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_basis(self.h, B.shape[0], _ptr(offsets), _ptr(rr), _ptr(species), _ptr(B), None,
                                       flags, st))

    def basis_to_device(self, offsets, rr, species, B, dB=None):
        """B (and dB) of host inputs into device tensors B (nEnv, nB) and dB
        (nNbr, nB, 3)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        rr = np.ascontiguousarray(rr, dtype=np.float64).reshape(-1, 3)
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        self._check(self.lib.ace_basis(self.h, len(offsets) - 1, _ptr(offsets), _ptr(rr), _ptr(sp),
                                       _ptr(B), _ptr(dB), ACE_OUTPUTS_ON_DEVICE, None))

    def set_params_multi(self, c):
        """c: (nB, nprop) -- one column of coefficients per property."""
        c = np.asarray(c, dtype=np.float64)
        cm = np.ascontiguousarray(c.T)
        self.nprop = cm.shape[0]
        self._check(self.lib.ace_set_params_multi(self.h, _ptr(cm), cm.shape[1], cm.shape[0]))

    def set_ctilde_complex(self, ct):
        """ct: complex (nprop, nAA); property p evaluates Re(sum_k ct[p, k] AA_k)."""
        ct = np.atleast_2d(np.asarray(ct, dtype=np.complex128))
        buf = np.ascontiguousarray(np.stack([ct.real, ct.imag], axis=-1))
        self._check(self.lib.ace_set_ctilde_complex(self.h, _ptr(buf), ct.shape[1], ct.shape[0]))
        self.nprop = ct.shape[0]

    def energy_forces_multi(self, offsets, rr, species=None):
        """E (nEnv, nprop) and dE/drr (nNbr, nprop, 3)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        rr = np.ascontiguousarray(rr, dtype=np.float64).reshape(-1, 3)
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        nenv = len(offsets) - 1
        E = np.empty((self.nprop, nenv))
        G = np.empty((self.nprop, len(rr), 3))
        self._check(self.lib.ace_energy_forces_multi(self.h, nenv, _ptr(offsets), _ptr(rr), _ptr(sp),
                                                     _ptr(E), _ptr(G), 0, None))
        return E.T.copy(), G.transpose(1, 0, 2).copy()

    def adjoint_eval_d(self, offsets, rr, w, species=None):
        """adjoint_EVAL_D: per environment, sum_j w_j . dB/drr_j (nEnv x nB)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        rr = np.ascontiguousarray(rr, dtype=np.float64).reshape(-1, 3)
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(-1, 3)
        sp = None if species is None else np.ascontiguousarray(species, dtype=np.int32)
        nenv = len(offsets) - 1
        out = np.empty((nenv, self.spec.nB))
        self._check(self.lib.ace_adjoint_eval_d(self.h, nenv, _ptr(offsets), _ptr(rr), _ptr(sp), _ptr(w),
                                                _ptr(out), 0, None))
        return out

    # device-buffer entry point (torch CUDA tensors in and out)
    def energy_forces_device(self, offsets, rr, species, E, G, stream=None, sync=True):
        flags = ACE_INPUTS_ON_DEVICE | ACE_OUTPUTS_ON_DEVICE | (0 if sync else ACE_ASYNC)
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_energy_forces(self.h, E.numel(), _ptr(offsets), _ptr(rr), _ptr(species),
                                               _ptr(E), _ptr(G), flags, st))

    # error control of the compensated form ("fp32c")
    def set_energy_tolerance(self, tol: float):
        """Environments whose estimated energy error exceeds tol * max(|E|,
        rms E of the launch) are evaluated again in double-float (0: off)."""
        self._check(self.lib.ace_set_energy_tolerance(self.h, float(tol)))

    def energy_error_estimates(self, n: int | None = None):
        """(estimates of the last energy call's first n environments (None:
        only the count), environments re-evaluated since creation)."""
        refined = C.c_int64(0)
        est = None if n is None else np.zeros(n, dtype=np.float64)
        self._check(self.lib.ace_energy_error_estimates(self.h, 0 if n is None else n,
                                                        None if est is None else _ptr(est), C.byref(refined)))
        return est, int(refined.value)

    def autotune(self, offsets, rr, species, E, G, reps=3, stream=None):
        """Pick the fastest launch configuration on this device batch (torch
        tensors); returns region_kb + 1000 * (item schedule chosen)."""
        choice = C.c_int32(0)
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_autotune(self.h, E.numel(), _ptr(offsets), _ptr(rr), _ptr(species), _ptr(E),
                                          _ptr(G), reps, st, C.byref(choice)))
        return int(choice.value)

    # learned radial form (device tensors for the training entry points)
    def set_radial_mlp(self, params, K, Q, nspecies, tmax, H=64):
        p = np.ascontiguousarray(params, dtype=np.float32)
        d = RadialMLPDesc(1, K, Q, nspecies, H, float(tmax), _ptr(p), len(p))
        self._check(self.lib.ace_set_radial_mlp(self.h, C.byref(d)))

    def radial_mlp_params(self):
        """(device address, length) of the context's MLP parameters."""
        ptr, n = C.c_void_p(), C.c_int64()
        self._check(self.lib.ace_radial_mlp_params(self.h, C.byref(ptr), C.byref(n)))
        return int(ptr.value), int(n.value)

    def radial_mlp_get_params(self):
        _, n = self.radial_mlp_params()
        out = np.empty(n, dtype=np.float32)
        self._check(self.lib.ace_radial_mlp_get_params(self.h, _ptr(out), 0))
        return out

    def radial_mlp_forward(self, rr, species, R, stream=None):
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_radial_mlp_forward(self.h, rr.shape[0], _ptr(rr), _ptr(species), _ptr(R), st))

    def radial_mlp_infer(self, rr, species, R, stream=None):
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_radial_mlp_infer(self.h, rr.shape[0], _ptr(rr), _ptr(species), _ptr(R), st))

    def radial_mlp_backward(self, rr, species, gR, wj, gparams, stream=None):
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_radial_mlp_backward(self.h, rr.shape[0], _ptr(rr), _ptr(species), _ptr(gR),
                                                     _ptr(wj), _ptr(gparams), st))

    def energy_radial_adjoint(self, offsets, rr, species, E, G, GR, stream=None):
        st = None if stream is None else C.c_void_p(int(stream))
        self._check(self.lib.ace_energy_radial_adjoint(self.h, E.numel(), _ptr(offsets), _ptr(rr), _ptr(species),
                                                       _ptr(E), _ptr(G), _ptr(GR), st))

    def adam_step(self, w, g, m, v, lr, step, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        st = None if stream is None else C.c_void_p(int(stream))
        w_ptr = C.c_void_p(w) if isinstance(w, int) else _ptr(w)
        self._check(self.lib.ace_adam_step(g.numel(), w_ptr, _ptr(g), _ptr(m), _ptr(v), lr, beta1, beta2, eps,
                                           step, st))

    def sync(self):
        self._check(self.lib.ace_sync(self.h))
