"""The boundary's error behaviour, on the CPU: ace_ctx_create validates the
spec bundle and its arguments before any device work and reports a status
code plus ace_last_error_string(NULL), never an exception or a crash.
These calls go through the real library (libace_b200.so)."""
import ctypes as C

import numpy as np
import pytest

from ace_gb300.spec import symmetric_basis

OK, INVALID, CUDA, UNSUPPORTED = 0, 1, 2, 5


@pytest.fixture(scope="module")
def lib():
    from ace_gb300 import lib as L
    from ace_gb300.build import build
    try:
        build()
    except RuntimeError as e:  # no nvcc on this host
        pytest.skip(str(e))
    return L


@pytest.fixture
def spec():
    # per test: the bundle may share the spec's arrays, which the cases edit
    return symmetric_basis(3, 6, maxL=6)


def create(L, bundle, prec=4, device=0):
    lib = L.load()
    out = C.c_void_p(None)
    rc = lib.ace_ctx_create(None if bundle is None else C.byref(bundle), prec, device, C.byref(out))
    msg = lib.ace_last_error_string(None)
    if rc == OK:  # only reachable with a GPU; not expected by these cases
        lib.ace_ctx_destroy(out)
    return rc, (msg or b"").decode(), out.value


def _mutated(L, spec, edit):
    b, keep = L.make_bundle(spec)
    edit(b, keep)
    return b, keep


CASES = [
    ("version", lambda b, k: setattr(b, "version", 99), INVALID, "version"),
    ("nR", lambda b, k: setattr(b, "nR", 0), UNSUPPORTED, "nR out of range"),
    ("nA", lambda b, k: setattr(b, "nA", 0), UNSUPPORTED, "nA out of range"),
    ("a_l", lambda b, k: k["a_l"].__setitem__(0, 25), UNSUPPORTED, "a_l out of range"),
    ("a_m", lambda b, k: k["a_m"].__setitem__(0, 3), INVALID, "|a_m| > a_l"),
    ("a_n", lambda b, k: k["a_n"].__setitem__(0, 99), INVALID, "a_n out of range"),
    ("nspecies", lambda b, k: setattr(b, "nspecies", 0), UNSUPPORTED, "nspecies out of range"),
    ("maxord", lambda b, k: setattr(b, "maxord", 9), UNSUPPORTED, "maxord"),
    ("orders", lambda b, k: k["orders"].__setitem__(5, 7), INVALID, "orders out of range"),
    ("iAA2iA", lambda b, k: k["iAA2iA"].__setitem__((5, 0), 10 ** 6), INVALID, "iAA2iA entry out of range"),
    ("U_indices", lambda b, k: k["U_indices"].__setitem__(0, 10 ** 8), INVALID, "U index out of range"),
    ("U_indptr", lambda b, k: k["U_indptr"].__setitem__(1, -1), INVALID, "U_indptr"),
]


@pytest.mark.parametrize("name,edit,code,text", CASES, ids=[c[0] for c in CASES])
def test_invalid_bundle_rejected_before_device_work(lib, spec, name, edit, code, text):
    b, keep = _mutated(lib, spec, edit)
    rc, msg, out = create(lib, b)
    assert rc == code and text in msg and out is None, (rc, msg)


def test_null_arguments(lib, spec):
    rc, msg, out = create(lib, None)
    assert rc == INVALID and "NULL" in msg and out is None
    b, keep = lib.make_bundle(spec)
    rc = lib.load().ace_ctx_create(C.byref(b), 4, 0, None)
    assert rc == INVALID


def test_unknown_precision_and_device(lib, spec):
    b, keep = lib.make_bundle(spec)
    rc, msg, out = create(lib, b, prec=7)
    assert rc == UNSUPPORTED and "precision" in msg and out is None
    # a device index that cannot exist: a CUDA-status error, with or without a GPU
    rc, msg, out = create(lib, b, device=-1)
    assert rc == CUDA and "device" in msg and out is None


def test_valid_bundle_passes_validation(lib, spec):
    # the untouched bundle fails only at device selection on a host without
    # a GPU, never in validation
    b, keep = lib.make_bundle(spec)
    rc, msg, out = create(lib, b, device=10 ** 6)
    assert rc == CUDA and "device" in msg
    assert np.all(keep["orders"] >= 0)


def test_every_entry_point_rejects_a_null_context(lib):
    L = lib.load()
    n = None
    calls = {
        "ace_set_params": (n, n, 0), "ace_set_ctilde": (n, n, 0), "ace_set_params_multi": (n, n, 0, 1),
        "ace_set_ctilde_complex": (n, n, 0, 1),
        "ace_energy_forces": (n, 1, n, n, n, n, n, 0, n), "ace_energy": (n, 1, n, n, n, n, 0, n),
        "ace_energy_forces_multi": (n, 1, n, n, n, n, n, 0, n), "ace_basis": (n, 1, n, n, n, n, n, 0, n),
        "ace_basis_noalloc": (n, 1, n, n, n, n, n), "ace_adjoint_eval_d": (n, 1, n, n, n, n, n, 0, n),
        "ace_autotune": (n, 1, n, n, n, n, n, 1, n, n), "ace_sync": (n,), "ace_get_spec_sizes": (n, n),
        "ace_set_radial_mlp": (n, n), "ace_radial_mlp_params": (n, n, n), "ace_radial_mlp_get_params": (n, n, 0),
        "ace_radial_mlp_forward": (n, 1, n, n, n, n), "ace_radial_mlp_infer": (n, 1, n, n, n, n),
        "ace_radial_mlp_backward": (n, 1, n, n, n, n, n, n),
        "ace_energy_radial_adjoint": (n, 1, n, n, n, n, n, n, n),
        "ace_set_energy_tolerance": (n, 1e-6), "ace_energy_error_estimates": (n, 0, n, n),
    }
    for name, args in calls.items():
        assert getattr(L, name)(*args) == INVALID, name
    assert L.ace_ctx_destroy(None) == OK
    assert L.ace_launch_count(None) == 0
    assert L.ace_last_error_string(None) is not None
    # the context-free Adam step: argument checks before any launch
    assert L.ace_adam_step(10, n, n, n, n, 1e-3, 0.9, 0.999, 1e-8, 1, n) == INVALID
    assert L.ace_adam_step(0, n, n, n, n, 1e-3, 0.9, 0.999, 1e-8, 1, n) == OK
