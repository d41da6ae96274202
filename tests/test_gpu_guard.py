"""Error control of the compensated form (ace_set_energy_tolerance,
ace_energy_error_estimates): each energy call of an ACE_PREC_FP32_COMP
context estimates every environment's energy rounding error, and with a
tolerance set evaluates the environments whose estimate is over it again in
double-float, on the device, within the same call.

Checked against the FP64 CPU oracle, on an order-4 and an order-5 basis:
* the estimate covers the measured error of every environment;
* with a tolerance, every environment's error is within it, and the
  environments re-evaluated are exactly those whose estimate was over it;
* a tolerance below any estimate re-evaluates every environment: the
  energies are then the double-float form's;
* energies-only calls run the double-float energy kernel (no estimate
  needed); the host-buffer pipeline (chunked launches) and a CUDA-graph
  replay keep the tolerance;
* the calls are refused for the other precision modes and bad tolerances."""
import numpy as np
import pytest

from ace_gb300.configs import random_batch
from ace_gb300.spec import random_coefficients, symmetric_basis

pytestmark = pytest.mark.gpu

ACE_ERR_INVALID = 1
ACE_ERR_UNSUPPORTED = 5

SPECS = {"ord4": dict(maxorder=4, maxdeg=12, maxL=12), "ord5": dict(maxorder=5, maxdeg=10, maxL=10)}
_cache = {}


def case(name):
    if name not in _cache:
        spec = symmetric_basis(**SPECS[name])
        c = random_coefficients(spec, seed=11)
        b = random_batch(300 if name == "ord4" else 120, 20, 60, seed=12)
        _cache[name] = (spec, c, b)
    return _cache[name]


def scale(E):
    return np.maximum(np.abs(E), np.sqrt(np.mean(E ** 2)))


@pytest.fixture(scope="module")
def L():
    from ace_gb300 import lib
    from ace_gb300.build import build
    build()
    return lib


@pytest.fixture(scope="module")
def oracle_E(oracle_mod):
    out = {}
    for name in SPECS:
        spec, c, b = case(name)
        out[name] = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, b.rr)
    return out


@pytest.mark.parametrize("name", ["ord4", "ord5"])
def test_estimate_covers_error(L, oracle_E, name):
    spec, c, b = case(name)
    Eref, Gref = oracle_E[name]
    ctx = L.Context(spec, "fp32c")
    ctx.set_params(c)
    ctx.set_energy_tolerance(0.0)
    _, r0 = ctx.energy_error_estimates()
    E, G = ctx.energy_forces(b.offsets, b.rr)
    est, r1 = ctx.energy_error_estimates(b.nenv)
    assert r1 == r0                                   # tolerance off: nothing re-evaluated
    assert np.all(est > 0) and np.all(np.isfinite(est))
    err = np.abs(E - Eref)
    assert np.all(err <= est), float(np.max(err / est))
    assert np.max(np.abs(G - Gref)) <= 1e-5 * np.max(np.abs(Gref))
    ctx.close()


@pytest.mark.parametrize("name", ["ord4", "ord5"])
def test_tolerance_holds(L, oracle_E, name):
    spec, c, b = case(name)
    Eref, Gref = oracle_E[name]
    ctx = L.Context(spec, "fp32c")
    ctx.set_params(c)
    ctx.set_energy_tolerance(0.0)
    Ec, _ = ctx.energy_forces(b.offsets, b.rr)
    est, _ = ctx.energy_error_estimates(b.nenv)
    tol = 1e-7
    expect = int(np.sum(est > tol * scale(Ec)))
    assert 0 < expect < b.nenv                        # a tolerance that splits the batch
    ctx.set_energy_tolerance(tol)
    _, r0 = ctx.energy_error_estimates()
    E, G = ctx.energy_forces(b.offsets, b.rr)
    _, r1 = ctx.energy_error_estimates()
    assert abs((r1 - r0) - expect) <= 1               # (rms summed in another order)
    assert np.all(np.abs(E - Eref) <= 1.01 * tol * scale(Eref))
    assert np.max(np.abs(G - Gref)) <= 1e-5 * np.max(np.abs(Gref))
    # energies only: the double-float energy kernel, nothing re-evaluated
    _, r0 = ctx.energy_error_estimates()
    E2 = ctx.energy_forces(b.offsets, b.rr, forces=False)
    _, r1 = ctx.energy_error_estimates()
    assert r1 == r0
    assert np.max(np.abs(E2 - Eref) / scale(Eref)) <= 1e-11
    ctx.close()


@pytest.mark.parametrize("name", ["ord4", "ord5"])
def test_item_runs(L, oracle_E, name, monkeypatch):
    """The same on the item runs (their estimate groups by item)."""
    spec, c, b = case(name)
    Eref, Gref = oracle_E[name]
    monkeypatch.setenv("ACE_B200_KERNEL", "items")   # read at context creation
    ctx = L.Context(spec, "fp32c")
    monkeypatch.delenv("ACE_B200_KERNEL")
    ctx.set_params(c)
    ctx.set_energy_tolerance(0.0)
    E, G = ctx.energy_forces(b.offsets, b.rr)
    est, _ = ctx.energy_error_estimates(b.nenv)
    assert np.all(np.abs(E - Eref) <= est)
    tol = 1e-7
    ctx.set_energy_tolerance(tol)
    E, G = ctx.energy_forces(b.offsets, b.rr)
    assert np.all(np.abs(E - Eref) <= 1.01 * tol * scale(Eref))
    assert np.max(np.abs(G - Gref)) <= 1e-5 * np.max(np.abs(Gref))
    ctx.close()


def test_all_reevaluated_is_double_float(L, oracle_E):
    spec, c, b = case("ord5")
    Eref, Gref = oracle_E["ord5"]
    ctx = L.Context(spec, "fp32c")
    ctx.set_params(c)
    ctx.set_energy_tolerance(1e-15)                   # below every estimate
    _, r0 = ctx.energy_error_estimates()
    E, G = ctx.energy_forces(b.offsets, b.rr)
    _, r1 = ctx.energy_error_estimates()
    assert r1 - r0 == b.nenv
    x2 = L.Context(spec, "fp32x2")
    x2.set_params(c)
    Ex, Gx = x2.energy_forces(b.offsets, b.rr)
    assert np.max(np.abs(E - Ex) / scale(Eref)) <= 1e-12
    assert np.max(np.abs(E - Eref) / scale(Eref)) <= 1e-11
    assert np.max(np.abs(G - Gref)) <= 1e-5 * np.max(np.abs(Gref))
    x2.close()
    ctx.close()


def test_pipeline_chunks(L):
    """Host buffers, 10,000 environments: the call runs as chunked launches;
    each chunk's estimates land at its offset and the tolerance holds."""
    spec = symmetric_basis(**SPECS["ord4"])
    c = random_coefficients(spec, seed=11)
    b = random_batch(10_000, 20, 60, seed=13)
    ref = L.Context(spec, "fp64")
    ref.set_params(c)
    Eref, _ = ref.energy_forces(b.offsets, b.rr)
    ref.close()
    ctx = L.Context(spec, "fp32c")
    ctx.set_params(c)
    tol = 2e-7
    ctx.set_energy_tolerance(tol)
    E, _ = ctx.energy_forces(b.offsets, b.rr)
    est, _ = ctx.energy_error_estimates(b.nenv)
    assert np.all(est > 0)                            # every chunk wrote its estimates
    assert np.all(np.abs(E - Eref) <= 1.05 * tol * scale(Eref))
    ctx.close()


def test_graph_replay_keeps_tolerance(L, oracle_mod):
    torch = pytest.importorskip("torch")
    spec, c, b = case("ord4")
    ctx = L.Context(spec, "fp32c")
    ctx.set_params(c)
    tol = 1e-7
    ctx.set_energy_tolerance(tol)
    off = torch.from_numpy(b.offsets).cuda()
    rr = torch.from_numpy(b.rr).cuda()
    E = torch.empty(b.nenv, dtype=torch.float64, device="cuda")
    G = torch.empty_like(rr)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.energy_forces_device(off, rr, None, E, G, stream=s.cuda_stream, sync=False)  # warm-up
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ctx.energy_forces_device(off, rr, None, E, G, stream=s.cuda_stream, sync=False)
    b2 = random_batch(b.nenv, 20, 60, seed=14)
    rr2 = np.resize(b2.rr, b.rr.shape)                # same neighbour counts, new positions
    rr.copy_(torch.from_numpy(np.ascontiguousarray(rr2)))
    g.replay()
    torch.cuda.synchronize()
    ctx.sync()
    Eref, _ = oracle_mod.Oracle(spec, c).energy_forces(b.offsets, rr2)
    assert np.all(np.abs(E.cpu().numpy() - Eref) <= 1.01 * tol * scale(Eref))
    ctx.close()


def test_refused(L):
    from ace_gb300.lib import AceError
    spec, c, b = case("ord4")
    ctx = L.Context(spec, "fp64")
    with pytest.raises(AceError) as ei:
        ctx.set_energy_tolerance(1e-6)
    assert ei.value.code == ACE_ERR_UNSUPPORTED
    ctx.close()
    ctx = L.Context(spec, "fp32c")
    ctx.set_params(c)
    for bad in (-1.0, float("nan"), float("inf")):
        with pytest.raises(AceError) as ei:
            ctx.set_energy_tolerance(bad)
        assert ei.value.code == ACE_ERR_INVALID
    ctx.energy_forces(b.offsets, b.rr)
    with pytest.raises(AceError) as ei:
        ctx.energy_error_estimates(b.nenv + 1)
    assert ei.value.code == ACE_ERR_INVALID
    ctx.close()
