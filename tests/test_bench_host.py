"""CPU checks of bench.py's host side: the reference arm's JSON line (the
oracle timed on the host cores) and the CPU-baseline sampler."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT, check=True).stdout
    d = json.loads(out.strip().splitlines()[-1])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1


def test_cpu_baseline_sampler():
    import bench
    from ace_gb300.configs import random_batch
    from ace_gb300.spec import random_coefficients, symmetric_basis
    spec = symmetric_basis(3, 6, maxL=6)
    c = random_coefficients(spec, seed=0)
    b = random_batch(300, 8, 16, seed=0)
    r = bench.cpu_baseline(spec, c, b, threads=2, target_s=0.05)
    assert r["value"] > 0 and r["cores"] == 2 and r["kind"] == "port"
    assert r["single_thread"]["value"] > 0


def test_flops_per_env_counts_the_reference_terms():
    import bench
    from ace_gb300.spec import symmetric_basis
    spec = symmetric_basis(3, 6, maxL=6)
    f0, f1 = bench.flops_per_env(spec, 0), bench.flops_per_env(spec, 1)
    nby = spec.info["nAA_by_order"]
    per_env = sum(n * (6 * (k - 1) + 2) + n * (18 * max(k - 2, 0) + 6 + 4 * k) for k, n in nby.items() if k > 0)
    assert f0 == per_env
    assert np.isclose(bench.flops_per_env(spec, 30) - f0, 30 * (f1 - f0))


def test_reference_arm_under_two_ranks_prints_one_line():
    # launched like the multi-GPU bench (torchrun, one rank per GPU): rank 0
    # alone runs the CPU reference and prints; the other rank exits 0
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port),
                        os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
