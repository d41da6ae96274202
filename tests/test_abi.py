"""The C-ABI library loads and exports every entry point include/ace_b200.h
declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "ace_b200.h")).read()
    return sorted(set(re.findall(r"\b(ace_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_boundary():
    syms = declared_symbols()
    for s in ("ace_ctx_create", "ace_ctx_destroy", "ace_set_params", "ace_energy_forces",
              "ace_energy", "ace_basis", "ace_sync", "ace_get_spec_sizes", "ace_last_error_string"):
        assert s in syms


def test_library_exports_declared_symbols():
    from ace_gb300.build import build
    try:
        path = build()
    except RuntimeError as e:  # no nvcc on this host
        pytest.skip(str(e))
    lib = ctypes.CDLL(path)
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_python_binding_lists_exports():
    from ace_gb300 import lib
    assert set(lib.EXPORTED) <= set(declared_symbols())


def test_header_compiles_as_c99(tmp_path):
    """include/ace_b200.h is plain C: a C99 consumer that names every entry
    point compiles with -Wall -Werror (the library is not linked or run)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    obj = str(tmp_path / "c_consumer.o")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-c",
                        "-I", os.path.join(root, "include"), os.path.join(root, "tests", "host", "c_consumer.c"),
                        "-o", obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_energy_force_kernels_do_not_spill(tmp_path):
    """The per-type register bounds of the energy/force kernel (ef_min_blocks,
    comp_min_blocks) leave the item-run and task-schedule instantiations of
    orders 2-5 without local-memory spills (ptxas resource report; the code
    itself is not read)."""
    import re
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    err = ""
    for name in ("ace_launch.cu", "ace_launch_comp.cu", "ace_launch_tasks.cu"):
        src = os.path.join(ROOT, "ace.jl_gb300", "csrc", name)
        r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xptxas", "-v",
                            "-I", os.path.join(ROOT, "include"), "-c", src, "-o", str(tmp_path / "l.o")],
                           capture_output=True, text=True, timeout=900)
        assert r.returncode == 0, r.stderr[-2000:]
        err += r.stderr
    cur, report = None, {}
    for line in err.splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line) or re.search(r"Function properties for (\S+)", line)
        if m:
            cur = m.group(1)
        elif cur and "spill stores" in line:
            report[cur] = int(re.search(r"(\d+) bytes spill stores", line).group(1))
    names = list(report)
    dem = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True).stdout.splitlines()
    checked = 0
    for mangled, d in zip(names, dem):
        m = re.search(r"ef_kernel<(.+), (\d), 128, true, true, false, (false|true), (false|true), (\d+)>", d)
        if m and 2 <= int(m.group(2)) <= 5:
            assert report[mangled] == 0, d
            checked += 1
    # {float, double-float, double, compensated} x (item runs: orders 2..5,
    # task schedule: orders 3..5 at the default and the high-occupancy bound)
    assert checked == 40
