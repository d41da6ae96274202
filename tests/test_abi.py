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
