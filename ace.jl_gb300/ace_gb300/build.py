"""Builds libace_b200.so in-tree with nvcc for sm_103a (GB300)."""
from __future__ import annotations

import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                 # .../ace.jl_gb300
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
LIB = os.path.join(ROOT, "libace_b200.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183, "arm64": 183}


def built_for_this_host(path: str) -> bool:
    """True when the shared object at `path` is an ELF file for this host's
    CPU architecture (a library compiled on another machine is rebuilt)."""
    import platform
    import struct
    want = _ELF_MACHINE.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    endian = "<" if head[5] == 1 else ">"
    machine = struct.unpack(endian + "H", head[18:20])[0]
    return want is None or machine == want


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    """Compile every .cu under csrc/ into libace_b200.so (skipped when up to
    date and built for this host's architecture)."""
    if not force and os.path.exists(LIB) and built_for_this_host(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps()):
            return LIB
    objs = []
    procs = []
    os.makedirs(os.path.join(ROOT, "_build"), exist_ok=True)
    for src in sources():
        obj = os.path.join(ROOT, "_build", os.path.basename(src) + ".o")
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", INCLUDE, "-c", src, "-o", obj, *extra]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src))
        objs.append(obj)
    for p, src in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{out.decode()}")
        if verbose and out:
            print(out.decode())
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode())
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv, extra=(["-Xptxas", "-v"] if "-v" in sys.argv else [])))
