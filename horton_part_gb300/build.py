"""Build ``libhpgpu.so`` in-tree with nvcc for sm_103a (GB300).

    python -m horton_part_gb300.build [--force]

Each ``csrc/*.cu`` translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into a
shared library next to this file. Rebuilds unless the stamp beside the
library records the same sources, flags and machine architecture.
"""

from __future__ import annotations

import glob
import hashlib
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libhpgpu.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


STAMP = LIB + ".stamp"


def _fingerprint(extra_flags=()):
    """Hash of every source and header, the flags and the host machine: a
    library built elsewhere (another architecture, other sources) never
    matches and is rebuilt."""
    h = hashlib.sha256()
    deps = sorted(sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h")))
    for path in deps:
        h.update(os.path.basename(path).encode())
        with open(path, "rb") as f:
            h.update(f.read())
    h.update(" ".join([*ARCH, *NVCC_FLAGS, *extra_flags]).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _stale(extra_flags=()):
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return True
    with open(STAMP) as f:
        return f.read().strip() != _fingerprint(extra_flags)


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link; returns the library path."""
    if not force and not _stale(extra_flags):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout, res.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(sources()))) as pool:
        objs = list(pool.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_fingerprint(extra_flags) + "\n")
    return LIB


if __name__ == "__main__":
    args = sys.argv[1:]
    extra = []
    if "--ptxas-v" in args:
        extra = ["-Xptxas", "-v"]
    print(build(force="--force" in args or bool(extra), verbose=True, extra_flags=extra))
