"""Build recipe of libstokes_gb300.so (CUDA for sm_103a + host C).

    python -m libstokes_gb300.build

Compiles every translation unit in csrc/ in parallel (nvcc for .cu, gcc for
.c) and links them into libstokes_gb300/_lib/libstokes_gb300.so, a plain
C-ABI shared library (no torch or Python symbols).  The output stays in the
source tree and is git-ignored.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libstokes_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-Wall", "--expt-relaxed-constexpr",
                     "-I", INCLUDE, "-I", CSRC]
# -ffp-contract=off: the host set-up gives the same bits on x86 and Arm
CC_FLAGS = ["-O2", "-fPIC", "-std=c11", "-Wall", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: libstokes_gb300 needs the CUDA toolkit")
    return cand


def _sources():
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".c"):
            yield os.path.join(CSRC, f)


def _deps(src: str):
    # every header of csrc/ and include/ is a dependency of every source
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return [src] + hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    base = os.path.basename(src)
    obj = os.path.join(OBJ_DIR, base + ".o")
    if not _stale(obj, _deps(src)):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["gcc"] + CC_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {base}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (incrementally) and link libstokes_gb300.so; return its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = list(_sources())
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
