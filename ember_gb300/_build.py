"""In-tree build of libember_gpu.so for sm_103a (GB300) with nvcc.

Each translation unit in ``csrc/`` is compiled in parallel into ``_build/``
and linked into ``ember_gb300/libember_gpu.so``. Nothing is installed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libember_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Translation units whose arithmetic must match the CPU oracle operation by
# operation: no automatic multiply-add contraction (explicit fma() only).
FILE_FLAGS = {"source.cu": ["--fmad=false"], "bdf.cu": ["--fmad=false"], "split.cu": ["--fmad=false"],
              "qss_adjoint.cu": ["--fmad=false"],
              "transport.cu": ["--fmad=false"], "convection.cu": ["--fmad=false"],
              # host code: the same rounding on x86-64 and aarch64 (no contraction into FMA)
              "grid.cpp": ["-Xcompiler", "-ffp-contract=off"]}
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libember_gpu.so")


def _deps() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(CSRC, "*.cpp")) +
                  glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile every CUDA source for sm_103a and link the shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = NVCC_FLAGS + ARCH + (extra_flags or [])
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        cmd = [cc, "-c", src, "-o", obj] + flags + FILE_FLAGS.get(os.path.basename(src), [])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    workers = max(1, min(len(sources), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(compile_one, sources))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
