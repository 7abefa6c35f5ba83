"""Compile the CUDA C-ABI library libwrs_gb300.so for sm_103a (in-tree).

Each translation unit is compiled in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -Xcompiler -fPIC
and linked into merian-wrs_gb300/libwrs_gb300.so.  Objects go to merian-wrs_gb300/_build/.
Rebuilds only what changed (by mtime against sources and headers).  The benchmark's C++
per-call driver (percall_driver.cpp, host code over include/wrs.hpp) is linked against it as
merian-wrs_gb300/libwrs_percall.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libwrs_gb300.so")
DRIVER_SRC = os.path.join(PKG, "percall_driver.cpp")
DRIVER_LIB = os.path.join(PKG, "libwrs_percall.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwrs_gb300.so")


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(nvcc: str, src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    if _stale(obj, [src] + _headers()):
        cmd = [nvcc, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    """Build (if needed) and return the path of libwrs_gb300.so."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs))
    if _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if _stale(DRIVER_LIB, [DRIVER_SRC, LIB] + _headers()):
        cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I",
               os.path.join(ROOT, "include"), DRIVER_SRC, "-o", DRIVER_LIB, "-L", PKG,
               "-lwrs_gb300", "-lcudart", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"per-call driver build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


def ptxas_report() -> str:
    """Registers / spills / shared memory of every kernel (-Xptxas -v)."""
    nvcc = _nvcc()
    out = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        r = subprocess.run([nvcc, *ARCH, *FLAGS, "-Xptxas", "-v", "-c", src, "-o", os.devnull],
                           capture_output=True, text=True)
        out.append(r.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "ptxas":
        print(ptxas_report())
    else:
        build(verbose=True)
