"""Builds the sm_103a shared library of the solver core in-tree.

One nvcc process per translation unit (they compile in parallel), then one link step into
fluidx3d_gb300/_lib/libfluidx3d_gb300.so. Everything is compiled for sm_103a only, without
floating-point contraction (-fmad=false for device code, -ffp-contract=off for host code): every
fused multiply-add in the kernels is written out (fmaf / packed fma), so results do not depend on
the compiler's fusion choices. (ptxas still fuses a packed FP32x2 multiply whose only use is a
packed add, even with -fmad=false and explicit .rn modifiers; the kernels' arithmetic is written
without that pattern.)
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libfluidx3d_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-fmad=false",
              "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fluidx3d_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.isfile(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    if _stale(obj, [src, os.path.abspath(__file__)] + headers()):
        tmp = obj + f".{os.getpid()}.tmp"
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}\n{r.stdout}")
        os.replace(tmp, obj)
    return obj


def build(verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    """Compile (incrementally) and link the library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    srcs = sources()
    with ThreadPoolExecutor(jobs or min(len(srcs), os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if _stale(LIB_PATH, objs):
        tmp = LIB_PATH + f".{os.getpid()}.tmp"
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}\n{r.stdout}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build())
