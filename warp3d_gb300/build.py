"""Builds the CUDA engine warp3d_gb300/_build/libw3g.so for sm_103a.

Plain nvcc, one process per translation unit, then one shared-library
link: no torch, no cmake. Usable as ``python -m warp3d_gb300.build``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libw3g.so")
SOURCES = ["w3g_api.cu", "w3g_tangent.cu", "w3g_tangent_tc.cu", "w3g_tangent_tcg.cu", "w3g_tangent_tc20.cu", "w3g_recover.cu", "w3g_mm10.cu",
           "w3g_solve.cu",
           "w3g_peak.cu", "w3g_noalloc.cu", "w3g_restart.cu",
           "w3g_tangent_full.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code without multiply-add contraction (aarch64 g++ contracts by
# default): the host-built tables follow the same operation order as the
# oracle
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"]
# the mm10 local Newton solve evaluates residuals and Jacobians in the
# reference's operation order (no fused multiply-add)
EXTRA_FLAGS = {"w3g_mm10.cu": ["-fmad=false"]}


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *EXTRA_FLAGS.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    """Compiles every CUDA source and links libw3g.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "w3g.h"))
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in deps)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv))
