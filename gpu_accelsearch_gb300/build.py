"""Build libaccelsearch.so in-tree (nvcc, sm_103a only).

    python -m gpu_accelsearch_gb300.build          # or __graft_entry__.build()

Each CUDA translation unit is compiled in parallel into _build/, then linked
with cuFFT into gpu_accelsearch_gb300/libaccelsearch.so.  bank.cu is built
with -fmad=false so that its double-precision template arithmetic rounds
operation by operation like the reference's host code; compat.cu and
dedisperse.cu keep the host compiler from contracting multiply-adds, so
that their host arithmetic gives the same numbers on every host.
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libaccelsearch.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "bank.cu", "search.cu", "search_plane_lo.cu", "search_plane_hi.cu",
           "search_fund_lo.cu", "search_fund_hi.cu", "tune.cu", "whiten.cu", "compat.cu",
           "server.cu", "sift.cu", "optimize.cu", "dedisperse.cu",
           "filterbank.cu", "compat_cxx.cu", "search_step.cu", "rfft.cu", "search_mixed5.cu",
           "search_mixed6.cu", "search_mixed7.cu", "search_mixed_prep.cu"]
EXTRA = {"bank.cu": ["-fmad=false"], "compat.cu": ["-Xcompiler", "-ffp-contract=off"],
         "dedisperse.cu": ["-Xcompiler", "-ffp-contract=off"]}
HEADERS = ["accel_common.cuh", "accel_internal.h", "context.h", "fft_smem.cuh", "search_kernels.cuh",
           "step_kernel.cuh", "fft_mixed.cuh", "mixed_kernels.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(ROOT, "include", h) for h in ("accelsearch.h", "bpd_compat.h", "bpd_compat_cxx.h")] + [__file__]
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc()] + _flags() + EXTRA.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
