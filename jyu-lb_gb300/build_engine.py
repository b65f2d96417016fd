"""Builds libjyulb_gb300.so in-tree for sm_103a (nvcc, no cmake).

Translation units compile in parallel into ``jyu-lb_gb300/_build`` and link
into ``jyu-lb_gb300/jyulb/libjyulb_gb300.so``.  The FP64 step and the set-up
kernels are compiled with ``-fmad=false`` so that their arithmetic is the
reference's operation for operation.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "jyulb", "libjyulb_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", CSRC, "-I", INCLUDE]
HOST_FLAGS = ["-x", "cu", "-Xcompiler", "-fopenmp", "-Xcompiler", "-ffp-contract=off"]
UNITS = {
    "lbm_fp64.cu": ["-fmad=false"],
    # the fast FP64 step: contracted on purpose
    "lbm_fp64fast.cu": [],
    # resident 128-thread blocks per SM.  The direct steps are latency-bound
    # on HBM: 8 blocks (<= 64 registers, 32 warps) keep more loads in flight
    # than 6 or 7, even where a few registers spill.  The persistent staged L
    # step keeps its loads in flight as bulk copies and runs fastest at 5
    # blocks for FP32 and 8 for FP16 (sweeps of 4..9 on the 256^3 cavity).
    # On the fluid-only layout (porous lattices) both steps are fastest at 7
    # (the P step holds its 18 neighbour indices in registers).
    "lbm_fp32.cu": ["-DJLB_MIN_BLOCKS=8", "-DJLB_MIN_BLOCKS_TMA=5", "-DJLB_MIN_BLOCKS_SPARSE=7"],
    "lbm_fp16.cu": ["-DJLB_MIN_BLOCKS=8", "-DJLB_MIN_BLOCKS_SPARSE=7"],
    "lbm_aux.cu": ["-fmad=false"],
    "lbm_noalloc.cu": [],
    "lbm_batch.cu": [],
    "lbm_adjoint.cu": [],
    "lbm_cxx.cu": ["-fmad=false"],
    # host arithmetic (relaxation rates, Ladd projections, the adjoint's chain
    # rule) must not be FMA-contracted either: gcc contracts by default on
    # aarch64
    "lbm_host.cpp": HOST_FLAGS,
    "lbm_batch_host.cpp": HOST_FLAGS,
    "lbm_adjoint_host.cpp": HOST_FLAGS,
}
HEADERS = ["lbm_common.h", "lbm_fp64.cuh", "lbm_solver.h", "lbm_step.cuh", "lbm_step_tma.cuh", "lbm_shifted.cuh", "lbm_aux.h", "lbm_batch.h", "lbm_adjoint.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    stamp = obj + ".flags"
    flags = " ".join(ARCH + COMMON + UNITS[os.path.basename(src)])
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        with open(stamp, "w") as fh:
            fh.write(flags)
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "jyulb_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(unit: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    if _stale(obj, src):
        cmd = [_nvcc()] + ARCH + COMMON + UNITS[unit] + ["-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
