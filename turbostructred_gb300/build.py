"""Builds the CUDA extension in-tree: turbostructred_gb300/libtsfvm.so.

Every translation unit is compiled for sm_103a only, in parallel, with nvcc.
ts_plain.cu (the bit-for-bit FP64 path) is compiled with --fmad=false so no
multiply-add contraction changes its rounding; the other units keep FMA.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtsfvm.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code never contracts a*b+c into an FMA (g++ does by default on
# aarch64): the grid accumulation must round exactly like the reference.
COMMON = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + INCLUDE, "-I" + CSRC]

UNITS = {
    "ts_plain.cu": ["--fmad=false"],
    # FP32 flux path: flush-to-zero and approximate FP32 division/sqrt; FP64
    # arithmetic is unaffected by these flags.
    "ts_mixed.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    "ts_mix3d.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    "ts_capi.cu": [],
    "ts_batch.cu": [],
    "ts_host.cpp": [],
    "ts_server.cpp": [],
    "ts_io.cpp": [],
}


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    if not _stale(obj, [src] + _headers() + [__file__]):
        return obj
    cmd = [NVCC] + ARCH + COMMON + UNITS[unit] + ["-c", src, "-o", obj]
    if unit.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    if _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-Xcompiler", "-fPIC", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
