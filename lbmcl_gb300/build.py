"""Build recipe of the native parts (nvcc / g++, no cmake, no torch extension).

    python -m lbmcl_gb300.build          # library + lbmcl host binary

Outputs (in-tree, git-ignored):
    lbmcl_gb300/liblbm_gb300.so   the C-ABI library (include/lbm.h), sm_103a
    lbmcl_gb300/bin/lbmcl         the C++ host program (reference CLI)

Translation units are compiled in parallel; one -gencode (sm_103a) only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblbm_gb300.so")
BIN = os.path.join(PKG, "bin", "lbmcl")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + INCLUDE, "-I" + CSRC]
CU_SOURCES = ["lbm_capi.cu", "lbm_kernels_f32.cu", "lbm_kernels_f64.cu", "lbm_kernels_f16.cu",
              "lbm_kernels_bf16.cu", "lbm_noalloc.cu", "lbm_adjoint_host.cu", "lbm_adjoint_f64.cu"]
HOST_SOURCES = ["host/main.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def build_library(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs) or ptxas_info:
            flags = NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else [])
            jobs.append([nv] + flags + ["-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose or ptxas_info:
            for o in outs:
                sys.stdout.write(o)
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


def build_host(verbose: bool = False) -> str:
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in HOST_SOURCES]
    host_hdrs = [os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host"))]
    if _stale(BIN, srcs + host_hdrs + [LIB, os.path.join(INCLUDE, "lbm.h")]):
        cxx = shutil.which("g++") or "g++"
        tmp = BIN + ".tmp"
        _run([cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-ffp-contract=off", "-I" + INCLUDE,
              "-I" + os.path.join(CSRC, "host"), "-o", tmp] + srcs +
             ["-L" + PKG, "-llbm_gb300", "-Wl,-rpath,$ORIGIN/.."])
        os.replace(tmp, BIN)
    return BIN


def build_all(verbose: bool = False) -> None:
    build_library(verbose)
    if os.path.exists(os.path.join(CSRC, "host", "main.cpp")):
        build_host(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    if "--ptxas" in sys.argv:
        build_library(ptxas_info=True)
    print(LIB)
