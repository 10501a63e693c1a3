"""Build recipe for the in-tree shared library ``libprc_d2z.so`` and the
``delta2zreion`` executable.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), the host C++ with g++
(``-ffp-contract=off`` so float expressions round per operation, as the
tables require), all in parallel; objects go to ``pr-calc_gb300/_build``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                      # pr-calc_gb300/
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
REPO = os.path.dirname(ROOT)
INCLUDE = os.path.join(REPO, "include")
LIB = os.path.join(PKG_DIR, "libprc_d2z.so")
EXE = os.path.join(ROOT, "bin", "delta2zreion")

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE]

CU_LIB = ["d2z_capi.cu", "inst_a.cu", "inst_b.cu", "inst_c.cu", "inst_d.cu", "inst_e.cu", "inst_f.cu",
          "d2z_noalloc.cu"]
CPP_LIB = ["errors.cpp", "cosmo.cpp", "history.cpp"]
CPP_EXE = ["main_d2z.cpp"]


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
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "prc_d2z.h"))
    return hs


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (incrementally) and return the path of libprc_d2z.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    hdrs = _headers()
    steps = []
    objs = []
    for f in CU_LIB:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    for f in CPP_LIB + CPP_EXE:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")
        if f in CPP_LIB:
            objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append([CXX] + CXXFLAGS + ["-c", src, "-o", obj])
    jobs = jobs or max(2, min(len(steps) or 1, os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for out in ex.map(_run, steps):
            if verbose and out.strip():
                print(out, file=sys.stderr)
    if _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    exe_obj = os.path.join(BUILD, "main_d2z.cpp.o")
    if _stale(EXE, [exe_obj, LIB]):
        _run([CXX, "-o", EXE, exe_obj, "-L", PKG_DIR, "-lprc_d2z",
              "-Wl,-rpath,$ORIGIN/../prc_d2z", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
