"""Build step for the GB300 library (in-tree, no cmake).

Compiles the CUDA kernels for sm_103a and the C++ host into
``hamstr_oop_gb300/lib/libhamstr_gb300.so`` and the ``bin/hamstr_gb300``
executable.  Translation units compile in parallel; objects go to
``hamstr_oop_gb300/_build``.  Every unit uses strict IEEE arithmetic
(no FMA contraction on host or device) because the path is bit-identical
to the reference.
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
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libhamstr_gb300.so")
EXE = os.path.join(BINDIR, "hamstr_gb300")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "--expt-relaxed-constexpr",
                  "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]
CXXFLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA_HOME, "include")]

CU_SOURCES = ["rhs.cu", "adi.cu", "api.cu", "trisolve.cu", "mixed.cu", "forces.cu", "mlp_gemm.cu", "mlp_api.cu", "mlp_net.cu", "checks.cu",
              "pointwise.cu", "strand5.cu"]
CXX_SOURCES = ["plan.cpp", os.path.join("host", "hamstr_host.cpp"), os.path.join("host", "hamstr_dropin.cpp")]


def _newer(src_list, dst):
    if not os.path.exists(dst):
        return True
    t = os.path.getmtime(dst)
    return any(os.path.getmtime(s) > t for s in src_list)


def _headers():
    hs = []
    for d, _, fs in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in fs if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "hamstr_gpu.h"))
    return hs


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile everything that is out of date; returns the library path."""
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at " + NVCC)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _newer([src] + hdrs, obj):
            jobs.append([NVCC] + NVFLAGS + ["-c", src, "-o", obj])
    for s in CXX_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _newer([src] + hdrs, obj):
            jobs.append(["g++"] + CXXFLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _newer(objs, LIB):
        _run([NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs + ["-lcudart"])
    main_src = os.path.join(CSRC, "host", "main.cpp")
    if force or _newer([main_src, LIB], EXE):
        _run(["g++"] + CXXFLAGS + [main_src, "-o", EXE, "-L" + LIBDIR, "-lhamstr_gb300",
                                   "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


def clean() -> None:
    for d in (BUILD,):
        shutil.rmtree(d, ignore_errors=True)
    for f in (LIB, EXE):
        if os.path.exists(f):
            os.remove(f)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
