"""Build libparphom_gpu.so (the C-ABI library) in-tree with nvcc for sm_103a,
and the native host driver parphom_gpu.x (C++, linked against it).

Translation units are compiled in parallel and linked with the CUDA runtime;
the results land in parphom_gb300/lib/.  No PyTorch is involved in either.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libparphom_gpu.so")
HOST = os.path.join(HERE, "host")
EXE = os.path.join(LIBDIR, "parphom_gpu.x")
HOST_SOURCES = ["h5min.cpp", "inputs.cpp", "parphom_gpu_main.cpp"]
SOURCES = ["pp_capi.cu", "pp_dynmat.cu", "pp_eigen.cu", "pp_noalloc.cu", "pp_dos.cu", "pp_tc.cu", "pp_errest.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "parphom_gpu.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    cc = nvcc()

    def one(src):
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_host(force: bool = False) -> str:
    """The host driver: g++, no contraction of a*b+c (the geometry matches
    the reference's evaluation order), rpath to the library's directory."""
    lib = build()
    srcs = [os.path.join(HOST, f) for f in HOST_SOURCES]
    deps = [lib, os.path.join(HERE, "..", "include", "parphom_gpu.h")] + srcs + \
        [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")]
    if not force and os.path.exists(EXE) and os.path.getmtime(EXE) >= max(os.path.getmtime(f) for f in deps):
        return EXE
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = EXE + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(HERE, "..", "include"), *srcs,
           "-o", tmp, "-L", LIBDIR, "-lparphom_gpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host driver build failed:\n{r.stderr}")
    os.replace(tmp, EXE)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_host(force="--force" in sys.argv))
