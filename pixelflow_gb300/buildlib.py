"""Build libpixelflow_gb300.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each .cu file under csrc/ is compiled in parallel to an object file, then the
objects are linked into pixelflow_gb300/libpixelflow_gb300.so.  No torch, no
cmake: plain nvcc, so the same recipe runs on x86-64 and aarch64 hosts.

The C++ host program host/pf_run.cpp (the reference's main program over the
C ABI) is then linked against that library as pixelflow_gb300/pf_run, with
-ffp-contract=off so that its text output has the same bits on x86-64 and
aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpixelflow_gb300.so")
HOST_SRC = os.path.join(HERE, "host", "pf_run.cpp")
HOST_BIN = os.path.join(HERE, "pf_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr"]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "pixelflow_gpu.h"))
    return hs


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJDIR, os.path.basename(src).replace(".cu", ".o"))
    cmd = [_nvcc(), *ARCH, *NVFLAGS, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    return obj


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in sources() + _headers())


def build_host(force: bool = False, verbose: bool = False) -> str:
    """Link host/pf_run.cpp against libpixelflow_gb300.so (g++, C++17)."""
    header = os.path.join(os.path.dirname(HERE), "include", "pixelflow_gpu.h")
    if (not force and os.path.exists(HOST_BIN)
            and all(os.path.getmtime(f) <= os.path.getmtime(HOST_BIN) for f in (HOST_SRC, header, LIB))):
        return HOST_BIN
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    tmp = HOST_BIN + ".tmp"
    common = ["-O2", "-std=c++17", "-I", os.path.dirname(header), HOST_SRC, "-o", tmp, "-L", HERE,
              "-lpixelflow_gb300"]
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx:
        cmd = [cxx, *common, "-pthread", "-Wall", "-ffp-contract=off", "-Wl,-rpath,$ORIGIN",
               f"-Wl,-rpath-link,{cuda_lib}"]
    else:  # nvcc hands a .cpp file to its own host compiler
        cmd = [_nvcc(), *common, "-Xcompiler", "-pthread,-Wall,-ffp-contract=off", "-Xlinker", "-rpath,$ORIGIN",
               "-Xlinker", f"-rpath-link,{cuda_lib}", "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(tmp, HOST_BIN)
    return HOST_BIN


def build(force: bool = False, verbose: bool = False) -> str:
    lib = build_lib(force=force, verbose=verbose)
    build_host(force=force, verbose=verbose)
    return lib


def build_lib(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", *objs, "-o", tmp, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
