"""Compile liboops_gb300.so in-tree with nvcc for sm_103a (GB300).

One -gencode (compute_103a -> sm_103a), translation units compiled in
parallel, then linked as a shared library next to this file.  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liboops_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-ffp-contract=off", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liboops_gb300")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include")
    deps += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith((".h", ".hpp"))]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps
                                   if os.path.exists(d)):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


HOST_DEMO_SRC = os.path.join(ROOT, "tests", "cpp", "host_demo.cpp")
HOST_DEMO = os.path.join(ROOT, "tests", "cpp", "_bin", "host_demo")
ENSNVEBATH_SRC = os.path.join(ROOT, "tests", "cpp", "ensnvebath_demo.cpp")
ENSNVEBATH = os.path.join(ROOT, "tests", "cpp", "_bin", "ensnvebath_demo")
ENSNVNBATH_SRC = os.path.join(ROOT, "tests", "cpp", "ensnvnbath_demo.cpp")
ENSNVNBATH = os.path.join(ROOT, "tests", "cpp", "_bin", "ensnvnbath_demo")


def _build_cpp(src, out):
    lib = build()
    os.makedirs(os.path.dirname(out), exist_ok=True)
    deps = [src, lib, os.path.join(ROOT, "include", "oops_host.hpp")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), src, "-o", out,
           "-L" + HERE, "-loops_gb300", "-Wl,-rpath," + HERE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(src)} build failed:\n{r.stdout}\n{r.stderr}")
    return out


def build_host_demo() -> str:
    """Compile the C++ host-layer test driver (tests/cpp/host_demo.cpp) with
    g++ against liboops_gb300.so; only the C/C++ headers are needed."""
    return _build_cpp(HOST_DEMO_SRC, HOST_DEMO)


def build_ensnvebath_demo() -> str:
    """Compile tests/cpp/ensnvebath_demo.cpp (the reference application's
    main over the C++ layer) against liboops_gb300.so."""
    return _build_cpp(ENSNVEBATH_SRC, ENSNVEBATH)


def build_ensnvnbath_demo() -> str:
    """Compile tests/cpp/ensnvnbath_demo.cpp (the reference's nuclear-bath
    application main over the C++ layer) against liboops_gb300.so."""
    return _build_cpp(ENSNVNBATH_SRC, ENSNVNBATH)


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
