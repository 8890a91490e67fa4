"""Build recipe of the native library ``libpmsz_gb300.so`` (and the ``pmsz``
command-line program).

Every CUDA translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, into
``pmsz_anonymous_gb300/_build/``; the shared library lands in
``pmsz_anonymous_gb300/lib/``.  ``-fmad=false`` keeps every floating-point
operation separately rounded, as the CPU oracle's ``-ffp-contract=off`` does.
Rebuilds only what is out of date.
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
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libpmsz_gb300.so")
CLI = os.path.join(LIBDIR, "pmsz")

CUDA_SOURCES = ["support.cu", "correct.cu", "verify.cu", "edits.cu", "gen.cu", "host.cu", "batch.cu", "server.cu", "naive.cu",
                "tune.cu"]
CXX_SOURCES = ["encode.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pmsz_anonymous_gb300")


def _headers():
    hs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra_defs=()) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _stale(obj, [path, *_headers()]):
        return obj
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false",
               "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-O3", f"-I{INCLUDE}",
               *extra_defs, "-c", path, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off",
               f"-I{INCLUDE}", *extra_defs, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    """Compile (if needed) and return the path of libpmsz_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = CUDA_SOURCES + CXX_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-l:libzstd.so.1"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB, *_headers()]):
        cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
        cudalib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"))
                        if os.path.exists(os.path.join(d, "libcudart.so"))), os.path.join(cuda, "lib64"))
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", f"-I{INCLUDE}", f"-I{os.path.join(cuda, 'include')}",
               cli_src, "-o", CLI, f"-L{LIBDIR}", "-lpmsz_gb300", f"-L{cudalib}", "-lcudart",
               f"-Wl,-rpath,$ORIGIN:{cudalib}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
