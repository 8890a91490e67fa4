"""Build recipe of the reference-kernel harness (test infrastructure only).

* ``oracle/_ref/pmsz_ref.cubin`` -- the UNMODIFIED reference ``pMSz.cu``,
  compiled where it lies (``$PMSZ_REFERENCE_DIR``, by default
  ``/root/reference``) into sm_103a device code, with
  the declaration-only headers of ``oracle/ref_shim`` standing in for MPI,
  SZ3, ZFP and zstd (the cubin keeps only the kernels; nothing of those
  libraries is called).  Built only where the reference sources exist; the
  cubin then travels with the repository copy.
* ``oracle/_ref/naive_ref.cubin`` -- the unmodified ``naive_MSz.cu``, the
  same way.
* ``oracle/_ref/ref_harness`` -- ``oracle/ref_harness.cpp`` (driver API),
  compiled on the machine that runs it.
* ``oracle/_ref/ref_encoder`` -- ``oracle/ref_encoder.cu``: the unmodified
  ``pMSz.cu`` included whole, host side, with the real ``libzstd.so.1``; it
  runs the reference's own edit-file encoder on the host (no GPU needed).

Everything lands in ``oracle/_ref/`` (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# where the reference's sources lie: $PMSZ_REFERENCE_DIR, by default the
# read-only checkout at /root/reference
REF_DIR = os.environ.get("PMSZ_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_DIR, "pMSz.cu")
CUBIN = os.path.join(OUT, "pmsz_ref.cubin")
NAIVE_SRC = os.path.join(REF_DIR, "naive_MSz.cu")
NAIVE_CUBIN = os.path.join(OUT, "naive_ref.cubin")
HARNESS = os.path.join(OUT, "ref_harness")
ENCODER = os.path.join(OUT, "ref_encoder")


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _cubin(src: str, out: str) -> str | None:
    if not os.path.exists(src):
        return out if os.path.exists(out) else None
    os.makedirs(OUT, exist_ok=True)
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        cmd = [os.path.join(_cuda_home(), "bin", "nvcc"), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
               "-std=c++17", "-I" + os.path.join(HERE, "ref_shim"), src, "-o", out]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def build_cubin() -> str | None:
    """pMSz.cu -> pmsz_ref.cubin, and naive_MSz.cu -> naive_ref.cubin."""
    _cubin(NAIVE_SRC, NAIVE_CUBIN)
    return _cubin(REF_SRC, CUBIN)


def build_harness() -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cpp")
    if not os.path.exists(HARNESS) or os.path.getmtime(HARNESS) < os.path.getmtime(src):
        cuda = _cuda_home()
        libdir = next(d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                  os.path.join(cuda, "targets", "sbsa-linux", "lib"))
                      if os.path.isdir(os.path.join(d, "stubs")))
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I" + os.path.join(cuda, "include"), src,
               "-o", HARNESS, "-L" + os.path.join(libdir, "stubs"), "-lcuda"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    return HARNESS


def build_encoder() -> str | None:
    """pMSz.cu (host side) + oracle/ref_encoder.cu -> ref_encoder; None where
    the reference's sources are absent."""
    src = os.path.join(HERE, "ref_encoder.cu")
    if not os.path.exists(REF_SRC):
        return ENCODER if os.path.exists(ENCODER) else None
    os.makedirs(OUT, exist_ok=True)
    deps = [src, REF_SRC, os.path.join(HERE, "ref_shim", "zstd.h")]
    if not os.path.exists(ENCODER) or any(os.path.getmtime(ENCODER) < os.path.getmtime(d) for d in deps):
        cmd = [os.path.join(_cuda_home(), "bin", "nvcc"), "-std=c++17", "-O1", "-gencode",
               "arch=compute_103a,code=sm_103a", "-I" + os.path.join(HERE, "ref_shim"), "-I" + REF_DIR, src, "-o",
               ENCODER, "-l:libzstd.so.1", "-Xcompiler", "-w"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    return ENCODER


if __name__ == "__main__":
    print(build_cubin())
    if "--harness" in sys.argv:
        print(build_harness())
    if "--encoder" in sys.argv:
        print(build_encoder())
