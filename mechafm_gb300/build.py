"""In-tree build of libmafm.so (sm_103a) and the mechafm-gpu executable.

nvcc compiles each CUDA translation unit for sm_103a only; g++ compiles the
host front-end.  Host code everywhere is compiled with -ffp-contract=off so
that it computes the same bits as the reference's x86-64 build (no fused
multiply-add in the host arithmetic of centring, mixing and matrix inverses).
relax64.cu is compiled with -fmad=false for the same reason on the device,
and so is relaxdf.cu, whose FP64 re-relaxation of near-tie columns must give
relax64.cu's bits (its double-float arithmetic uses explicitly rounded
intrinsics, which -fmad does not touch).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(HERE, "libmafm.so")
BIN_DIR = os.path.join(HERE, "bin")
CLI = os.path.join(BIN_DIR, "mechafm-gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _units():
    nv = _nvcc()
    common = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-I" + INCLUDE, "-Xcompiler",
                     "-fPIC,-ffp-contract=off", "-c"]
    cuda_inc = os.path.join(_cuda_home(), "include")
    return [
        ([nv] + common + ["-fmad=false", os.path.join(CSRC, "relax64.cu")], "relax64.o"),
        ([nv] + common + [os.path.join(CSRC, "relax32.cu")], "relax32.o"),
        ([nv] + common + ["-fmad=false", os.path.join(CSRC, "relaxdf.cu")], "relaxdf.o"),
        ([nv] + common + [os.path.join(CSRC, "scan.cu")], "scan.o"),
        ([nv] + common + [os.path.join(CSRC, "noalloc.cu")], "noalloc.o"),
        ([nv] + common + [os.path.join(CSRC, "adjoint.cu")], "adjoint.o"),
        ([nv] + common + [os.path.join(CSRC, "df.cu")], "df.o"),
        ([nv] + common + ["-fmad=false", os.path.join(CSRC, "flex.cu")], "flex.o"),
        (["g++", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-Wall",
          "-I" + INCLUDE, "-I" + cuda_inc, "-c", os.path.join(CSRC, "frontend.cpp")],
         "frontend.o"),
    ]


def build(verbose: bool = False) -> str:
    """Compile every translation unit in parallel and link libmafm.so and the CLI."""
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for cmd, obj in _units():
        jobs.append((cmd + ["-o", os.path.join(BUILD, obj)], obj))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for l in logs:
            print(l)
    objs = [os.path.join(BUILD, o) for _, o in jobs]
    tmp = LIB + ".tmp"
    _run([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs +
         ["-lcufft", "-Xcompiler", "-fopenmp"])
    os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "mechafm_gpu.cpp")
    if os.path.exists(cli_src):
        os.makedirs(BIN_DIR, exist_ok=True)
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-pthread", "-I" + INCLUDE,
              cli_src, "-o", CLI, "-L" + HERE, "-lmafm", "-Wl,-rpath,$ORIGIN/.."])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
