"""Build the engine's CUDA library in-tree (rheocell_gb300/_build/).

Compiles every translation unit under csrc/ for sm_103a with nvcc (in
parallel), links librheocell_gb300.so with the CUDA runtime statically, and
never touches site-packages.  FP64 kernels are compiled without FMA
contraction so that single evaluations match the reference's arithmetic;
the FP32-only units (FMA_UNITS) keep it.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "librheocell_gb300.so")
CLI = os.path.join(BUILD, "rheocell")
GEN = os.path.join(BUILD, "confgenerator")
HOST_SRC = os.path.join(HERE, "host", "rheocell.cpp")
GEN_SRC = os.path.join(HERE, "host", "confgenerator.cpp")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3"]
# Translation units whose FP32 arithmetic is not held to the reference bit for
# bit (FP32 cell kernels, network training) keep FMA contraction; every other
# unit -- the FP64 kernels, box sums, solves and observables -- is compiled
# without it, as the reference's exact build evaluates its expressions.
FMA_UNITS = ("rc_cells_f32.cu", "rc_unet.cu")


def unit_flags(src: str):
    return NVCC_FLAGS + ["--fmad=" + ("true" if os.path.basename(src) in FMA_UNITS else "false")]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the GB300 engine needs the CUDA toolkit to build")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(HERE, "..", "include", "rheocell_gb300.h")]


def up_to_date() -> bool:
    if not all(os.path.exists(f) for f in (LIB, CLI, GEN)):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI), os.path.getmtime(GEN))
    return all(os.path.getmtime(d) <= t for d in _deps() + [HOST_SRC, GEN_SRC])


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nv] + unit_flags(src) + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 8, len(sources()) or 1)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    # the command-line driver (C++ host above the C ABI)
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", HOST_SRC, "-o", CLI + ".tmp",
           "-L" + BUILD, "-lrheocell_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host driver build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(CLI + ".tmp", CLI)
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", GEN_SRC, "-o", GEN + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("confgenerator build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(GEN + ".tmp", GEN)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
