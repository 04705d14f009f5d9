"""Build libfemgpu.so in-tree: CUDA kernels for sm_103a (nvcc) plus the host C
driver (gcc), linked against the CUDA runtime.  No torch extension machinery:
the library has a plain C ABI (include/femgpu.h)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libfemgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + HOST,
       "-I" + os.path.join(CUDA_HOME, "include")]

# Translation units whose arithmetic must round every operation separately
# (element builds and the AMG smoother: bit-parity with the reference compiled
# without contraction).
NO_FMA = {"amg.cu", "build.cu", "ebe_block.cu", "euler_build.cu", "ns_build.cu"}


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(HOST) if f.endswith(".c"))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
        [os.path.join(HOST, f) for f in os.listdir(HOST)] + [os.path.join(ROOT, "include", "femgpu.h")]
    return cu, c, deps


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    cu, c, deps = _sources()
    if not force and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= mt for d in deps):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs, objs = [], []
    for f in cu:
        o = os.path.join(BUILD, f + ".o")
        flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3"]
        # build-time tuning macros (e.g. -DFG_SW2_CW=24: consumer warps of the ILU(0) sweeps)
        flags += os.environ.get("FEMGPU_NVCC_EXTRA", "").split()
        if f in NO_FMA:
            flags += ["--fmad=false"]
        jobs.append([NVCC] + ARCH + flags + INC + ["-c", os.path.join(CSRC, f), "-o", o])
        objs.append(o)
    for f in c:
        o = os.path.join(BUILD, f + ".o")
        jobs.append(["gcc", "-O2", "-fPIC", "-std=c11", "-Wall", "-Wno-unused-function",
                     "-ffp-contract=off"] + INC + ["-c", os.path.join(HOST, f), "-o", o])
        objs.append(o)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(_compile, jobs))
    if verbose:
        for o in outs:
            if o:
                sys.stderr.write(o)
    tmp = LIB + ".tmp"
    _compile([NVCC] + ARCH + ["-shared", "-o", tmp] + objs +
             ["-L" + os.path.join(CUDA_HOME, "lib64"), "-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
