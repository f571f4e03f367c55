"""In-tree build of the native libraries (no setuptools, no cmake).

  _build/libawg_sim.so          seeded input generator (host C++)
  _build/libargweaver_gb300.so  the threading HMM: sm_103a CUDA kernels + host runtime +
                                the reference-compatible C ABI (include/argweaver_gb300.h)

Translation units compile in parallel; a unit is rebuilt only when its source, a header
or the flags changed. Both libraries build without a GPU (nvcc cross-compiles).
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

SIM_LIB = os.path.join(BUILD, "libawg_sim.so")
CUDA_LIB = os.path.join(BUILD, "libargweaver_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall"]
# FP64 kernels keep IEEE products and sums separate (no FMA contraction) so the plain path
# rounds like the reference's host code. Translation units of FP32-only kernels (FMA_SOURCES)
# compile with contraction on; their error-free transforms use explicitly rounded intrinsics.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC] + ARCH
FMA_SOURCES: set = set()


def nvcc_flags(src: str):
    if src in FMA_SOURCES:
        return [f if f != "--fmad=false" else "--fmad=true" for f in NVCC_FLAGS]
    return NVCC_FLAGS

CUDA_SOURCES = ["host_plan.cpp", "tables.cu", "forward.cu", "traceback.cu",
                "backward.cu", "batch.cu", "static_run.cu", "dense_hmm.cu", "dense_tables.cu",
                "arg_prob.cu", "recomb.cu", "capi.cpp", "server.cpp", "formats.cpp",
                "arg_surgery.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _digest(paths, flags) -> str:
    h = hashlib.sha256()
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _headers():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _run_parallel(jobs):
    procs = [(desc, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
             for desc, cmd in jobs]
    failed = []
    for desc, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((desc, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(f"--- {d} ---\n{o}" for d, o in failed)
        raise RuntimeError(f"native build failed:\n{msg}")


def build_sim(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "sim.cpp")
    stamp = SIM_LIB + ".stamp"
    key = _digest([src], HOST_FLAGS)
    if os.path.exists(SIM_LIB) and os.path.exists(stamp) and open(stamp).read() == key:
        return SIM_LIB
    cxx = os.environ.get("CXX", "g++")
    _run_parallel([("sim.cpp", [cxx] + HOST_FLAGS + ["-shared", "-o", SIM_LIB, src])])
    with open(stamp, "w") as f:
        f.write(key)
    return SIM_LIB


def build_cuda(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs, objs = [], []
    for src in CUDA_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        stamp = obj + ".stamp"
        key = _digest([path] + headers, nvcc_flags(src))
        if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
            continue
        cmd = [nvcc] + nvcc_flags(src) + ["-c", "-o", obj, path]
        jobs.append((src, cmd))
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
    _run_parallel(jobs)
    for src, _ in jobs:
        obj = os.path.join(BUILD, src + ".o")
        with open(obj + ".stamp", "w") as f:
            f.write(_digest([os.path.join(CSRC, src)] + headers, nvcc_flags(src)))
    link = [nvcc] + ARCH + ["-shared", "-o", CUDA_LIB] + objs + ["-lcudart_static", "-lrt",
                                                                  "-lpthread", "-ldl"]
    _run_parallel([("link", link)])
    return CUDA_LIB


def build_all(verbose: bool = False) -> None:
    build_sim(verbose)
    build_cuda(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(CUDA_LIB)
