"""Build of libanacor_gb300.so (sm_103a kernels + host C ABI), in-tree.

    python -m anacor_public_gb300.build          # builds anacor_public_gb300/_build/

Translation units compile in parallel: the CUDA file with nvcc for
``compute_103a/sm_103a`` only, the host C++ files with g++ and
``-ffp-contract=off`` (the host set-up must round exactly like the
reference's C, which is never contracted into FMA).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libanacor_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-std=c++17", "-Wall"]

CU_SOURCES = ["trace_kernels.cu", "voxel_order.cu", "noalloc.cu", "surrogate.cu", "gridding.cu", "sampling.cu",
              "distance_field.cu"]
CPP_SOURCES = ["reflection_setup.cpp", "capi.cpp", "gridding_capi.cpp"]


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES] + \
        [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(INCLUDE, "anacor_gb300.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I", CSRC, "-I", INCLUDE]
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(OUT, f + ".o")
        objs.append(o)
        cmd = [NVCC, *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xptxas", "-v", "-c",
               "-Xcompiler", ",".join(HOST_FLAGS), *inc, os.path.join(CSRC, f), "-o", o]
        jobs.append(cmd)
    gxx = shutil.which("g++") or "g++"
    for f in CPP_SOURCES:
        o = os.path.join(OUT, f + ".o")
        objs.append(o)
        jobs.append([gxx, *HOST_FLAGS, *inc, "-I", os.path.join(CUDA_HOME, "include"), "-c",
                     os.path.join(CSRC, f), "-o", o])
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for c in jobs]
    logs = []
    for c, p in zip(jobs, procs):
        out, _ = p.communicate()
        logs.append(out)
        if p.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(c) + "\n" + out)
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    tmp = LIB + ".tmp"
    link = [NVCC, *GENCODE, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: " + " ".join(link) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        f.write("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
