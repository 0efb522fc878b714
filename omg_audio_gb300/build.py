"""Build libomg_cuda.so in-tree for sm_103a (nvcc + g++, compiled in parallel).

CUDA files build with -fmad=false so every f32 operation rounds as written
(the tracer reproduces the reference's f32 arithmetic term by term); host
C++ builds with -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libomg_cuda.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["trace.cu", "wavefront.cu", "coop.cu", "reverb.cu", "lbvh.cu", "sah3.cu", "dome.cu", "noalloc.cu", "mlp.cu", "late.cu", "early.cu"]
CPP_SOURCES = ["api.cpp", "api_scene.cpp", "api_dome.cpp", "api_mlp.cpp", "api_late.cpp", "api_wire.cpp", "api_early.cpp", "scene.cpp"]


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES]


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "omg_cuda.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "..", "include"), "-I", CSRC]
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xptxas", "-v",
                     "-Xcompiler", "-fPIC", *inc, "-c", os.path.join(CSRC, f), "-o", obj])
    for f in CPP_SOURCES:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wno-unused-function",
                     "-I", os.path.join(CUDA_HOME, "include"), *inc, "-c", os.path.join(CSRC, f), "-o", obj])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stderr.write(o)
    objs = [os.path.join(BUILD, f + ".o") for f in CU_SOURCES + CPP_SOURCES]
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl", "-lgomp"])
    os.replace(tmp, LIB)
    # ptxas register / spill report for the record
    with open(os.path.join(BUILD, "ptxas.txt"), "w") as fh:
        fh.write("\n".join(outs))
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
