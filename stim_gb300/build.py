"""Builds libstim_gb300.so in-tree: nvcc for the sm_103a kernels, g++ for the host runtime, linked with
the CUDA runtime statically so the library needs nothing but the driver at run time."""

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libstim_gb300.so")
ROOT = os.path.dirname(HERE)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["kernels.cu", "frame_lean.cu", "formats.cu", "noalloc.cu"]
CC_SOURCES = ["circuit.cc", "lower.cc", "tableau.cc", "formats.cc", "capi.cc", "batch.cc", "serve.cc", "m2d.cc", "dem.cc", "dem_sampler.cc", "feed.cc"]
HEADERS = ["gfs_contract.h", "gfs_gates.h", "frame_rules.h", "circuit.h", "lower.h", "program.h", "kernels.h", "frame_device.cuh", "noalloc.h", "sampler.h", "batch_engine.h", "tableau.h", "formats.h", "formats_device.h", "dem.h"]


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in CU_SOURCES + CC_SOURCES + HEADERS]
    paths.append(os.path.join(ROOT, "include", "stim_gb300.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC,
                     "-c", os.path.join(CSRC, f), "-o", o])
    for f in CC_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", "-I", CSRC,
                     "-I", os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, f), "-o", o])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs]
    failed = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out)
        if p.returncode:
            failed.append(" ".join(j))
    if failed:
        raise RuntimeError("build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    subprocess.run([NVCC, *ARCH, "-shared", "-cudart=static", "-o", tmp, *objs], check=True)
    shutil.move(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
