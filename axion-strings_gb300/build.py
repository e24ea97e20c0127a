"""Build recipe for libaxs.so (CUDA, sm_103a) and the axs_run driver.

Compiles each CUDA translation unit in parallel with nvcc for
sm_103a only, links them with cuFFT into an in-tree shared library, and
builds the C++ host driver against it. No CMake; no torch extension machinery.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaxs.so")
DRIVER = os.path.join(HERE, "host", "axs_run")

CUDA_SOURCES = ["axs_step.cu", "axs_step_r.cu", "axs_init.cu", "axs_analysis.cu", "axs_api.cu"]
HOST_SOURCES = ["axs_params.cpp", "axs_fileio.cpp", "axs_run.cpp"]

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, "axs_internal.h"), os.path.join(CSRC, "axs_tma.cuh"), os.path.join(ROOT, "include", "axs.h")]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcufft", "-lcudart"])
    hsrc = [os.path.join(HOST, s) for s in HOST_SOURCES]
    if all(os.path.exists(s) for s in hsrc) and (force or _stale(DRIVER, hsrc + [LIB, os.path.join(HOST, "axs_host.h")])):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(_which(NVCC))), "lib64")
        _run([CXX, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-o", DRIVER]
             + hsrc + ["-L" + HERE, "-laxs", "-Wl,-rpath," + HERE, "-L" + cuda_lib, "-Wl,-rpath," + cuda_lib, "-lcudart"])
    return LIB


def _which(prog):
    if os.path.isabs(prog):
        return prog
    for d in os.environ.get("PATH", "").split(os.pathsep):
        p = os.path.join(d, prog)
        if os.path.exists(p):
            return p
    return "/usr/local/cuda/bin/nvcc"


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
