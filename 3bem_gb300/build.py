"""Build the in-tree shared library lib/libtbem_gpu.so for sm_103a.

Host C++ (tree.cpp) is compiled by g++ without FMA contraction so that the
octree arithmetic rounds like the reference on x86 and Arm alike; every .cu
file is compiled by nvcc for sm_103a only, all translation units in parallel,
and linked against cuBLAS / cuSOLVER.  Rebuilds only what changed.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libtbem_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code of the .cu files rounds as on any host: no FMA contraction (GCC
# contracts by default on aarch64, not on x86-64); device code keeps nvcc's
# default (--fmad=true)
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + INCLUDE] + ARCH
CXX_FLAGS = ["-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-I" + INCLUDE]


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    deps = _headers() + [os.path.abspath(__file__)]  # a change of flags rebuilds everything
    steps = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            steps.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            steps.append([NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj])
    jobs = jobs or max(1, min(len(steps), os.cpu_count() or 4))
    if steps:
        with cf.ThreadPoolExecutor(jobs) as ex:
            for out in ex.map(_run, steps):
                if verbose and out.strip():
                    print(out)
    if steps or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcusolver", "-lcublas", "-lcudart",
                                                               "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
