"""Build libvxr.so (the C ABI renderer) in-tree: smallproject_gb300/lib/libvxr.so.

CUDA sources compile for sm_103a only (-gencode arch=compute_103a,code=sm_103a) with
--fmad=false: the render path's float arithmetic must round every operation
separately to stay bit-identical with the reference. Host C++ uses -ffp-contract=off
for the same reason (Arm compilers contract by default).
"""
import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libvxr.so")
INCLUDE = os.path.join(ROOT, "include")

CU_SOURCES = ["kernels.cu", "runtime.cu", "batch.cu", "noalloc.cu", "proposal.cu", "proposal_api.cu", "train.cu"]
CPP_SOURCES = ["world.cpp", "scene.cpp", "camera.cpp", "capi_world.cpp", "cluster.cpp", "sky.cpp"]
HEADERS = ["device.cuh", "kernels.hpp", "world.hpp", "camera.hpp", "internal.hpp", "proposal.cuh", "proposal.hpp", "proposal_dev.cuh", "view.hpp"]

# the learned proposal is checked with tolerances, not bit for bit: FMA contraction on
FMA_SOURCES = {"proposal.cu", "train.cu"}

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-I" + INCLUDE, "-I" + CSRC]


def _digest():
    h = hashlib.sha256()
    for f in CU_SOURCES + CPP_SOURCES + HEADERS:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(f.encode() + fh.read())
    with open(os.path.join(INCLUDE, "vxr.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of libvxr.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(LIBDIR, "libvxr.stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = os.path.join(objdir, s + ".o")
        flags = [f for f in NVCC_FLAGS if f != "--fmad=false"] if s in FMA_SOURCES else NVCC_FLAGS
        jobs.append([NVCC, *flags, "-Xptxas", "-v", "-c", os.path.join(CSRC, s), "-o", o])
        objs.append(o)
    for s in CPP_SOURCES:
        o = os.path.join(objdir, s + ".o")
        jobs.append(["g++", *CXX_FLAGS, "-c", os.path.join(CSRC, s), "-o", o])
        objs.append(o)
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
