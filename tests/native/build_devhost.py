"""Build tests/native/_build/libdevhost.so (device.cuh compiled for the host)."""
import hashlib
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def cuda_include():
    for p in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if p and os.path.exists(os.path.join(p, "include", "cuda_runtime.h")):
            return os.path.join(p, "include")
    return None


def build():
    inc = cuda_include()
    if inc is None:
        return None
    out = os.path.join(HERE, "_build")
    os.makedirs(out, exist_ok=True)
    lib = os.path.join(out, "libdevhost.so")
    srcs = [os.path.join(HERE, "devhost.cpp"), os.path.join(ROOT, "smallproject_gb300", "csrc", "device.cuh")]
    h = hashlib.sha256(b"".join(open(s, "rb").read() for s in srcs)).hexdigest()
    stamp = lib + ".stamp"
    if os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read() == h:
        return lib
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-I" + inc, "-I" + os.path.join(ROOT, "smallproject_gb300", "csrc"), srcs[0], "-o", lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    open(stamp, "w").write(h)
    return lib
