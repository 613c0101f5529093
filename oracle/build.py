"""Build the CPU oracles (test infrastructure only).

- oracle/_build/liborc.so : the plain-C restatement (oracle/vxr_oracle.c); always built.
- oracle/_ref/libvxref.so : the reference's own kernel source compiled for the CPU
  (oracle/ref_build.py); built when the reference checkout is present, or from a
  previously generated source in oracle/_ref/.
"""
import hashlib
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIBORC = os.path.join(BUILD, "liborc.so")


def build_port(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "vxr_oracle.c"), os.path.join(HERE, "vxr_oracle.h"),
            os.path.join(ROOT, "include", "vxr.h")]
    h = hashlib.sha256()
    for s in srcs:
        h.update(open(s, "rb").read())
    stamp = os.path.join(BUILD, "liborc.stamp")
    if not force and os.path.exists(LIBORC) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return LIBORC
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-I" + os.path.join(ROOT, "include"), "-I" + HERE, os.path.join(HERE, "vxr_oracle.c"), "-o",
           LIBORC + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(LIBORC + ".tmp", LIBORC)
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    return LIBORC


LIBSCENE = os.path.join(BUILD, "libscenehost.so")


def build_scene_host(force=False):
    """The project's scene generator (host C++ only) behind oracle/scene_host.cpp, for the
    reference arm of the benchmark: the same scenes without the CUDA library."""
    os.makedirs(BUILD, exist_ok=True)
    csrc = os.path.join(ROOT, "smallproject_gb300", "csrc")
    srcs = [os.path.join(HERE, "scene_host.cpp"), os.path.join(csrc, "world.cpp"), os.path.join(csrc, "scene.cpp")]
    deps = srcs + [os.path.join(csrc, "world.hpp"), os.path.join(ROOT, "include", "vxr.h")]
    h = hashlib.sha256()
    for s in deps:
        h.update(open(s, "rb").read())
    stamp = os.path.join(BUILD, "libscenehost.stamp")
    if not force and os.path.exists(LIBSCENE) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return LIBSCENE
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I" + os.path.join(ROOT, "include"), "-I" + csrc, *srcs, "-o", LIBSCENE + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("scene host build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(LIBSCENE + ".tmp", LIBSCENE)
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    return LIBSCENE


def build_ref(force=False):
    """Returns the reference-oracle library path, or None when it cannot be built here."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("ref_build", os.path.join(HERE, "ref_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force, quiet=True)


def build_stb():
    """Returns the stb_image checker library path (oracle/stb_ref.c), or None."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("ref_build", os.path.join(HERE, "ref_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build_stb(quiet=True)


def build_ogt():
    """Returns the ogt_vox checker library path (oracle/ogt_ref.cpp), or None."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("ref_build", os.path.join(HERE, "ref_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build_ogt(quiet=True)


def build_all(force=False):
    port = build_port(force)
    build_scene_host(force)
    try:
        ref = build_ref(force)
    except RuntimeError:
        ref = None
    for b in (build_stb, build_ogt):
        try:
            b()
        except RuntimeError:
            pass
    return port, ref


if __name__ == "__main__":
    print(build_all(force=True))
