"""Build recipe for the reference oracle (oracle/_ref/libvxref.so).

TEST INFRASTRUCTURE ONLY. The reference renderer's per-frame path is OpenCL C
(cl/*.cl of marsicplusplus/SmallProject); there is no OpenCL runtime here, so this
recipe compiles the reference's OWN kernel source as C++17 for the host CPU:

1. read the hot-path sources where they lie in the reference checkout
   (template/common.h, cl/trace.cl, cl/tools.cl, cl/reservoir.cl, cl/phat.cl,
   cl/spatialSampling.cl, cl/ris.cl and two kernels of cl/kernels.cl);
2. apply mechanical rewrites only (OpenCL syntax -> C++ syntax):
   - address-space / access qualifiers removed;
   - vector literals "(float3)(a, b, c)" -> "vx_make_float3(a, b, c)" (compiled as
     C++ unchanged they would silently become comma expressions);
   - ".xyz" swizzle -> ".xyz()";
   - double literals -> float literals (the reference builds with
     -cl-single-precision-constant, template/template.cpp:1419);
   - SCRWIDTH/SCRHEIGHT become runtime variables, VOXELSAREPOINTLIGHTS overridable;
   - editor helpers that the parity configuration never calls (editorEnabled = 0)
     are replaced by aborting stubs;
3. write the result to oracle/_ref/vxref_gen.inc (git-ignored: reference source is
   never committed) and compile it with oracle/ref_shim.inc + oracle/ref_driver.cpp
   into oracle/_ref/libvxref.so, once per light model (area / point).

Usage: python oracle/ref_build.py [--reference PATH] [--force]
"""
import argparse
import hashlib
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: VXR_REFERENCE, else where this container mounts it
DEFAULT_REF = os.environ.get("VXR_REFERENCE", "/root/reference")

# tools.cl functions on the render path (the rest of tools.cl is TAA / tonemapping /
# editor code that the path never reaches)
TOOLS_FUNCS = [
    "WangHash", "RandomInt", "RandomFloat", "GenerateCameraRay", "GetAlpha", "GetAlphaf",
    "ToFloatRGB", "FromFloatRGBA", "VoxelNormal", "getRandomIndex", "indexToCoordinates",
    "GridCoordinatesFromHit", "Uint3CubeEquals", "ReprojectWorldPoint", "IsInBounds",
    "RandomPointOnVoxel", "GenerateLightCandidate", "PointOnVoxelLight", "UniformSampleHemisphere",
    # sky-dome sampling (skyDomeSampling = 1): SampleSky and its spherical angles, the
    # blue-noise sampler and the cosine-weighted hemisphere sample
    "SphericalTheta", "SphericalPhi", "SampleSky", "blueNoiseSampler", "DiffuseReflectionCosWeighted",
]
# render_di_gfxexp + renderPathTracer: the reference's ground-truth mode (GFXEXP = 1)
KERNELS_FUNCS = ["accumulatorFinalizer", "updateUberGrid", "render_di_gfxexp", "renderPathTracer"]

STUBS = r"""
// ---- stubs: referenced by render_di_ris only under editorEnabled, 0 in every
// ---- configuration this oracle runs; reaching one is a test bug.
inline bool HitSelectedBox(const float3, const float3, const float3, const float3, const float, float*) { std::abort(); }
inline bool HitWorldGrid(const float3, const float3) { std::abort(); }
"""


def read(ref, rel):
    with open(os.path.join(ref, rel), "r", encoding="utf-8-sig") as f:
        return f.read()


def extract_function(src, name):
    """Return the full definition of function `name` (signature through matching brace)."""
    m = re.search(r"(^|\n)([A-Za-z_][\w \t\*]*?\b" + re.escape(name) + r"\s*\()", src)
    if not m:
        raise RuntimeError(f"function {name} not found")
    start = m.start(2)
    # find end of parameter list
    i = src.index("(", m.start(2) + len(m.group(2)) - 1)
    depth = 0
    while True:
        c = src[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                break
        i += 1
    j = src.index("{", i)
    depth = 0
    k = j
    while True:
        c = src[k]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                break
        k += 1
    return src[start:k + 1]


NUM_RE = re.compile(
    r"0[xX][0-9a-fA-F]+[uUlL]*"                                  # hex integer
    r"|(?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?[fF]?"                 # decimal with point
    r"|\d+[eE][-+]?\d+[fF]?"                                     # exponent without point
    r"|\d+[uUlL]*"                                               # decimal integer
)


def float_literals(code):
    """Suffix every floating literal with f (-cl-single-precision-constant)."""
    out = []
    pos = 0
    for m in NUM_RE.finditer(code):
        s, e = m.span()
        # skip numbers that are part of identifiers
        if s > 0 and (code[s - 1].isalnum() or code[s - 1] == "_"):
            continue
        tok = m.group(0)
        out.append(code[pos:s])
        is_float = (not tok.lower().startswith("0x")) and ("." in tok or "e" in tok.lower())
        if is_float and not tok.endswith(("f", "F")):
            tok += "f"
        out.append(tok)
        pos = e
    out.append(code[pos:])
    return "".join(out)


def strip_comments(code):
    code = re.sub(r"/\*.*?\*/", " ", code, flags=re.S)
    return re.sub(r"//[^\n]*", "", code)


def rewrite(code):
    code = strip_comments(code)
    for q in ("__kernel", "__global", "__constant", "__read_only", "__write_only",
              "__local", "write_only", "read_only"):
        code = re.sub(r"\b" + q + r"\b", "", code)
    code = re.sub(r"\((float|int|uint|uchar)([234])\)\s*\(", r"vx_make_\1\2(", code)
    code = re.sub(r"\.xyz\b(?!\s*\()", ".xyz()", code)
    code = float_literals(code)
    return code


def rewrite_common(code):
    code = re.sub(r"#define\s+SCRWIDTH\s+\d+", "#define SCRWIDTH vxref_scr_width", code)
    code = re.sub(r"#define\s+SCRHEIGHT\s+\d+", "#define SCRHEIGHT vxref_scr_height", code)
    code = re.sub(r"#define\s+VOXELSAREPOINTLIGHTS\s+(\d+)",
                  r"#ifndef VOXELSAREPOINTLIGHTS\n#define VOXELSAREPOINTLIGHTS \1\n#endif", code)
    return rewrite(code)


def generate(ref):
    parts = ["// GENERATED by oracle/ref_build.py from the reference sources; do not commit.\n"]
    parts.append(rewrite_common(read(ref, "template/common.h")))
    parts.append("\n#define BRICKPARAMS brick0\n")          # kernels.cl:6-7 (ONEBRICKBUFFER == 1)
    parts.append(rewrite(read(ref, "cl/reservoir.cl")))
    tools = read(ref, "cl/tools.cl")
    parts.append("\n#define NUMBEROFVOXELSIDES 6\n")        # tools.cl:497
    parts.append(STUBS)
    for fn in TOOLS_FUNCS:
        parts.append(rewrite(extract_function(tools, fn)) + "\n")
    parts.append(rewrite(read(ref, "cl/trace.cl")))
    parts.append(rewrite(read(ref, "cl/phat.cl")))
    parts.append(rewrite(read(ref, "cl/spatialSampling.cl")))
    parts.append(rewrite(read(ref, "cl/ris.cl")))
    kern = read(ref, "cl/kernels.cl")
    for fn in KERNELS_FUNCS:
        parts.append(rewrite(extract_function(kern, fn)) + "\n")
    return "\n".join(parts)


def build(ref=DEFAULT_REF, force=False, quiet=False):
    """Generate (if the reference is present) and compile oracle/_ref/libvxref.so.

    Returns the library path, or None when neither the reference checkout nor a
    previously generated source is available.
    """
    os.makedirs(OUT, exist_ok=True)
    gen = os.path.join(OUT, "vxref_gen.inc")
    if os.path.isdir(ref):
        text = generate(ref)
        old = open(gen).read() if os.path.exists(gen) else None
        if old != text:
            with open(gen, "w") as f:
                f.write(text)
    elif not os.path.exists(gen):
        return None
    lib = os.path.join(OUT, "libvxref.so")
    srcs = [gen, os.path.join(HERE, "ref_shim.inc"), os.path.join(HERE, "ref_driver.cpp"),
            os.path.join(HERE, "..", "include", "vxr.h")]
    h = hashlib.sha256()
    for s in srcs:
        h.update(open(s, "rb").read())
    stamp = os.path.join(OUT, "libvxref.stamp")
    if (not force and os.path.exists(lib) and os.path.exists(stamp)
            and open(stamp).read() == h.hexdigest()):
        return lib
    flags = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
             "-ftrivial-auto-var-init=zero", "-fpermissive", "-w",
             "-I" + os.path.join(HERE, "..", "include"), "-I" + HERE]
    objs = []
    procs = []
    for variant, name in ((0, "area"), (1, "point")):
        obj = os.path.join(OUT, f"ref_driver_{name}.o")
        cmd = ["g++", *flags, f"-DVOXELSAREPOINTLIGHTS={variant}", f"-DVXREF_VARIANT={variant}",
               "-c", os.path.join(HERE, "ref_driver.cpp"), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("reference oracle build failed:\n" + " ".join(cmd) + "\n" + out.decode())
    cmd = ["g++", "-shared", "-fopenmp", "-o", lib, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: " + r.stdout + r.stderr)
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    if not quiet:
        print("built", lib)
    return lib


def build_stb(ref=DEFAULT_REF, quiet=False):
    """Compile oracle/stb_ref.c against the reference's vendored stb_image headers
    (lib/stb_image.h, lib/stb_image_write.h, included where they lie) into
    oracle/_ref/libstbref.so. Returns the path, or None without the reference checkout
    (and no earlier build)."""
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libstbref.so")
    inc = os.path.join(ref, "lib")
    if not os.path.isfile(os.path.join(inc, "stb_image.h")):
        return lib if os.path.exists(lib) else None
    src = os.path.join(HERE, "stb_ref.c")
    h = hashlib.sha256()
    for s in (src, os.path.join(inc, "stb_image.h"), os.path.join(inc, "stb_image_write.h")):
        h.update(open(s, "rb").read())
    stamp = os.path.join(OUT, "libstbref.stamp")
    if os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return lib
    cmd = ["gcc", "-O1", "-shared", "-fPIC", "-w", "-I" + inc, src, "-o", lib, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("stb_image checker build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    if not quiet:
        print("built", lib)
    return lib


def build_ogt(ref=DEFAULT_REF, quiet=False):
    """Compile oracle/ogt_ref.cpp against the reference's vendored lib/ogt_vox.h (included
    where it lies) into oracle/_ref/libogtref.so. Returns the path, or None without the
    reference checkout (and no earlier build)."""
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libogtref.so")
    inc = os.path.join(ref, "lib")
    if not os.path.isfile(os.path.join(inc, "ogt_vox.h")):
        return lib if os.path.exists(lib) else None
    src = os.path.join(HERE, "ogt_ref.cpp")
    h = hashlib.sha256()
    for s in (src, os.path.join(inc, "ogt_vox.h")):
        h.update(open(s, "rb").read())
    stamp = os.path.join(OUT, "libogtref.stamp")
    if os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return lib
    cmd = ["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-w", "-DNDEBUG", "-I" + inc, src, "-o", lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("ogt_vox checker build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    if not quiet:
        print("built", lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REF)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    r = build(a.reference, a.force)
    build_stb(a.reference)
    build_ogt(a.reference)
    if r is None:
        sys.exit("reference checkout not found and no generated source present")
