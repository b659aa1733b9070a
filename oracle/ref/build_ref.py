"""Build oracle/_ref/libcrtref.so: the reference's own device code on the CPU.

TEST INFRASTRUCTURE ONLY (part of the oracle).  The reference (mbartling/
cuda-rt) has no CPU path and no tests.  Its hot-path device functions are
plain C++ behind __host__/__device__ qualifiers, so they compile for the host
with g++ once shim.h gives host meanings to the few CUDA built-ins they use.
The only lines that cannot compile as C++ are the host launch wrappers
(``kernel<<<grid, block>>>(...)``); those are left out and harness.cpp plays
their part.

Recipe (run from this container, where the reference checkout exists):
  * whole files, unmodified: kernels/mrand.cu, kernels/Light.cu,
    kernels/material.cu, kernels/camera.cu;
  * kernels/bvh.cu without lines 3-4 (thrust includes) and 259-293
    (BVH_d::computeMortonCodes / sortMortonCodes / setupLeafNodes /
    buildTree, the launch wrappers);
  * kernels/raytracer.cu without lines 55-92 (RayTracer::run, the launch
    wrapper);
  * kernels/scene.cu without lines 4-6 (thrust includes) and 48-85
    (Scene_d::computeBoundingBoxes, AverageSuperSampling, findMinMax: launch
    wrappers and the thrust reduction, restated in harness.cpp).
The kept line ranges are written to oracle/_ref/src/ and the checkout's
headers (inc/) to oracle/_ref/inc/ (git-ignored build intermediates, never
committed) and compiled with ``-O2 -ffp-contract=off -fopenmp`` so the double
arithmetic is evaluated exactly as written (no FMA contraction), as in the
oracle.  Where no checkout exists but those intermediates do (a machine that
received this tree with its build directory, e.g. an Arm GPU host, where the
x86 objects are of no use), ``build_extracted`` compiles them again.

Usage: python oracle/ref/build_ref.py [--reference DIR]
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libcrtref.so")

# (file, kept 1-based inclusive line ranges or None for the whole file)
PIECES = [
    ("kernels/bvh.cu", [(1, 2), (5, 258), (294, None)]),
    ("kernels/raytracer.cu", [(1, 54), (93, None)]),
    ("kernels/scene.cu", [(1, 3), (7, 47), (86, None)]),
    ("kernels/mrand.cu", None),
    ("kernels/Light.cu", None),
    ("kernels/material.cu", None),
    ("kernels/camera.cu", None),
]


# Where this container mounts the reference checkout; CRT_REFERENCE_DIR
# overrides it.  Every script that reads the reference's sources asks here.
REFERENCE_CHECKOUT = "/root/reference"


def default_reference():
    return os.environ.get("CRT_REFERENCE_DIR", REFERENCE_CHECKOUT)


def extract(ref, rel, ranges):
    with open(os.path.join(ref, rel)) as f:
        lines = f.readlines()
    if ranges is None:
        kept = lines
    else:
        kept = []
        for a, b in ranges:
            kept.extend(lines[a - 1:(b if b is not None else len(lines))])
    text = "".join(kept)
    if "<<<" in text:
        raise RuntimeError(f"{rel}: kept lines still contain a kernel launch; line ranges out of date")
    name = os.path.basename(rel).replace(".cu", "_ref.cpp")
    dst = os.path.join(OUT, "src", name)
    with open(dst, "w") as f:
        f.write(f'#line 1 "{rel}"\n' if ranges is None else "")
        f.write(text)
    return dst


def copy_headers(ref):
    dst = os.path.join(OUT, "inc")
    os.makedirs(dst, exist_ok=True)
    for name in sorted(os.listdir(os.path.join(ref, "inc"))):
        with open(os.path.join(ref, "inc", name), "rb") as f:
            data = f.read()
        with open(os.path.join(dst, name), "wb") as f:
            f.write(data)


def extracted_sources():
    srcs = [os.path.join(OUT, "src", os.path.basename(rel).replace(".cu", "_ref.cpp")) for rel, _ in PIECES]
    return srcs if all(os.path.exists(p) for p in srcs) and os.path.isdir(os.path.join(OUT, "inc")) else None


def build(ref=None, quiet=False):
    ref = ref or default_reference()
    if not os.path.isdir(os.path.join(ref, "kernels")):
        if not quiet:
            print(f"build_ref: no reference checkout at {ref}; skipped")
        return None
    os.makedirs(os.path.join(OUT, "src"), exist_ok=True)
    srcs = [extract(ref, rel, ranges) for rel, ranges in PIECES]
    copy_headers(ref)
    return _compile(srcs, quiet)


def build_extracted(quiet=False):
    """Compile the intermediates a build from a checkout left in oracle/_ref/."""
    srcs = extracted_sources()
    if srcs is None:
        if not quiet:
            print("build_ref: no extracted reference sources; skipped")
        return None
    return _compile(srcs, quiet)


def _compile(srcs, quiet):
    srcs = list(srcs) + [os.path.join(HERE, "harness.cpp")]
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-w",
             "-include", os.path.join(HERE, "shim.h"),
             "-I", os.path.join(OUT, "inc"), "-I", os.path.join(OUT, "src"), "-I", cuda_inc]
    objs, procs = [], []
    for src in srcs:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        procs.append(subprocess.Popen(["g++", *flags, "-x", "c++", "-c", src, "-o", obj]))
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("build_ref: compile failed")
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", LIB, *objs])
    if not quiet:
        print(f"build_ref: built {LIB}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    sys.exit(0 if build(a.reference) else 1)
