"""Compile the CUDA library (libcrt.so) for sm_103a, in tree.

The library is built with nvcc directly: one translation unit per stage
family (build.cu, trace.cu, capi.cu, ...), compiled in parallel, linked with
the static CUDA runtime into ``cuda-rt_gb300/lib/libcrt.so``.  ``-fmad=false``
is required: the exact double-precision routines must not have their
multiply-adds contracted into FMAs (the reference's results are defined by
separately rounded products and sums).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libcrt.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
CLI_DIR = os.path.join(PKG, "cli")
CLI = os.path.join(LIBDIR, "crt_raytracer")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    srcs = sources()
    if not force and not _stale(LIB, srcs + headers + [__file__]):
        build_cli()
        return LIB
    objs, procs = [], []
    for src in srcs:
        obj = os.path.join(LIBDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [nvcc(), *ARCH, *FLAGS, *extra_flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out))
        elif verbose and out:
            print(out)
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    build_cli()
    return LIB


def build_cli() -> str:
    """The drop-in command-line renderer (cli/crt_raytracer.cpp), linked
    against libcrt.so next to it."""
    src = os.path.join(CLI_DIR, "crt_raytracer.cpp")
    if _stale(CLI, [src, LIB, os.path.join(INCLUDE, "crt.h"), os.path.join(INCLUDE, "crt.hpp")]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", INCLUDE, src, "-L", LIBDIR, "-lcrt",
                               "-Wl,-rpath,$ORIGIN", "-o", CLI])
    return CLI


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
