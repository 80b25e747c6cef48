"""Build libcmag_sph.so in-tree: every translation unit compiled by nvcc for
sm_103a in parallel, then linked as one shared library."""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcmag_sph.so")

SOURCES = ["sort.cu", "cells.cu", "density.cu", "force.cu", "integrate.cu", "reduce.cu", "system.cu", "batch.cu", "closure.cu", "closure_api.cu", "render.cu", "verlet.cu",
           "host_scenes.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no fused multiply-add, so host float arithmetic (parameters, scenes,
# phase mirror) matches the reference expressions on x86_64 and aarch64 alike.
# device code (-fmad=false): only the fused multiply-adds written out in the
# kernels, so every template variant of a kernel rounds identically
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-ffp-contract=off", "-fmad=false", "--expt-relaxed-constexpr", "-I" + SRC]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, extra):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + list(extra) + ["-c", os.path.join(SRC, src), "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), out.stderr))
    return obj, out.stderr


def build(verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), out.stderr))
    os.replace(tmp, LIB)
    return LIB


HARNESS = os.path.join(OUT_DIR, "report")


def build_harness():
    """The ported Report programs (host C++ on include/cmag/systems.hpp)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    root = os.path.dirname(PKG)
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(root, "include"),
           "-I" + os.path.join(cuda, "include"), os.path.join(PKG, "harness", "report.cpp"),
           "-L" + PKG, "-lcmag_sph", "-Wl,-rpath," + PKG, "-o", HARNESS]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("harness build failed:\n%s\n%s" % (" ".join(cmd), out.stderr))
    return HARNESS


def stale():
    """True when the library is missing or older than any source or header."""
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps.append(os.path.join(os.path.dirname(PKG), "include", "cmag_sph.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_if_stale():
    return build() if stale() else LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ()))
