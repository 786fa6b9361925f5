"""Builds libgbpx.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel with nvcc and
linked into ``physx_gb300/libgbpx.so``; ``csrc/immediate.cpp`` (the
reference's immediate-mode entry points over that C ABI) becomes
``physx_gb300/libgbpx_immediate.so``.  Nothing is installed anywhere.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbpx.so")
LIB_IMMEDIATE = os.path.join(HERE, "libgbpx_immediate.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no fused multiply-add, so contact and solver arithmetic rounds
# like the reference (whose SSE2 build has no FMA).  IEEE division and square
# root stay on (no fast-math flags).
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                     "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 extension cannot be built")


def _compile(nvcc, src):
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(NVCC_FLAGS)
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
        with open(stamp, "w") as fh:
            fh.write(flags)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s), srcs))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        if verbose:
            print("built", LIB, file=sys.stderr)
    _build_immediate(verbose)
    return LIB


def _build_immediate(verbose=False):
    src = os.path.join(CSRC, "immediate.cpp")
    include = os.path.join(os.path.dirname(HERE), "include")
    deps = [src, LIB, os.path.join(include, "gbpx.h"), os.path.join(include, "gbpx_immediate.h")]
    if os.path.exists(LIB_IMMEDIATE) and os.path.getmtime(LIB_IMMEDIATE) >= max(os.path.getmtime(d) for d in deps):
        return LIB_IMMEDIATE
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-fvisibility=hidden", "-I" + include, src, "-o", LIB_IMMEDIATE,
           "-L" + HERE, "-lgbpx", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("immediate-mode library build failed:\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB_IMMEDIATE, file=sys.stderr)
    return LIB_IMMEDIATE


if __name__ == "__main__":
    build(verbose=True)
