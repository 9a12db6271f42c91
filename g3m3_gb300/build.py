"""Build libg3m3_gpu.so (sm_103a) in-tree: g3m3_gb300/lib/libg3m3_gpu.so.

Every translation unit is compiled in parallel with nvcc for sm_103a only,
with IEEE division and square root and no multiply-add contraction
(-fmad=false): the kernels are written to reproduce the reference's FP32
operation order bit for bit, and bandwidth, not arithmetic, bounds them.
The reverse-mode kernels are the exception (FAST_MATH_FILES).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libg3m3_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
         "-ftz=false", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         # host-side float arithmetic (time steps, geometry) must not be fused
         # either: gcc contracts a*b+c into fma by default on aarch64
         "-Xcompiler", "-ffp-contract=off",
         "-I", os.path.join(HERE, "..", "include")]


# The reverse-mode kernels (k_adj.cu) compute gradients, which no bitwise
# comparison constrains: they build with contraction and the fast division
# and square root.
FAST_MATH_FILES = {"k_adj.cu"}
FAST = {"-fmad=false": "-fmad=true", "-prec-div=true": "-prec-div=false", "-prec-sqrt=true": "-prec-sqrt=false"}


def flags_for(src):
    if os.path.basename(src) in FAST_MATH_FILES:
        return [FAST.get(f, f) for f in FLAGS]
    return FLAGS


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


# Sources also built in the contracted flavour (FMA contraction, quotients
# by shared denominators as reciprocal products), into g3m3::contracted.
CONTRACTED_FILES = {"k_push_tiled.cu"}


def units():
    """(source, object, extra flags) of every translation unit."""
    out = []
    for src in sources():
        base = os.path.basename(src)[:-3]
        out.append((src, os.path.join(BUILD_DIR, base + ".o"), flags_for(src)))
        if os.path.basename(src) in CONTRACTED_FILES:
            fl = [FAST.get(f, f) if f == "-fmad=false" else f for f in FLAGS] + ["-DG3M3_CONTRACTED"]
            out.append((src, os.path.join(BUILD_DIR, base + "_contracted.o"), fl))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(HERE, "..", "include", f) for f in os.listdir(os.path.join(HERE, "..", "include"))]
    jobs = []
    objs = []
    for src, obj, fl in units():
        objs.append(obj)
        if _stale(obj, [src] + headers + [__file__]):
            jobs.append([nvcc(), *ARCH, *fl, *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4) or 1) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd[-3:]) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                failed.append(cmd[-3])
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(failed))
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
