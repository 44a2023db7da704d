"""Build recipe for libffea_gb300.so (sm_103a), in-tree.

The translation units are compiled in parallel with nvcc and linked into one
shared library next to this file, against the CUDA runtime only.  No cmake, no torch extension machinery:
the library exposes only the C ABI of include/ffea_gpu.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libffea_gb300.so")
SOURCES = ["kernels.cu", "api.cu", "host_build.cpp", "noalloc.cu", "coarse.cu", "learned.cu", "ssint.cu",
           "script.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build ffea_gb300")


def _flags(src: str) -> list[str]:
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing", "-lineinfo"]
    if src.endswith("ssint.cu"):
        # products and sums round as in the reference's FP64 code (no FMA contraction)
        return common + ARCH + ["-Xptxas", "-O3", "-fmad=false"]
    if src.endswith(".cu"):
        return common + ARCH + ["-Xptxas", "-O3"]
    return common + ["-x", "cu"] + ARCH


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "ffea_gpu.h"))
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d)):
            return LIB
    cc = nvcc()
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s) + ".o")
        cmd = [cc, *_flags(s), "-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), s))
        objs.append(o)
    errors = []
    for p, s in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"{s}:\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    link = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
