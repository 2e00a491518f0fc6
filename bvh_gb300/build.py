"""Compile libbvh_gb300.so in-tree for sm_103a with nvcc (no CMake).

Translation units are compiled in parallel and linked into bvh_gb300/libbvh_gb300.so.
Device arithmetic is compiled with -fmad=false and host code with -ffp-contract=off, so every
float operation rounds as written (the kernels use explicit FMAs where the reference's
compiled code has them).  trace.cu is the exception: it keeps nvcc's default -fmad=true so that
the device tanf it calls (generateRay's tan(fov/2)) is compiled as the reference's is; every
float operation written in that file is an explicitly rounded intrinsic, which is never fused.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libbvh_gb300.so")
OBJ_DIR = os.path.join(HERE, "_build")

SOURCES = ["lbvh.cu", "treelet.cu", "ploc.cu", "trace.cu", "batched.cu", "capi.cu", "noalloc.cu", "serve.cu", "evaluate.cu", "fixrun.cu", "objload.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "--expt-relaxed-constexpr"]
FMAD = {"trace.cu": "-fmad=true"}  # every other translation unit: -fmad=false


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + [FMAD.get(src, "-fmad=false")] + list(extra) + ["-c", os.path.join(CSRC, src),
                                                                                         "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(objs) -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "bvh_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_library(force: bool = False, extra=(), verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    if not force and not _stale(SOURCES):
        return OUT
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = OUT + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    if verbose:
        print(f"built {OUT}")
    return OUT


def ptxas_report(src: str = "lbvh.cu") -> str:
    """Registers / spills / shared memory per kernel (-Xptxas -v)."""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + [FMAD.get(src, "-fmad=false"), "-Xptxas", "-v", "-c", os.path.join(CSRC, src),
                                          "-o", os.devnull]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
