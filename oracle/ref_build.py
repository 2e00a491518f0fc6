"""Build recipe for oracle/_ref/ (TEST INFRASTRUCTURE; outputs stay out of git).

* With the reference sources present (REF_ROOT, default /root/reference):
  - ref_{lbvh,lbvh_plus,ploc,render}.fatbin: the reference's own .cu files, unmodified, compiled
    to sm_103a device code with the reference's default (non-Release) flags; *_fast.fatbin with
    its Release flags (-O3 --use_fast_math, CMakeLists.txt:41-45).
  - libref_eval.so: the reference's src/evaluator.cpp with ref_eval_shim.cpp (host only).
  - libref_loader.so: the reference's src/loader.cpp with ref_loader_shim.cpp (host only).
  - libref_render_host.so: the reference's src/render_engine.cu, included by ref_render_shim.cu,
    for its host post-processing (heatmap colormap, PPM bytes); used by CPU tests only.
  - ref_trace.fatbin: the reference's src/render_engine.cu, included by ref_trace_shim.cu, whose
    two kernels run the reference's generateRay and traverseBVH on given rays (default flags).
* Anywhere (GPU machines included): libref_runner.so from ref_runner.cu (our host code that loads the
  fatbins and replays the reference builders with CUB/Thrust).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("REF_ROOT", "/root/reference")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FATBINS = {
    "ref_lbvh": "src/cuda/lbvh_builder.cu",
    "ref_lbvh_plus": "src/cuda/lbvh_plus_builder.cu",
    "ref_ploc": "src/cuda/ploc_builder.cu",
    "ref_render": "src/render_engine.cu",
}


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)


def _fresh(out, *inputs):
    """True when `out` exists and is newer than every input (then its build step is skipped)."""
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(i) <= t for i in inputs if os.path.exists(i))


def have_reference() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, "src", "cuda"))


def build_fatbins():
    jobs = []
    inc = ["-I" + os.path.join(REF_ROOT, "include")]
    for name, rel in FATBINS.items():
        src = os.path.join(REF_ROOT, rel)
        out, out_fast = os.path.join(OUT, name + ".fatbin"), os.path.join(OUT, name + "_fast.fatbin")
        if not _fresh(out, src):
            jobs.append([_nvcc(), "-fatbin"] + ARCH + ["-std=c++17"] + inc + [src, "-o", out])
        if not _fresh(out_fast, src):
            jobs.append([_nvcc(), "-fatbin"] + ARCH + ["-std=c++17", "-O3", "--use_fast_math"] + inc
                        + [src, "-o", out_fast])
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))


def build_eval():
    if _fresh(os.path.join(OUT, "libref_eval.so"), os.path.join(HERE, "ref_eval_shim.cpp"),
              os.path.join(REF_ROOT, "src", "evaluator.cpp")):
        return
    _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
          "-I" + os.path.join(REF_ROOT, "include"), "-I/usr/local/cuda/include",
          os.path.join(HERE, "ref_eval_shim.cpp"), os.path.join(REF_ROOT, "src", "evaluator.cpp"),
          "-o", os.path.join(OUT, "libref_eval.so")])


def build_loader():
    if _fresh(os.path.join(OUT, "libref_loader.so"), os.path.join(HERE, "ref_loader_shim.cpp"),
              os.path.join(REF_ROOT, "src", "loader.cpp")):
        return
    _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC",
          "-I" + os.path.join(REF_ROOT, "include"), "-I/usr/local/cuda/include",
          os.path.join(HERE, "ref_loader_shim.cpp"), os.path.join(REF_ROOT, "src", "loader.cpp"),
          "-o", os.path.join(OUT, "libref_loader.so")])


def build_render_host():
    if _fresh(os.path.join(OUT, "libref_render_host.so"), os.path.join(HERE, "ref_render_shim.cu"),
              os.path.join(REF_ROOT, "src", "render_engine.cu")):
        return
    _run([_nvcc()] + ARCH + ["-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off",
                             "-I" + os.path.join(REF_ROOT, "include"), "-I" + os.path.join(REF_ROOT, "src"),
                             os.path.join(HERE, "ref_render_shim.cu"),
                             "-o", os.path.join(OUT, "libref_render_host.so")])


def build_trace_shim():
    out = os.path.join(OUT, "ref_trace.fatbin")
    shim = os.path.join(HERE, "ref_trace_shim.cu")
    if _fresh(out, shim, os.path.join(REF_ROOT, "src", "render_engine.cu")):
        return
    _run([_nvcc(), "-fatbin"] + ARCH + ["-std=c++17", "-I" + os.path.join(REF_ROOT, "include"),
                                        "-I" + os.path.join(REF_ROOT, "src"), shim, "-o", out])


def build_runner():
    if _fresh(os.path.join(OUT, "libref_runner.so"), os.path.join(HERE, "ref_runner.cu")):
        return
    _run([_nvcc()] + ARCH + ["-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                             os.path.join(HERE, "ref_runner.cu"), "-o", os.path.join(OUT, "libref_runner.so"),
                             "-lcuda"])


def fatbins_present() -> bool:
    return all(os.path.exists(os.path.join(OUT, n + ".fatbin")) for n in FATBINS)


def build(runner: bool = True):
    os.makedirs(OUT, exist_ok=True)
    if have_reference():
        build_fatbins()
        build_eval()
        build_loader()
        build_render_host()
        build_trace_shim()
    if runner and fatbins_present():
        build_runner()


if __name__ == "__main__":
    build(runner="--no-runner" not in sys.argv)
