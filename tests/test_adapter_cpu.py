"""The C++ BVHBuilder adapters compile and link as a reference caller would use them: standalone,
and against the reference's own headers with its evaluator (where the reference sources are
present).  Without a GPU the program must report the error, not crash."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "bvh_gb300")
from oracle.ref_build import REF_ROOT as REF  # the reference tree the build recipe reads (skip if absent)


def _build_and_run(tmp_path, flags, sources=()):
    if not os.path.exists(os.path.join(LIBDIR, "libbvh_gb300.so")):
        from bvh_gb300 import build
        build.build_library()
    exe = str(tmp_path / "adapter_main")
    cmd = (["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include"]
           + list(flags) + [os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp")] + list(sources)
           + ["-L" + LIBDIR, "-lbvh_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return subprocess.run([exe, "2000"], capture_output=True, text=True, timeout=120)


def _check(p):
    from tests.conftest import has_gpu
    if has_gpu():
        assert p.returncode == 0, p.stdout + p.stderr
        assert p.stdout.count("nodes=") == 3
    else:
        assert p.returncode == 1, (p.returncode, p.stdout, p.stderr)  # an error, not a signal
        assert "error" in p.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_adapters_standalone(tmp_path):
    _check(_build_and_run(tmp_path, ["-DBVH_GB300_STANDALONE"]))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include")), reason="reference sources absent")
def test_adapters_against_reference_headers_and_evaluator(tmp_path):
    _check(_build_and_run(tmp_path, ["-I" + os.path.join(REF, "include")], [os.path.join(REF, "src", "evaluator.cpp")]))
