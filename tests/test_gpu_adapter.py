"""The C++ BVHBuilder adapters (include/bvh_gb300_builder.hpp) on the GPU: a C++ program builds a
mesh through Gb300LBVHBuilder, Gb300LBVHPlusBuilder and Gb300PLOCBuilder(25) -- the classes a
reference caller substitutes for LBVHBuilderCUDA, LBVHPlusBuilderCUDA and PLOCBuilderCUDA --
and prints a hash of each tree's node fields.  The hashes must equal those of the same builds
through the Python path, and the LBVH+ and PLOC trees must equal the oracle's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "bvh_gb300")


def _hash(nodes) -> str:
    """FNV-1a over min xyz, max xyz, left, right of every node (as adapter_main.cpp computes it)."""
    rec = np.zeros((nodes.shape[0], 32), np.uint8)
    rec[:, 0:12] = nodes["min"].astype(np.float32).view(np.uint8).reshape(-1, 12)
    rec[:, 12:24] = nodes["max"].astype(np.float32).view(np.uint8).reshape(-1, 12)
    rec[:, 24:28] = nodes["left"].astype(np.int32).view(np.uint8).reshape(-1, 4)
    rec[:, 28:32] = nodes["right"].astype(np.int32).view(np.uint8).reshape(-1, 4)
    h = 1469598103934665603
    for b in rec.reshape(-1).tobytes():
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_cpp_adapters_build_on_the_gpu(gpu, oracle_lib, tmp_path):
    m = meshgen.clustered(3000, seed=61)
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as f:
        for a in m.arrays():
            f.write(np.ascontiguousarray(a, np.float32).tobytes())
    exe = str(tmp_path / "adapter_main")
    cmd = ["g++", "-std=c++17", "-O1", "-DBVH_GB300_STANDALONE", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp"), "-L" + LIBDIR, "-lbvh_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    p = subprocess.run([exe, str(path)], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    got = {}
    for line in p.stdout.splitlines():
        name = line.split(" nodes=")[0]
        fields = dict(kv.split("=") for kv in line.split()[-3:])
        got[name] = (int(fields["nodes"]), fields["hash"])
    ctx = Context(0)
    cases = {"LBVH": ctx.params(C.ALGO_LBVH), "LBVH+": ctx.params(C.ALGO_LBVH_PLUS),
             "PLOC CUDA (r=25)": ctx.params(C.ALGO_PLOC, ploc_radius=25)}
    for name, params in cases.items():
        nodes, idx = ctx.build_host(m, params)
        assert got[name] == (nodes.shape[0], _hash(nodes)), name
        if name == "LBVH+":
            on, _ = oracle_lib.lbvh_plus(m.arrays(), 60, 1)
            assert oracle_lib.node_fields_equal(nodes, on)
        elif name.startswith("PLOC"):
            on, _, _, _, rc = oracle_lib.ploc(m.arrays(), 25)
            assert rc == 0 and oracle_lib.node_fields_equal(nodes, on)
        else:
            on, _, _ = oracle_lib.lbvh(m.arrays(), 30)
            assert oracle_lib.node_fields_equal(nodes, on)
    ctx.close()
