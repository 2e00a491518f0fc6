"""The CUDA path against the committed golden fixtures: the reference's own kernels' outputs on
seeded meshes (tests/golden/make_golden.py).  Bit-exact node fields and indices for LBVH-30 and
LBVH+-60; canonical tree equality for PLOC, whose reference node ids come from atomicAdd."""
import glob
import os

import numpy as np
import pytest

from bvh_gb300 import Context, TriangleMesh, _capi as C
from tests.gpu_util import build

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))), ids=os.path.basename)
def test_cuda_path_matches_reference_golden(ctx, gpu, oracle_lib, path):
    O = oracle_lib
    g = np.load(path)
    mesh = TriangleMesh(*[g[f"v{k}"] for k in range(9)])
    kind = str(g["kind"])
    ref_nodes = g["nodes"].view(C.NODE_DTYPE).reshape(-1)
    if kind == "lbvh30":
        params = ctx.params(C.ALGO_LBVH, morton_bits=30)
    elif kind == "lbvh_plus60":
        params = ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=1)
    elif kind.startswith("ploc"):
        params = ctx.params(C.ALGO_PLOC, ploc_radius=int(g["radius"]))
    else:
        pytest.skip(f"unknown golden kind {kind}")
    nodes, idx, _, _ = build(ctx, gpu, mesh, params)
    assert np.array_equal(idx, g["indices"])
    if kind.startswith("ploc"):
        assert O.canonical_equal(nodes, ref_nodes)
    else:
        assert O.node_fields_equal(nodes, ref_nodes)
