"""Config 2 shapes (displaced icosphere surface, long thin strand triangles) at test size:
LBVH+ and PLOC(10/25/100) bit-exact against the oracle, and sphere-ray traversal of each tree."""
import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from tests.gpu_util import build, stream
from tests.treecheck import check_tree

pytestmark = pytest.mark.gpu

MESHES = {
    "icosphere_l5": lambda: meshgen.icosphere(levels=5, seed=2),   # 20,480 triangles
    "strands_200x50": lambda: meshgen.strands(200, 50, seed=3),    # 10,000 thin triangles
}


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def meshes():
    return {k: f() for k, f in MESHES.items()}


def _trace_check(ctx, gpu, O, mesh, nodes, tree, mts):
    ro, rd = meshgen.sphere_rays(mesh, 8192, seed=5)
    rts = [gpu.from_numpy(np.ascontiguousarray(a)).cuda()
           for a in (ro[:, 0], ro[:, 1], ro[:, 2], rd[:, 0], rd[:, 1], rd[:, 2])]
    hts = [gpu.empty(ro.shape[0], dtype=gpu.float32, device="cuda")] + \
          [gpu.empty(ro.shape[0], dtype=gpu.int32, device="cuda") for _ in range(4)]
    ctx.trace(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], mesh.size(), [t.data_ptr() for t in rts],
              ro.shape[0], [h.data_ptr() for h in hts], stream(gpu))
    gpu.cuda.synchronize()
    got = [h.cpu().numpy() for h in hts]
    exp = O.trace(nodes, mesh.arrays(), ro, rd)
    assert np.array_equal(got[0].view(np.uint32), exp[0].view(np.uint32))
    for g, e in zip(got[1:], exp[1:]):
        assert np.array_equal(g, e)


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("radius", [10, 25, 100])
def test_ploc_c2(ctx, gpu, oracle_lib, meshes, name, radius):
    O = oracle_lib
    m = meshes[name]
    nodes, idx, tree, mts = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=radius))
    onodes, oidx, it, cs, rc = O.ploc(m.arrays(), radius)
    assert rc == 0 and np.array_equal(idx, oidx) and O.node_fields_equal(nodes, onodes)
    check_tree(nodes, m.size())
    _trace_check(ctx, gpu, O, m, nodes, tree, mts)


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("rounds", [1, 3])
def test_lbvh_plus_c2(ctx, gpu, oracle_lib, meshes, name, rounds):
    O = oracle_lib
    m = meshes[name]
    nodes, idx, tree, mts = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=rounds))
    onodes, oidx = O.lbvh_plus(m.arrays(), 60, rounds)
    assert np.array_equal(idx, oidx) and O.node_fields_equal(nodes, onodes)
    _trace_check(ctx, gpu, O, m, nodes, tree, mts)


@pytest.mark.parametrize("name", list(MESHES))
def test_plus_and_ploc_not_worse_than_lbvh(ctx, gpu, oracle_lib, meshes, name):
    """Quality ordering the reference reports (README.md:348-352): restructured trees score a
    lower SAH than the plain LBVH on these surfaces."""
    O = oracle_lib
    m = meshes[name]
    sah = {}
    for label, p in (("lbvh", ctx.params(C.ALGO_LBVH, morton_bits=60)),
                     ("plus", ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=3)),
                     ("ploc", ctx.params(C.ALGO_PLOC, ploc_radius=25))):
        nodes, _, _, _ = build(ctx, gpu, m, p)
        sah[label] = O.sah(nodes)
    assert sah["plus"] < sah["lbvh"]
