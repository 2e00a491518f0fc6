"""GPU parity of PLOC and LBVH+ against the CPU oracle and the reference's own kernels."""
import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from tests import meshes
from tests.gpu_util import build
from tests.treecheck import check_tree

pytestmark = pytest.mark.gpu

CASES = meshes.small_cases()


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


def _runner():
    from oracle import ref
    if not ref.runner_available():
        pytest.skip("reference fatbins not present")
    return ref.RefRunner()


@pytest.mark.parametrize("radius", [1, 10, 25, 100])
@pytest.mark.parametrize("name", ["uniform1", "uniform2", "uniform3", "uniform17", "uniform257", "uniform4097",
                                  "identical100", "flat2000", "clumped5000", "negscaled3000", "clustered20000"])
def test_ploc_bit_exact_vs_oracle(ctx, gpu, oracle_lib, name, radius):
    O = oracle_lib
    m = CASES[name]
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=radius))
    onodes, oidx, it, cs, rc = O.ploc(m.arrays(), radius)
    assert rc == 0
    assert np.array_equal(idx, oidx)
    assert O.node_fields_equal(nodes, onodes)
    t = ctx.last_timing()
    assert t.ploc_iterations == it and t.ploc_cluster_sum == cs


@pytest.mark.parametrize("name", ["uniform17", "uniform4097", "clumped5000", "clustered20000"])
def test_ploc_canonical_vs_reference_kernels(ctx, gpu, name):
    from oracle import oracle as O
    m = CASES[name]
    rn, ri, rit, _, rc = _runner().ploc(m.arrays(), 25)
    assert rc == 0
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=25))
    assert np.array_equal(idx, ri)
    assert O.canonical_equal(nodes, rn)
    assert ctx.last_timing().ploc_iterations == rit


@pytest.mark.parametrize("radius", [1, 25, 100])
@pytest.mark.parametrize("name", ["uniform3", "uniform4097", "clumped5000", "clustered20000"])
def test_ploc_host_driven_loop_equals_graph_loop(ctx, gpu, oracle_lib, name, radius):
    m = CASES[name]
    g_nodes, g_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=radius))
    g_it = ctx.last_timing().ploc_iterations
    h_nodes, h_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=radius, host_loops=True))
    t = ctx.last_timing()
    assert np.array_equal(g_idx, h_idx)
    assert oracle_lib.node_fields_equal(g_nodes, h_nodes)
    assert t.ploc_iterations == g_it


@pytest.mark.parametrize("rounds", [1, 3])
@pytest.mark.parametrize("name", ["uniform17", "uniform4097", "clustered20000"])
def test_lbvh_plus_host_driven_loop_equals_graph_loop(ctx, gpu, oracle_lib, name, rounds):
    m = CASES[name]
    p = dict(morton_bits=60, treelet_rounds=rounds)
    g_nodes, g_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, **p))
    h_nodes, h_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, host_loops=True, **p))
    assert np.array_equal(g_idx, h_idx)
    assert oracle_lib.node_fields_equal(g_nodes, h_nodes)


def test_ploc_nan_mesh_reports_no_progress(ctx, gpu):
    m = meshgen.uniform_small(64, seed=1)
    for a in m.arrays():
        a[:] = np.nan
    for host_loop in (False, True):
        with pytest.raises(C.BVHError) as e:
            ctx.build_host(m, ctx.params(C.ALGO_PLOC, ploc_radius=4, host_loops=host_loop))
        assert e.value.status == C.BVH_ERR_NO_PROGRESS


@pytest.mark.parametrize("rounds", [1, 3])
@pytest.mark.parametrize("name", ["uniform2", "uniform3", "uniform5", "uniform17", "uniform257", "uniform4097",
                                  "identical100", "flat2000", "clumped5000", "clustered20000"])
def test_lbvh_plus_bit_exact_vs_oracle(ctx, gpu, oracle_lib, name, rounds):
    O = oracle_lib
    m = CASES[name]
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=rounds))
    onodes, oidx = O.lbvh_plus(m.arrays(), 60, rounds)
    assert np.array_equal(idx, oidx)
    assert O.node_fields_equal(nodes, onodes)
    boxes, _ = O.tri_bounds(m.arrays())
    check_tree(nodes, m.size(), boxes)


@pytest.mark.parametrize("name", ["uniform17", "uniform4097", "clumped5000", "clustered20000"])
def test_lbvh_plus_bit_exact_vs_reference_kernels(ctx, gpu, name):
    from oracle import oracle as O
    m = CASES[name]
    rn, ri, _ = _runner().lbvh_plus(m.arrays())
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=1))
    assert np.array_equal(idx, ri)
    assert O.node_fields_equal(nodes, rn)


@pytest.mark.parametrize("rounds", [1, 3])
def test_lbvh_plus_with_nan_triangles_equals_oracle(ctx, gpu, oracle_lib, rounds):
    """Treelets whose root box has a NaN area are not grown (growth expands only areas above -1),
    so those subtrees keep their shape; the rest are restructured as usual.  One triangle in 50
    carries a NaN coordinate, so NaN boxes appear at every height, height 1 included."""
    O = oracle_lib
    m = meshgen.clustered(60_000, seed=91)
    arrs = [np.array(a, copy=True) for a in m.arrays()]
    rng = np.random.default_rng(5)
    bad = rng.choice(m.size(), m.size() // 50, replace=False)
    for k, idx in enumerate(np.array_split(bad, 9)):
        arrs[k][idx] = np.nan
    mesh = type(m)(*arrs)
    nodes, idx, _, _ = build(ctx, gpu, mesh, ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=rounds))
    onodes, oidx = O.lbvh_plus(mesh.arrays(), 60, rounds)
    assert np.array_equal(idx, oidx)
    assert O.node_fields_equal(nodes, onodes)
