"""Builds without cooperative kernels give the trees of the default path.

PLOC's middle iterations (k_ploc_grid) and LBVH+'s narrow tree heights (k_tl_narrow) are
cooperative launches with grid barriers.  When the device refuses such a launch (a client limited
to part of the GPU) a build runs the same work as one launch per kernel and iteration or height,
driven from the host; BVH_NO_COOPERATIVE takes that path on purpose, and these tests check it
against the oracle and against the cooperative path.
"""
import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from tests.gpu_util import build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("n,radius", [(70_000, 25), (150_000, 8), (150_000, 100)])
def test_ploc_without_cooperative_kernel_equals_oracle(ctx, gpu, oracle_lib, n, radius):
    m = meshgen.clustered(n, seed=n + radius)
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=radius, no_cooperative=True))
    t = ctx.last_timing()
    onodes, oidx, it, cs, rc = oracle_lib.ploc(m.arrays(), radius)
    assert rc == 0
    assert np.array_equal(idx, oidx)
    assert oracle_lib.node_fields_equal(nodes, onodes)
    assert t.ploc_iterations == it and t.ploc_cluster_sum == cs


@pytest.mark.parametrize("host_loops", [False, True])
def test_ploc_without_cooperative_kernel_equals_cooperative_2m(ctx, gpu, oracle_lib, host_loops):
    """2M triangles: the loop hands over to the middle iterations part-way, so the fallback starts
    from a state the graph (or host) loop left."""
    m = meshgen.clustered(2_000_000, seed=17)
    p = dict(ploc_radius=25, host_loops=host_loops)
    a_nodes, a_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, **p))
    ta = ctx.last_timing()
    b_nodes, b_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, no_cooperative=True, **p))
    tb = ctx.last_timing()
    assert np.array_equal(a_idx, b_idx)
    assert oracle_lib.node_fields_equal(a_nodes, b_nodes)
    assert ta.ploc_iterations == tb.ploc_iterations and ta.ploc_cluster_sum == tb.ploc_cluster_sum
    # every iteration of the fallback is its own four launches
    assert tb.kernel_launches > ta.kernel_launches


@pytest.mark.parametrize("rounds", [1, 3])
def test_lbvh_plus_without_cooperative_kernel_equals_oracle(ctx, gpu, oracle_lib, rounds):
    m = meshgen.clustered(60_000, seed=23)
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=rounds,
                                                     no_cooperative=True))
    onodes, oidx = oracle_lib.lbvh_plus(m.arrays(), 60, rounds)
    assert np.array_equal(idx, oidx)
    assert oracle_lib.node_fields_equal(nodes, onodes)


def test_lbvh_plus_without_cooperative_kernel_equals_cooperative_2m(ctx, gpu, oracle_lib):
    m = meshgen.clustered(2_000_000, seed=29)
    p = dict(morton_bits=60, treelet_rounds=2)
    a_nodes, a_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, **p))
    ta = ctx.last_timing()
    b_nodes, b_idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, no_cooperative=True, **p))
    tb = ctx.last_timing()
    assert np.array_equal(a_idx, b_idx)
    assert oracle_lib.node_fields_equal(a_nodes, b_nodes)
    assert tb.kernel_launches > ta.kernel_launches
