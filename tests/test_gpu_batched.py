"""Batched builds (LBVH-30 and PLOC): every mesh's part equals its standalone build, bit for bit."""
import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from bvh_gb300.builders import TriangleMesh
from tests.gpu_util import build, to_device, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


def _sub(mesh, a, b):
    return TriangleMesh(*[x[a:b] for x in mesh.arrays()])


def _check_batch(ctx, gpu, mesh, offsets, use_graph=False, repeats=1, oracle=None, algo=C.ALGO_LBVH, radius=25,
                 host_loops=False):
    ts, ptrs = to_device(gpu, mesh.arrays())
    p = ctx.params(algo, ploc_radius=radius, host_loops=host_loops)
    for _ in range(repeats):
        tree = ctx.build_batched(ptrs, offsets, p, stream(gpu), use_graph=use_graph)
    ctx.sync()
    iters = ctx.last_timing().ploc_iterations
    nodes, idx = ctx.download(tree, stream(gpu))
    count = offsets.shape[0] - 1
    assert nodes.shape[0] == 2 * int(offsets[-1]) - count
    single = Context(0)
    most = 0
    for m in range(count):
        a, b = int(offsets[m]), int(offsets[m + 1])
        sub = _sub(mesh, a, b)
        sn, si, _, _ = build(single, gpu, sub, single.params(algo, ploc_radius=radius))
        if algo == C.ALGO_PLOC:
            most = max(most, single.last_timing().ploc_iterations)
        nb = 2 * a - m
        part = nodes[nb: nb + 2 * (b - a) - 1]
        assert np.array_equal(idx[a:b], si), m
        from oracle import oracle as O
        assert O.node_fields_equal(part, sn), m
        if oracle is not None and m % 7 == 0:
            if algo == C.ALGO_PLOC:
                on, oi, _, _, rc = oracle.ploc(sub.arrays(), radius)
                assert rc == 0
            else:
                on, oi, _ = oracle.lbvh(sub.arrays(), 30)
            assert np.array_equal(oi, si) and oracle.node_fields_equal(on, sn)
    single.close()
    if algo == C.ALGO_PLOC:
        assert iters == most  # the batch iterates as long as its slowest mesh


def test_batched_small_meshes(ctx, gpu, oracle_lib):
    counts = [1, 2, 3, 1, 64, 257, 1000, 5, 3073, 2, 1, 4096, 17]
    mesh, offsets = meshgen.batch(counts, seed=11)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib)


def test_batched_log_uniform(ctx, gpu, oracle_lib):
    counts = meshgen.batch_counts(200, 64, 20000, seed=12)
    mesh, offsets = meshgen.batch(counts, seed=13)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib)


def test_batched_few_meshes_whole_key_sort(ctx, gpu, oracle_lib):
    """At most 4 meshes: 32-bit keys, sorted whole (no run fix-up)."""
    mesh, offsets = meshgen.batch([3000, 17, 4097, 1], seed=16)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib)


def test_batched_long_runs(ctx, gpu, oracle_lib):
    """Meshes of identical triangles: runs of equal high key bits longer than 64 (the fix-up's
    block-wide path) inside a batch of 10 meshes."""
    from tests import meshes as M
    parts = [M.identical(3000), meshgen.uniform_small(2000, seed=3), M.identical(70), M.dense_cell(5000)]
    parts += [meshgen.uniform_small(100 + 37 * k, seed=20 + k) for k in range(6)]
    arrays = [np.concatenate([p.arrays()[k] for p in parts]) for k in range(9)]
    mesh = TriangleMesh(*arrays)
    offsets = np.concatenate([[0], np.cumsum([p.size() for p in parts])]).astype(np.int64)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib)


def test_batched_graph_replay(ctx, gpu):
    counts = meshgen.batch_counts(100, 64, 8000, seed=14)
    mesh, offsets = meshgen.batch(counts, seed=15)
    _check_batch(ctx, gpu, mesh, offsets, use_graph=True, repeats=3)


def test_batched_rejects_bad_offsets(ctx, gpu):
    mesh, offsets = meshgen.batch([10, 20], seed=1)
    ts, ptrs = to_device(gpu, mesh.arrays())
    bad = offsets.copy()
    bad[1] = bad[0]  # empty mesh
    with pytest.raises(C.BVHError):
        ctx.build_batched(ptrs, bad, ctx.params(C.ALGO_LBVH), stream(gpu))
    with pytest.raises(C.BVHError) as e:  # LBVH+ is not batched
        ctx.build_batched(ptrs, offsets, ctx.params(C.ALGO_LBVH_PLUS), stream(gpu))
    assert e.value.status == C.BVH_ERR_UNSUPPORTED
    with pytest.raises(C.BVHError):  # 63-bit codes are not batched
        ctx.build_batched(ptrs, offsets, ctx.params(C.ALGO_LBVH, morton_bits=63), stream(gpu))


@pytest.mark.parametrize("radius", [1, 10, 25, 100])
def test_batched_ploc_small_meshes(ctx, gpu, oracle_lib, radius):
    """Meshes of 1, 2 and 3 triangles, tile-boundary sizes and meshes smaller than the window,
    side by side: every window is clipped at its mesh, every mesh numbered on its own."""
    counts = [1, 2, 3, 1, 64, 257, 1000, 5, 3073, 2, 1, 4096, 17]
    mesh, offsets = meshgen.batch(counts, seed=21)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib, algo=C.ALGO_PLOC, radius=radius)


def test_batched_ploc_log_uniform(ctx, gpu, oracle_lib):
    counts = meshgen.batch_counts(200, 64, 20000, seed=22)
    mesh, offsets = meshgen.batch(counts, seed=23)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib, algo=C.ALGO_PLOC, radius=25)


def test_batched_ploc_long_runs_and_clusters(ctx, gpu, oracle_lib):
    from tests import meshes as M
    parts = [M.identical(3000), meshgen.clustered(20000, seed=4), M.identical(70), M.dense_cell(5000)]
    parts += [meshgen.uniform_small(100 + 37 * k, seed=20 + k) for k in range(6)]
    arrays = [np.concatenate([p.arrays()[k] for p in parts]) for k in range(9)]
    mesh = TriangleMesh(*arrays)
    offsets = np.concatenate([[0], np.cumsum([p.size() for p in parts])]).astype(np.int64)
    _check_batch(ctx, gpu, mesh, offsets, oracle=oracle_lib, algo=C.ALGO_PLOC, radius=10)


@pytest.mark.parametrize("host_loops", [False, True])
def test_batched_ploc_graph_and_host_loop(ctx, gpu, host_loops):
    """The whole batch as one replayed graph (the clustering loop a conditional node inside it),
    three times in a row; and the same kernels driven from a host loop."""
    counts = meshgen.batch_counts(100, 64, 8000, seed=24)
    mesh, offsets = meshgen.batch(counts, seed=25)
    _check_batch(ctx, gpu, mesh, offsets, use_graph=not host_loops, repeats=3, algo=C.ALGO_PLOC, radius=25,
                 host_loops=host_loops)


def test_batched_ploc_then_lbvh_on_one_context(ctx, gpu):
    """Alternating algorithms on one context rebuilds the cached graph each time."""
    counts = meshgen.batch_counts(40, 64, 3000, seed=26)
    mesh, offsets = meshgen.batch(counts, seed=27)
    for algo in (C.ALGO_PLOC, C.ALGO_LBVH, C.ALGO_PLOC):
        _check_batch(ctx, gpu, mesh, offsets, use_graph=True, repeats=2, algo=algo, radius=25)


def test_batched_ploc_nan_mesh_reports_no_progress(ctx, gpu):
    mesh, offsets = meshgen.batch([50, 64, 30], seed=28)
    arrs = [a.copy() for a in mesh.arrays()]
    for a in arrs:
        a[50:114] = np.nan  # the middle mesh has no finite area
    ts, ptrs = to_device(gpu, arrs)
    ctx.build_batched(ptrs, offsets, ctx.params(C.ALGO_PLOC, ploc_radius=4), stream(gpu))
    with pytest.raises(C.BVHError) as e:
        ctx.sync()
    assert e.value.status == C.BVH_ERR_NO_PROGRESS
