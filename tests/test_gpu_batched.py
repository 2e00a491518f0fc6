"""Batched builds: every mesh's part equals its standalone build, bit for bit."""
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


def _check_batch(ctx, gpu, mesh, offsets, use_graph=False, repeats=1, oracle=None):
    ts, ptrs = to_device(gpu, mesh.arrays())
    p = ctx.params(C.ALGO_LBVH)
    for _ in range(repeats):
        tree = ctx.build_batched(ptrs, offsets, p, stream(gpu), use_graph=use_graph)
    ctx.sync()
    nodes, idx = ctx.download(tree, stream(gpu))
    count = offsets.shape[0] - 1
    assert nodes.shape[0] == 2 * int(offsets[-1]) - count
    single = Context(0)
    for m in range(count):
        a, b = int(offsets[m]), int(offsets[m + 1])
        sub = _sub(mesh, a, b)
        sn, si, _, _ = build(single, gpu, sub, single.params(C.ALGO_LBVH))
        nb = 2 * a - m
        part = nodes[nb: nb + 2 * (b - a) - 1]
        assert np.array_equal(idx[a:b], si), m
        from oracle import oracle as O
        assert O.node_fields_equal(part, sn), m
        if oracle is not None and m % 7 == 0:
            on, oi, _ = oracle.lbvh(sub.arrays(), 30)
            assert np.array_equal(oi, si) and oracle.node_fields_equal(on, sn)
    single.close()


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
    with pytest.raises(C.BVHError):
        ctx.build_batched(ptrs, offsets, ctx.params(C.ALGO_PLOC), stream(gpu))
