"""GPU parity of LBVH (30/60/63-bit) against the CPU oracle and the reference's own kernels."""
import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from tests import meshes
from tests.gpu_util import build, to_device, stream
from tests.treecheck import check_tree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


CASES = meshes.small_cases()


@pytest.mark.parametrize("bits", [30, 60, 63])
@pytest.mark.parametrize("name", list(CASES.keys()))
def test_lbvh_bit_exact_vs_oracle(ctx, gpu, oracle_lib, name, bits):
    O = oracle_lib
    m = CASES[name]
    nodes, idx, tree, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=bits))
    onodes, oidx, _ = O.lbvh(m.arrays(), bits)
    assert np.array_equal(idx, oidx)
    assert O.node_fields_equal(nodes, onodes)
    boxes, _ = O.tri_bounds(m.arrays())
    check_tree(nodes, m.size(), boxes)


@pytest.mark.parametrize("n,bits", [(100_000, 30), (1_000_003, 63), (1_000_000, 60)])
def test_lbvh_clustered_bit_exact(ctx, gpu, oracle_lib, n, bits):
    O = oracle_lib
    m = meshgen.clustered(n, seed=n) if bits != 30 else meshgen.uniform_small(n, seed=0)
    nodes, idx, tree, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=bits))
    onodes, oidx, _ = O.lbvh(m.arrays(), bits)
    assert np.array_equal(idx, oidx)
    assert O.node_fields_equal(nodes, onodes)


@pytest.mark.parametrize("bits", [60, 63])
@pytest.mark.parametrize("n,size", [(200_000, 1e-4), (300_000, 2e-3), (300_000, 2e-2)])
def test_lbvh_long_runs_across_tiles(ctx, gpu, oracle_lib, bits, n, size):
    """Runs of equal high code halves spanning many fix-up tiles (block-wide path) and many
    runs of a few dozen (shared-memory ranks), against the oracle's full-key sort."""
    m = meshes.dense_cell(n, size=size, spread=0.02, seed=n)
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=bits))
    onodes, oidx, _ = oracle_lib.lbvh(m.arrays(), bits)
    assert np.array_equal(idx, oidx)
    assert oracle_lib.node_fields_equal(nodes, onodes)


def test_lbvh_unaligned_input_takes_scalar_path(ctx, gpu, oracle_lib):
    O = oracle_lib
    m = meshgen.uniform_small(5000, seed=42)
    ts = [gpu.from_numpy(np.concatenate([[0.0], a]).astype(np.float32)).cuda() for a in m.arrays()]
    ptrs = [t.data_ptr() + 4 for t in ts]  # 4-byte aligned only
    tree = ctx.build_device(ptrs, m.size(), ctx.params(C.ALGO_LBVH), stream(gpu))
    ctx.sync()
    nodes, idx = ctx.download(tree, stream(gpu))
    onodes, oidx, _ = O.lbvh(m.arrays(), 30)
    assert np.array_equal(idx, oidx) and O.node_fields_equal(nodes, onodes)


@pytest.mark.parametrize("bits", [30, 60, 63])
@pytest.mark.parametrize("n", [2, 3, 257, 50_000, 2_000_000])
def test_host_path_equals_device_path(ctx, gpu, bits, n):
    """bvh_build_host copies the indices and the leaves out on a second stream while the build
    finishes; the result equals the device build's."""
    m = meshgen.clustered(n, seed=5)
    p = ctx.params(C.ALGO_LBVH, morton_bits=bits)
    hn, hi = ctx.build_host(m, p)
    dn, di, _, _ = build(ctx, gpu, m, p)
    assert np.array_equal(hi, di)
    assert np.array_equal(hn[["min", "max", "left", "right"]], dn[["min", "max", "left", "right"]])


def test_host_path_repeated_and_mixed(ctx, gpu, oracle_lib):
    """Host builds of shrinking and growing sizes, between device builds, against the oracle."""
    O = oracle_lib
    for n, bits in ((30000, 63), (300, 30), (30000, 30), (7, 63), (2, 30), (1, 63), (12000, 60)):
        m = meshgen.uniform_small(n, seed=200 + n)
        hn, hi = ctx.build_host(m, ctx.params(C.ALGO_LBVH, morton_bits=bits))
        onodes, oidx, _ = O.lbvh(m.arrays(), bits)
        assert np.array_equal(hi, oidx) and O.node_fields_equal(hn, onodes)
        build(ctx, gpu, meshgen.uniform_small(999, seed=n), ctx.params(C.ALGO_PLOC))


def test_repeated_builds_reuse_workspace(ctx, gpu, oracle_lib):
    """Builds of different sizes on one context (epoch-tagged rendezvous words, shrinking n)."""
    O = oracle_lib
    for n in (20000, 300, 20000, 7, 1):
        m = meshgen.uniform_small(n, seed=100 + n)
        nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
        onodes, oidx, _ = O.lbvh(m.arrays(), 30)
        assert np.array_equal(idx, oidx) and O.node_fields_equal(nodes, onodes)


def test_empty_mesh(ctx, gpu):
    m = meshgen.uniform_small(0)
    nodes, idx = ctx.build_host(m, ctx.params(C.ALGO_LBVH))
    assert nodes.shape[0] == 0 and idx.shape[0] == 0


def test_invalid_params_rejected(ctx, gpu):
    m = meshgen.uniform_small(10)
    p = ctx.params(C.ALGO_LBVH, morton_bits=31)
    with pytest.raises(C.BVHError):
        ctx.build_host(m, p)


def _runner():
    from oracle import ref
    if not ref.runner_available():
        pytest.skip("reference fatbins not present")
    return ref.RefRunner()


@pytest.mark.parametrize("name", ["uniform1", "uniform2", "uniform17", "uniform4097", "identical100", "flat2000",
                                  "clumped5000", "negscaled3000", "clustered20000"])
def test_lbvh30_bit_exact_vs_reference_kernels(ctx, gpu, name):
    m = CASES[name]
    R = _runner()
    rn, ri, _ = R.lbvh(m.arrays())
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
    from oracle import oracle as O
    assert np.array_equal(idx, ri)
    assert O.node_fields_equal(nodes, rn)


def test_lbvh30_c0_bit_exact_vs_reference_kernels(ctx, gpu):
    """Config 0: 100,000 triangles, seed 0."""
    m = meshgen.uniform_small(100_000, seed=0)
    R = _runner()
    rn, ri, _ = R.lbvh(m.arrays())
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
    from oracle import oracle as O
    assert np.array_equal(idx, ri)
    assert O.node_fields_equal(nodes, rn)


@pytest.mark.slow
def test_lbvh63_full_size_c1_bit_exact(ctx, gpu, oracle_lib):
    """Config 1 at full size: 10,000,000 clustered triangles, 63-bit Morton."""
    O = oracle_lib
    m = meshgen.clustered(10_000_000, seed=1)
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=63))
    onodes, oidx, _ = O.lbvh(m.arrays(), 63)
    assert np.array_equal(idx, oidx)
    assert O.node_fields_equal(nodes, onodes)
    assert O.sah(nodes) == O.sah(onodes)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4])
def test_every_sort_variant_bit_exact(ctx, gpu, oracle_lib, variant):
    O = oracle_lib
    ctx.set_tuning(variant)
    try:
        for bits, m in ((30, meshgen.uniform_small(70_001, seed=3)), (63, meshgen.clustered(90_007, seed=4))):
            nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=bits))
            onodes, oidx, _ = O.lbvh(m.arrays(), bits)
            assert np.array_equal(idx, oidx) and O.node_fields_equal(nodes, onodes)
    finally:
        ctx.set_tuning(0)


def test_autotune_table(ctx, gpu, oracle_lib):
    table = ctx.autotune(1 << 20)
    assert 0 <= table["sort"]["chosen"] < 5
    assert len(table["sort"]["variants"]) == 5 and all(v["ms"] > 0 for v in table["sort"]["variants"])
    assert ctx.tuning() == table["sort"]["chosen"]
    m = meshgen.clustered(50_000, seed=8)
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=63))
    onodes, oidx, _ = oracle_lib.lbvh(m.arrays(), 63)
    assert np.array_equal(idx, oidx) and oracle_lib.node_fields_equal(nodes, onodes)


def test_untuned_context_picks_sort_variant_by_size(gpu, oracle_lib):
    """Without bvh_tuning_set or an autotune, a build sorts with the variant its size calls for
    (8 keys per thread below 600k triangles, 24 keys from 2M) and still equals the oracle."""
    O = oracle_lib
    ctx = Context(0)
    try:
        for n, want in ((100_000, 3), (2_500_000, 2)):
            m = meshgen.clustered(n, seed=40 + n % 7)
            nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=63))
            assert ctx.tuning() == want
            onodes, oidx, _ = O.lbvh(m.arrays(), 63)
            assert np.array_equal(idx, oidx) and O.node_fields_equal(nodes, onodes)
        ctx.set_tuning(0)  # an explicit choice holds for every size
        m = meshgen.clustered(100_000, seed=43)
        build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=30))
        assert ctx.tuning() == 0
    finally:
        ctx.close()
