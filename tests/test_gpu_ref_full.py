"""Parity with the reference's own builders at the configurations' full sizes.

The reference kernels (its unmodified .cu files, default flags, replayed in their host order by
oracle/ref_runner.cu) and this library build the same mesh:
  c1  10,000,000 triangles in 64 Gaussian clusters;
  c2a the 1,310,720-triangle icosphere with fBm displacement;
  c2b 2,000,000 thin strand triangles.
LBVH (30-bit) and LBVH+ (60-bit codes, one treelet pass) must be bit-exact: indices and every
node's min, max, left and right.  PLOC must be canonically equal (same tree read from the root,
children in order, same leaf primitives and boxes).  The reference numbers its PLOC nodes with
atomicAdd, so only that form can compare.  Its iteration count must also agree.
"""
import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from tests.gpu_util import build

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def R(gpu):
    from oracle import ref
    if not ref.runner_available():
        pytest.skip("reference fatbins not present")
    return ref.RefRunner()


_MESHES = {}


def _mesh(name):
    if name not in _MESHES:
        _MESHES.clear()  # hold one full-size mesh at a time
        _MESHES[name] = {"c1": lambda: meshgen.clustered(10_000_000, seed=1),
                         "c2a": lambda: meshgen.icosphere(8, seed=2),
                         "c2b": lambda: meshgen.strands(seed=3)}[name]()
    return _MESHES[name]


def _diff_report(nodes, rn, idx, ri):
    """Counts of differing indices and node fields (for the failure message)."""
    if nodes.shape != rn.shape:
        return {"node_count": (nodes.shape[0], rn.shape[0])}
    return {"indices": int((idx != ri).sum()),
            "min": int((nodes["min"].view(np.uint32) != rn["min"].view(np.uint32)).any(axis=1).sum()),
            "max": int((nodes["max"].view(np.uint32) != rn["max"].view(np.uint32)).any(axis=1).sum()),
            "left": int((nodes["left"] != rn["left"]).sum()), "right": int((nodes["right"] != rn["right"]).sum())}


@pytest.mark.parametrize("name", ["c1", "c2a", "c2b"])
def test_lbvh30_bit_exact_vs_reference_full_size(ctx, gpu, R, oracle_lib, name):
    m = _mesh(name)
    rn, ri, _ = R.lbvh(m.arrays())
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=30))
    ok = np.array_equal(idx, ri) and oracle_lib.node_fields_equal(nodes, rn)
    assert ok, _diff_report(nodes, rn, idx, ri)


@pytest.mark.parametrize("name", ["c1", "c2a", "c2b"])
def test_lbvh_plus_bit_exact_vs_reference_full_size(ctx, gpu, R, oracle_lib, name):
    m = _mesh(name)
    rn, ri, _ = R.lbvh_plus(m.arrays())
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH_PLUS, morton_bits=60, treelet_rounds=1))
    ok = np.array_equal(idx, ri) and oracle_lib.node_fields_equal(nodes, rn)
    if not ok:  # is the reference itself repeatable on this mesh?
        rn2, ri2, _ = R.lbvh_plus(m.arrays())
        pytest.fail(f"vs reference {_diff_report(nodes, rn, idx, ri)}; reference run twice "
                    f"{_diff_report(rn2, rn, ri2, ri)}")


@pytest.mark.parametrize("name,radius", [("c1", 25), ("c2a", 10), ("c2a", 25), ("c2a", 100), ("c2b", 10),
                                         ("c2b", 25), ("c2b", 100)])
def test_ploc_canonical_vs_reference_full_size(ctx, gpu, R, oracle_lib, name, radius):
    m = _mesh(name)
    rn, ri, rit, _, rc = R.ploc(m.arrays(), radius, max_iter=100_000)
    assert rc == 0
    nodes, idx, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_PLOC, ploc_radius=radius))
    assert np.array_equal(idx, ri)
    assert oracle_lib.canonical_equal(nodes, rn)
    assert ctx.last_timing().ploc_iterations == rit
