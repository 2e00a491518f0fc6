"""CPU tests of the oracle: pinned against the reference's own evaluator and golden vectors."""
import glob
import os

import numpy as np
import pytest

from bvh_gb300 import meshgen
from tests import meshes
from tests.treecheck import check_tree

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_fmin_fmax_match_gpu_semantics(oracle_lib):
    O = oracle_lib
    L = O.lib()
    pz, nz = np.float32(0.0), np.float32(-0.0)
    # measured on the GB300: fminf(+0,-0) = fminf(-0,+0) = -0, fmaxf(...) = +0, NaN ignored
    assert np.signbit(L.orc_fmin(pz, nz)) and np.signbit(L.orc_fmin(nz, pz))
    assert not np.signbit(L.orc_fmax(pz, nz)) and not np.signbit(L.orc_fmax(nz, pz))
    assert L.orc_fmin(float("nan"), 1.0) == 1.0 and L.orc_fmax(1.0, float("nan")) == 1.0


def test_surface_area_form(oracle_lib):
    """2*(dx*dy+dy*dz+dz*dx) evaluated as 2*fma(dz,dx,fma(dx,dy,dy*dz)) (the reference's compiled form)."""
    O = oracle_lib
    box = np.zeros(1, O.AABB_DTYPE)[0]
    box["min"] = (0.1, 0.2, 0.3)
    box["max"] = (0.7, 1.3, 0.9)
    x, y, z = np.float32(0.7) - np.float32(0.1), np.float32(1.3) - np.float32(0.2), np.float32(0.9) - np.float32(0.3)
    import math
    inner = np.float32(math.fsum([float(x) * float(y), float(np.float32(y * z))]))
    outer = np.float32(math.fsum([float(z) * float(x), float(inner)]))
    assert O.sa(box) == np.float32(2.0) * outer


@pytest.mark.parametrize("name", list(meshes.small_cases().keys()))
def test_oracle_trees_are_valid(oracle_lib, name):
    O = oracle_lib
    m = meshes.small_cases()[name]
    boxes, _ = O.tri_bounds(m.arrays())
    for bits in (30, 60, 63):
        nodes, idx, keys = O.lbvh(m.arrays(), bits)
        check_tree(nodes, m.size(), boxes)
        assert np.all(np.diff(keys.astype(np.float64)) >= 0)
    nodes, idx = O.lbvh_plus(m.arrays(), 60, 1)
    check_tree(nodes, m.size(), boxes)
    nodes, idx, it, cs, rc = O.ploc(m.arrays(), 25)
    assert rc == 0
    check_tree(nodes, m.size(), boxes)


def _ref_eval():
    from oracle import ref
    if not ref.eval_available():
        pytest.skip("reference evaluator not built here (needs the reference sources)")
    return ref.RefEval()


@pytest.mark.parametrize("name", ["uniform1", "uniform17", "uniform4097", "identical100", "flat2000",
                                  "clumped5000", "clustered20000"])
def test_oracle_sah_matches_reference_evaluator(oracle_lib, name):
    O = oracle_lib
    ev = _ref_eval()
    m = meshes.small_cases()[name]
    trees = [O.lbvh(m.arrays(), 30)[0], O.lbvh_plus(m.arrays(), 60, 1)[0], O.ploc(m.arrays(), 10)[0]]
    for nodes in trees:
        sah, nc, lc, md, avg = ev.evaluate(nodes)
        assert O.sah(nodes) == np.float32(sah)
        omd, oavg, olc = O.depth_stats(nodes)
        assert (omd, olc, nc) == (md, lc, nodes.shape[0])
        assert np.float32(oavg) == np.float32(avg)


def test_ploc_no_progress_on_nan(oracle_lib):
    """NaN areas stop every merge; the reference loops forever, the oracle reports no progress."""
    O = oracle_lib
    m = meshgen.uniform_small(50, seed=3)
    for a in m.arrays():
        a[:] = np.nan
    nodes, idx, it, cs, rc = O.ploc(m.arrays(), 5, 100)
    assert rc == 3


def _golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.mark.parametrize("path", _golden_files(), ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_golden(oracle_lib, path):
    """Fixtures made by running the reference's own kernels on a GB300 (tests/golden/make_golden.py)."""
    O = oracle_lib
    g = np.load(path)
    arrays = [g[f"v{k}"] for k in range(9)]
    kind = str(g["kind"])
    ref_nodes = g["nodes"].view(O.NODE_DTYPE).reshape(-1)
    if kind == "lbvh30":
        nodes, idx, _ = O.lbvh(arrays, 30)
        assert np.array_equal(idx, g["indices"])
        assert O.node_fields_equal(nodes, ref_nodes)
    elif kind == "lbvh_plus60":
        nodes, idx = O.lbvh_plus(arrays, 60, 1)
        assert np.array_equal(idx, g["indices"])
        assert O.node_fields_equal(nodes, ref_nodes)
    elif kind.startswith("ploc"):
        r = int(g["radius"])
        nodes, idx, it, cs, rc = O.ploc(arrays, r)
        assert rc == 0
        assert np.array_equal(idx, g["indices"])
        assert O.canonical_equal(nodes, ref_nodes)
    else:
        pytest.skip(f"unknown golden kind {kind}")
