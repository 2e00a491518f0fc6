"""Autotuner for whole builds: launch shapes never change the tree; tree-changing choices are
reported with their SAH; the table is kept per (algorithm, size bucket) and survives export and
import."""
import json

import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C
from tests.gpu_util import build, to_device, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mesh_dev(gpu):
    m = meshgen.clustered(150_000, seed=71)
    ts, ptrs = to_device(gpu, m.arrays())
    return m, ts, ptrs


@pytest.mark.parametrize("algo,kw,knob,values", [
    (C.ALGO_PLOC, dict(ploc_radius=25), "ploc_radius", [10, 25, 50, 100]),
    (C.ALGO_LBVH, dict(morton_bits=63), "morton_bits", [30, 60, 63]),
    (C.ALGO_LBVH_PLUS, dict(morton_bits=60, treelet_rounds=1), "treelet_rounds", [1, 2, 3]),
])
def test_autotune_keeps_the_tree_and_reports_quality(gpu, oracle_lib, mesh_dev, algo, kw, knob, values):
    m, ts, ptrs = mesh_dev
    ctx = Context(0)
    params = ctx.params(algo, **kw)
    ref_nodes, ref_idx, _, _ = build(ctx, gpu, m, params)  # default shapes
    rep = ctx.autotune_build(ptrs, m.size(), params, stream(gpu))
    assert rep["trials"] and all(t["same_tree"] for t in rep["trials"])
    if algo == C.ALGO_PLOC:  # the PLOC shapes were all tried
        assert {t["ploc_tail_pairs"] for t in rep["trials"]} >= {0, 50000, 100000, 200000}
        assert {t["ploc_grid_max"] for t in rep["trials"]} >= {0, 65536, 150000, 2**32 - 1}
    assert [q[knob] for q in rep["tree_changing"]] == values
    assert all(q["sah"] > 0 and q["ms"] > 0 for q in rep["tree_changing"])
    chosen = rep["chosen"]
    assert chosen["algo"] == algo and chosen["bucket"] == int(np.log2(m.size()))
    # the next build uses the chosen shapes and gives the same tree
    nodes, idx, tree, _ = build(ctx, gpu, m, params)
    assert np.array_equal(idx, ref_idx) and oracle_lib.node_fields_equal(nodes, ref_nodes)
    # the reported SAH of the configured choice is the evaluator's
    st = ctx.evaluate(tree.nodes, tree.n_nodes, stream(gpu))
    q = [q for q in rep["tree_changing"] if q[knob] == kw.get(knob, 1)][0]
    assert abs(q["sah"] - st["sah"]) <= 1e-9 * st["sah"]
    table = json.loads(ctx.tuning_export())
    assert any(e["algo"] == algo and e["bucket"] == chosen["bucket"] for e in table["entries"])
    ctx.close()


def test_odd_shapes_from_an_imported_table_give_the_same_tree(gpu, oracle_lib, mesh_dev):
    m, ts, ptrs = mesh_dev
    bucket = int(np.log2(m.size()))
    ctx = Context(0)
    params = ctx.params(C.ALGO_PLOC, ploc_radius=25)
    ref_nodes, ref_idx, _, _ = build(ctx, gpu, m, params)
    for shape in ({"sort_variant": 3, "ploc_tail_pairs": 0, "ploc_nn_bps": 2, "ploc_mg_bps": 16,
                   "ploc_grid_max": 0},
                  {"sort_variant": 4, "ploc_tail_pairs": 200000, "ploc_nn_bps": 4, "ploc_mg_bps": 4,
                   "ploc_grid_max": 100000},
                  {"sort_variant": 1, "ploc_tail_pairs": 0, "ploc_nn_bps": 3, "ploc_mg_bps": 8,
                   "ploc_grid_max": 2**32 - 1}):
        entry = dict(algo=C.ALGO_PLOC, bucket=bucket, **shape)
        ctx.tuning_import(json.dumps({"entries": [entry]}))
        assert json.loads(ctx.tuning_export())["entries"] == [entry]
        nodes, idx, _, _ = build(ctx, gpu, m, params)
        assert np.array_equal(idx, ref_idx) and oracle_lib.node_fields_equal(nodes, ref_nodes)
    ctx.close()


def test_tuning_import_rejects_bad_tables(gpu):
    ctx = Context(0)
    for bad in ("", "{}", '{"entries": [{"algo": 2}]}',
                '{"entries": [{"algo": 2, "bucket": 10, "sort_variant": 9}]}',
                '{"entries": [{"algo": 2, "bucket": 10, "ploc_nn_bps": 0}]}'):
        with pytest.raises(C.BVHError):
            ctx.tuning_import(bad)
    ctx.close()
