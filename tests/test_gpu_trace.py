"""GPU traversal parity: bit-exact against the oracle, counters against the reference kernel."""
import numpy as np
import pytest

from bvh_gb300 import Context, auto_camera, meshgen, _capi as C
from bvh_gb300.builders import pinhole_rays
from tests.gpu_util import build, to_device, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


def _hits(torch, n):
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    ints = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(4)]
    return [t] + ints, [x.data_ptr() for x in [t] + ints]


@pytest.mark.parametrize("algo", [C.ALGO_LBVH, C.ALGO_PLOC, C.ALGO_LBVH_PLUS])
def test_trace_sphere_rays_bit_exact(ctx, gpu, oracle_lib, algo):
    O = oracle_lib
    m = meshgen.clustered(30000, seed=21)
    nodes, idx, tree, mts = build(ctx, gpu, m, ctx.params(algo))
    ro, rd = meshgen.sphere_rays(m, 20000, seed=3)
    rts = [gpu.from_numpy(np.ascontiguousarray(a)).cuda() for a in (ro[:, 0], ro[:, 1], ro[:, 2], rd[:, 0], rd[:, 1], rd[:, 2])]
    hts, hptr = _hits(gpu, ro.shape[0])
    ctx.trace(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], m.size(), [t.data_ptr() for t in rts],
              ro.shape[0], hptr, stream(gpu))
    gpu.cuda.synchronize()
    got = [h.cpu().numpy() for h in hts]
    exp = O.trace(nodes, m.arrays(), ro, rd)
    assert np.array_equal(got[0].view(np.uint32), exp[0].view(np.uint32))
    for g, e in zip(got[1:], exp[1:]):
        assert np.array_equal(g, e)
    assert (got[1] >= 0).sum() > 1000  # rays do hit


def _gpu_pinhole_rays(gpu, cam, w, h):
    ts = [gpu.empty(w * h, dtype=gpu.float32, device="cuda") for _ in range(6)]
    pinhole_rays(cam, w, h, [t.data_ptr() for t in ts], stream(gpu))
    gpu.cuda.synchronize()
    a = [t.cpu().numpy() for t in ts]
    return np.stack(a[:3], axis=1), np.stack(a[3:], axis=1)


def test_pinhole_rays_and_trace_match_oracle(ctx, gpu, oracle_lib):
    """bvh_trace_pinhole against the oracle's traversal of the rays bvh_pinhole_rays generates (the
    device's tanf may differ from the host's in the last place, so the oracle takes the GPU's rays;
    those are pinned against the reference's generateRay in test_gpu_trace_ref.py).  The oracle's
    own pinhole generator agrees with the GPU's on all but a few rays."""
    O = oracle_lib
    m = meshgen.clustered(20000, seed=22)
    nodes, idx, tree, mts = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
    cam = auto_camera(nodes[0])
    w, h = 160, 90
    hts, hptr = _hits(gpu, w * h)
    ctx.trace_pinhole(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], m.size(), cam, w, h, hptr, stream(gpu))
    gpu.cuda.synchronize()
    got = [x.cpu().numpy() for x in hts]
    ro, rd = _gpu_pinhole_rays(gpu, cam, w, h)
    oro, ord_ = O.pinhole_rays(list(cam.eye), list(cam.look_at), list(cam.up), cam.fov_y_deg, w, h)
    assert np.array_equal(ro, oro)
    assert (np.abs(rd - ord_) <= 1e-6).all()
    exp = O.trace(nodes, m.arrays(), ro, rd)
    assert np.array_equal(got[0].view(np.uint32), exp[0].view(np.uint32))
    for g, e in zip(got[1:], exp[1:]):
        assert np.array_equal(g, e)


def test_pinhole_counters_vs_reference_render_kernel(ctx, gpu, oracle_lib):
    """Per-pixel nodes visited / AABB tests / triangle tests and hit/miss against the reference's
    kRenderKernel on its own LBVH: identical on every pixel."""
    from oracle import ref
    if not ref.runner_available():
        pytest.skip("reference fatbins not present")
    R = ref.RefRunner()
    m = meshgen.clustered(20000, seed=23)
    rn, ri, _ = R.lbvh(m.arrays())
    nodes, idx, tree, mts = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
    cam = auto_camera(nodes[0])
    w, h = 320, 180
    cam10 = list(cam.eye) + list(cam.look_at) + list(cam.up) + [cam.fov_y_deg]
    rv, ra, rt, rgb, _ = R.render(rn, m.arrays(), cam10, w, h, mode=1)
    hts, hptr = _hits(gpu, w * h)
    ctx.trace_pinhole(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], m.size(), cam, w, h, hptr, stream(gpu))
    gpu.cuda.synchronize()
    got = [x.cpu().numpy() for x in hts]
    assert oracle_lib.node_fields_equal(nodes, rn)  # the same tree on both sides
    same = (got[2] == rv) & (got[3] == ra) & (got[4] == rt)
    assert same.all(), f"{int((~same).sum())} pixels differ"
    bg = np.all(rgb == np.array([0.15, 0.15, 0.18], np.float32), axis=1)
    assert np.array_equal(got[1] < 0, bg)


@pytest.mark.parametrize("algo", [C.ALGO_LBVH, C.ALGO_PLOC, C.ALGO_LBVH_PLUS])
def test_gpu_evaluator_matches_reference_evaluator_restatement(ctx, gpu, oracle_lib, algo):
    """bvh_evaluate against the oracle's restatement of BVHEvaluator (itself pinned bit-equal to
    the reference's evaluator.cpp): SAH within 1e-5 relative, counts and depths exact."""
    O = oracle_lib
    m = meshgen.clustered(50_000, seed=31)
    nodes, idx, tree, _ = build(ctx, gpu, m, ctx.params(algo))
    st = ctx.evaluate(tree.nodes, tree.n_nodes, stream(gpu))
    sah = O.sah(nodes)
    md, avg, lc = O.depth_stats(nodes)
    assert abs(st["sah"] - sah) <= 1e-5 * abs(sah)
    assert st["node_count"] == nodes.shape[0] and st["leaf_count"] == lc and st["max_depth"] == md
    assert abs(st["avg_leaf_depth"] - avg) <= 1e-5 * avg
