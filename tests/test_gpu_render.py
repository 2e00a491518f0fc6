"""Device shading, heatmap and byte conversion (kRenderKernel's shading, applyHeatmapColormap,
savePPM's conversion): bit-exact against the oracle and against the reference's kRenderKernel."""
import numpy as np
import pytest

from bvh_gb300 import Context, auto_camera, meshgen, _capi as C
from bvh_gb300.builders import pinhole_rays
from tests.gpu_util import build, stream

pytestmark = pytest.mark.gpu

LIGHT = np.array([0.5, 0.8, 0.6], np.float32)
LIGHT = (LIGHT / np.float32(np.sqrt(np.float32((LIGHT[0] * LIGHT[0] + LIGHT[1] * LIGHT[1]) + LIGHT[2] * LIGHT[2])))).astype(np.float32)


@pytest.fixture(scope="module")
def ctx(gpu):
    c = Context(0)
    yield c
    c.close()


def _synthetic_lut(seed=5):
    """An arbitrary 256 x 3 colormap (the library takes the colormap from the caller)."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.random((256, 3), dtype=np.float32), axis=0)


def _traced(ctx, gpu, m, w, h, algo=C.ALGO_LBVH):
    nodes, idx, tree, mts = build(ctx, gpu, m, ctx.params(algo))
    cam = auto_camera(nodes[0])
    t = gpu.empty(w * h, dtype=gpu.float32, device="cuda")
    ints = [gpu.empty(w * h, dtype=gpu.int32, device="cuda") for _ in range(4)]
    hts = [t] + ints
    ctx.trace_pinhole(tree.nodes, tree.n_nodes, [x.data_ptr() for x in mts], m.size(), cam, w, h,
                      [x.data_ptr() for x in hts], stream(gpu))
    return nodes, cam, mts, hts


def _diag(nodes):
    r = nodes[0]
    e = (r["max"] - r["min"]).astype(np.float32)
    d = np.float32(np.sqrt(np.float32((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2])))
    return float(d) if d >= 1e-6 else 1.0


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 7])
def test_shade_matches_oracle_bit_exact(ctx, gpu, oracle_lib, mode):
    O = oracle_lib
    m = meshgen.icosphere(5, seed=31)
    w, h = 200, 120
    nodes, cam, mts, hts = _traced(ctx, gpu, m, w, h)
    diag = _diag(nodes)
    rgb = gpu.empty(w * h * 3, dtype=gpu.float32, device="cuda")
    hp = [x.data_ptr() for x in hts]
    ctx.shade([x.data_ptr() for x in mts], m.size(), cam, w, h, hp, mode, diag, LIGHT, rgb.data_ptr(), stream(gpu))
    gpu.cuda.synchronize()
    got = rgb.cpu().numpy().reshape(-1, 3)
    t, prim, vis = hts[0].cpu().numpy(), hts[1].cpu().numpy(), hts[2].cpu().numpy()
    rts = [gpu.empty(w * h, dtype=gpu.float32, device="cuda") for _ in range(6)]
    pinhole_rays(cam, w, h, [x.data_ptr() for x in rts], stream(gpu))
    gpu.cuda.synchronize()
    rd = np.stack([x.cpu().numpy() for x in rts[3:]], axis=1)  # the GPU's rays (device tanf)
    exp = O.shade(m.arrays(), rd, t, prim, vis, mode, diag, LIGHT)
    assert (prim >= 0).sum() > 1000 and (prim < 0).sum() > 100  # hits and misses both present
    assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_shade_vs_reference_render_kernel(ctx, gpu, mode):
    """RGB against kRenderKernel on the reference's own LBVH: bit-equal on every pixel."""
    from oracle import ref
    if not ref.runner_available():
        pytest.skip("reference fatbins not present")
    R = ref.RefRunner()
    m = meshgen.icosphere(5, seed=32)
    rn, _, _ = R.lbvh(m.arrays())
    w, h = 320, 180
    nodes, cam, mts, hts = _traced(ctx, gpu, m, w, h)
    diag = _diag(nodes)
    cam10 = list(cam.eye) + list(cam.look_at) + list(cam.up) + [cam.fov_y_deg]
    _, _, _, rrgb, _ = R.render(rn, m.arrays(), cam10, w, h, mode=mode, scene_diag=diag, light=LIGHT)
    rgb = gpu.empty(w * h * 3, dtype=gpu.float32, device="cuda")
    ctx.shade([x.data_ptr() for x in mts], m.size(), cam, w, h, [x.data_ptr() for x in hts], mode, diag, LIGHT,
              rgb.data_ptr(), stream(gpu))
    gpu.cuda.synchronize()
    got = rgb.cpu().numpy().reshape(-1, 3)
    same = np.all(got.view(np.uint32) == rrgb.view(np.uint32), axis=1)
    assert same.all(), f"mode {mode}: {int((~same).sum())} pixels differ"


@pytest.mark.parametrize("case", ["percentile", "fixed", "all_zero", "one_pixel", "large_counts"])
def test_heatmap_matches_oracle_bit_exact(ctx, gpu, oracle_lib, case):
    O = oracle_lib
    rng = np.random.default_rng(41)
    n = 200 * 120
    fixed = 0.0
    if case == "all_zero":
        vis = np.zeros(n, np.int32)
    elif case == "one_pixel":
        vis = np.zeros(n, np.int32)
        vis[n // 3] = 77
    elif case == "large_counts":  # counts across several high-16-bit bins
        vis = rng.integers(0, 1 << 20, n, dtype=np.int32)
        vis[rng.random(n) < 0.3] = 0
    else:
        vis = rng.geometric(0.02, n).astype(np.int32)
        vis[rng.random(n) < 0.25] = 0
        if case == "fixed":
            fixed = 40.0
    lut = _synthetic_lut()
    dv = gpu.from_numpy(vis).cuda()
    dl = gpu.from_numpy(lut.reshape(-1)).cuda()
    rgb = gpu.empty(n * 3, dtype=gpu.float32, device="cuda")
    used = gpu.zeros(1, dtype=gpu.float32, device="cuda")
    ctx.heatmap(dv.data_ptr(), n, dl.data_ptr(), rgb.data_ptr(), fixed_max=fixed, used_max_ptr=used.data_ptr(),
                stream=stream(gpu))
    gpu.cuda.synchronize()
    exp, mx = O.heatmap(vis, lut, fixed)
    assert float(used.cpu()[0]) == mx
    assert np.array_equal(rgb.cpu().numpy().reshape(-1, 3).view(np.uint32), exp.view(np.uint32))


def test_heatmap_of_traced_visits(ctx, gpu, oracle_lib):
    """The renderImage heatmap flow: trace, then colour the per-pixel node-visit counts."""
    O = oracle_lib
    m = meshgen.clustered(20000, seed=33)
    w, h = 256, 144
    nodes, cam, mts, hts = _traced(ctx, gpu, m, w, h)
    lut = _synthetic_lut(6)
    dl = gpu.from_numpy(lut.reshape(-1)).cuda()
    rgb = gpu.empty(w * h * 3, dtype=gpu.float32, device="cuda")
    used = gpu.zeros(1, dtype=gpu.float32, device="cuda")
    ctx.heatmap(hts[2].data_ptr(), w * h, dl.data_ptr(), rgb.data_ptr(), used_max_ptr=used.data_ptr(),
                stream=stream(gpu))
    gpu.cuda.synchronize()
    exp, mx = O.heatmap(hts[2].cpu().numpy(), lut)
    assert float(used.cpu()[0]) == mx
    assert np.array_equal(rgb.cpu().numpy().reshape(-1, 3).view(np.uint32), exp.view(np.uint32))


def test_rgb8_matches_oracle(ctx, gpu, oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(42)
    v = (rng.random(100003, dtype=np.float32) * 1.4 - 0.2).astype(np.float32)
    v[:6] = [0.0, 1.0, -0.0, 0.5 / 255.0, 254.5 / 255.0, 3.0]
    dv = gpu.from_numpy(v).cuda()
    out = gpu.empty(v.shape[0], dtype=gpu.uint8, device="cuda")
    ctx.rgb8(dv.data_ptr(), v.shape[0], out.data_ptr(), stream(gpu))
    gpu.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), O.rgb8(v))


def test_render_entry_points_reject_bad_arguments(ctx, gpu):
    with pytest.raises(RuntimeError):
        ctx.heatmap(0, 10, 0, 0)
    with pytest.raises(RuntimeError):
        ctx.rgb8(0, 10, 0)
    ctx.heatmap(0, 0, 0, 0)  # nothing to do
    ctx.rgb8(0, 0, 0)
