"""Traversal parity against the reference's own device code on identical rays.

The reference's generateRay (src/render_engine.cu:155-188) and traverseBVH (:289-356) run as
kernels from oracle/_ref/ref_trace.fatbin: its unmodified render_engine.cu, compiled with its
default flags and wrapped by oracle/ref_trace_shim.cu.  The library's rays must equal generateRay's
bit for bit.  Its traversal must equal traverseBVH's on every ray: t bit-equal, hit primitive
equal, and node, AABB and triangle counters equal.  The oracle's traversal is checked on the same
rays too, which pins the CPU restatement to the reference.
"""
import numpy as np
import pytest

from bvh_gb300 import Context, auto_camera, meshgen, _capi as C
from bvh_gb300.builders import pinhole_rays
from tests.gpu_util import build, stream

pytestmark = pytest.mark.gpu


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
    r = ref.RefRunner()
    if not r.trace_available():
        pytest.skip("reference traversal fatbin not present")
    return r


def _cam10(cam):
    return list(cam.eye) + list(cam.look_at) + list(cam.up) + [cam.fov_y_deg]


def _our_rays(gpu, cam, w, h):
    ts = [gpu.empty(w * h, dtype=gpu.float32, device="cuda") for _ in range(6)]
    pinhole_rays(cam, w, h, [t.data_ptr() for t in ts], stream(gpu))
    gpu.cuda.synchronize()
    a = [t.cpu().numpy() for t in ts]
    return np.stack(a[:3], axis=1), np.stack(a[3:], axis=1)


def _trace(ctx, gpu, tree, mts, n_tris, ro, rd):
    rts = [gpu.from_numpy(np.ascontiguousarray(a[:, k], np.float32)).cuda() for a in (ro, rd) for k in range(3)]
    nr = ro.shape[0]
    hts = [gpu.empty(nr, dtype=gpu.float32, device="cuda")] + [gpu.empty(nr, dtype=gpu.int32, device="cuda")
                                                             for _ in range(4)]
    ctx.trace(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], n_tris, [t.data_ptr() for t in rts], nr,
              [h.data_ptr() for h in hts], stream(gpu))
    gpu.cuda.synchronize()
    return [h.cpu().numpy() for h in hts]


def _assert_same_hits(got, ref, what):
    """t bit-equal, prim equal, counters equal -- on every ray; the message counts each kind."""
    t_ok = got[0].view(np.uint32) == ref[0].view(np.uint32)
    bad = {"t": int((~t_ok).sum())}
    for name, g, r in zip(("prim", "visits", "aabb_tests", "tri_tests"), got[1:5], ref[1:5]):
        bad[name] = int((g != r).sum())
    assert all(v == 0 for v in bad.values()), f"{what}: rays that differ {bad} of {got[0].shape[0]}"


def _custom_cameras(root):
    lo, hi = root["min"].astype(np.float32), root["max"].astype(np.float32)
    c = (lo + hi) * np.float32(0.5)
    cams = []
    for eye_off, up, fov in (((2.5, 0.4, -1.7), (0.0, 1.0, 0.0), 45.0), ((-0.3, 3.1, 0.2), (0.3, 0.1, 0.9), 90.0),
                             ((0.9, -1.2, 2.2), (0.0, 0.0, 1.0), 17.5)):
        cam = C.Camera()
        for k in range(3):
            cam.eye[k] = float(c[k] + np.float32(eye_off[k]))
            cam.look_at[k] = float(c[k])
            cam.up[k] = up[k]
        cam.fov_y_deg = fov
        cams.append(cam)
    return cams


def test_pinhole_rays_equal_reference_generate_ray(ctx, gpu, R):
    """bvh_pinhole_rays against generateRay for autoCamera at 1920x1080 and three other cameras
    and image shapes (odd sizes, tilted up vectors, narrow and wide fields of view)."""
    m = meshgen.clustered(20000, seed=51)
    nodes, _, _, _ = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
    cases = [(auto_camera(nodes[0]), 1920, 1080)]
    cases += list(zip(_custom_cameras(nodes[0]), (640, 333, 1), (480, 217, 1)))
    for cam, w, h in cases:
        ro, rd = _our_rays(gpu, cam, w, h)
        rro, rrd = R.generate_rays(_cam10(cam), w, h)
        assert np.array_equal(ro.view(np.uint32), rro.view(np.uint32)), (w, h)
        diff = (rd.view(np.uint32) != rrd.view(np.uint32)).any(axis=1)
        assert not diff.any(), f"{w}x{h} fov {cam.fov_y_deg}: {int(diff.sum())} directions differ"


@pytest.mark.slow
@pytest.mark.parametrize("algo", [C.ALGO_LBVH, C.ALGO_LBVH_PLUS, C.ALGO_PLOC])
def test_sphere_rays_equal_reference_traverse_c2a(ctx, gpu, R, oracle_lib, algo):
    """Config c2a at full size: the 1,310,720-triangle displaced icosphere, 1M random-direction rays
    from a sphere around it; every ray identical to traverseBVH's result on the same tree."""
    m = meshgen.icosphere(8, seed=2)
    nodes, _, tree, mts = build(ctx, gpu, m, ctx.params(algo))
    ro, rd = meshgen.sphere_rays(m, 1_000_000, seed=6)
    got = _trace(ctx, gpu, tree, mts, m.size(), ro, rd)
    ref = R.traverse(nodes, m.arrays(), ro, rd)
    assert (ref[1] >= 0).sum() > 300_000  # most rays hit
    _assert_same_hits(got, ref, "c2a sphere rays")
    # the oracle's restatement on the first 100,000 rays
    exp = oracle_lib.trace(nodes, m.arrays(), ro[:100_000], rd[:100_000])
    _assert_same_hits([g[:100_000] for g in got], exp, "oracle, c2a sphere rays")


@pytest.mark.slow
def test_pinhole_1080p_equals_reference_c1_sample(ctx, gpu, R, oracle_lib):
    """1920x1080 primary rays from autoCamera over a 1M-triangle sample of config c1 (64 Gaussian
    clusters), LBVH with 63-bit codes: bvh_trace_pinhole against generateRay + traverseBVH."""
    m = meshgen.clustered(1_000_000, seed=1)
    nodes, _, tree, mts = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH, morton_bits=63))
    cam = auto_camera(nodes[0])
    w, h = 1920, 1080
    hts = [gpu.empty(w * h, dtype=gpu.float32, device="cuda")] + [gpu.empty(w * h, dtype=gpu.int32, device="cuda")
                                                               for _ in range(4)]
    ctx.trace_pinhole(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], m.size(), cam, w, h,
                      [x.data_ptr() for x in hts], stream(gpu))
    gpu.cuda.synchronize()
    got = [x.cpu().numpy() for x in hts]
    rro, rrd = R.generate_rays(_cam10(cam), w, h)
    ref = R.traverse(nodes, m.arrays(), rro, rrd)
    assert (ref[1] >= 0).sum() > 10_000
    _assert_same_hits(got, ref, "1080p pinhole")
    sel = np.arange(0, w * h, 7)
    exp = oracle_lib.trace(nodes, m.arrays(), rro[sel], rrd[sel])
    _assert_same_hits([g[sel] for g in got], exp, "oracle, 1080p pinhole")


@pytest.mark.parametrize("algo", [C.ALGO_LBVH, C.ALGO_PLOC])
def test_small_meshes_equal_reference_traverse(ctx, gpu, R, algo):
    """Small and degenerate scenes: 1 and 2 triangles, identical triangles, a flat scene, rays
    starting inside the box and axis-aligned directions (inverse direction +-1e30)."""
    rng = np.random.default_rng(52)
    meshes = [meshgen.uniform_small(1, seed=1), meshgen.uniform_small(2, seed=2), meshgen.uniform_small(3000, seed=3)]
    same = meshgen.uniform_small(1, seed=4)
    meshes.append(type(same)(*[np.repeat(a, 300) for a in same.arrays()]))
    flat = meshgen.uniform_small(2000, seed=5)
    arrs = [a.copy() for a in flat.arrays()]
    for k in (2, 5, 8):
        arrs[k][:] = np.float32(0.25)
    meshes.append(type(flat)(*arrs))
    for m in meshes:
        nodes, _, tree, mts = build(ctx, gpu, m, ctx.params(algo))
        ro, rd = meshgen.sphere_rays(m, 20000, seed=7)
        lo, hi = meshgen.scene_box(m)
        ro[:5000] = (lo + rng.random((5000, 3)) * (hi - lo)).astype(np.float32)  # origins inside the box
        axis = np.zeros((3000, 3), np.float32)
        axis[np.arange(3000), rng.integers(0, 3, 3000)] = rng.choice([-1.0, 1.0], 3000).astype(np.float32)
        rd[5000:8000] = axis
        got = _trace(ctx, gpu, tree, mts, m.size(), ro, rd)
        ref = R.traverse(nodes, m.arrays(), ro, rd)
        _assert_same_hits(got, ref, f"{m.size()} triangles")


def test_hit_normals_equal_reference(ctx, gpu, R):
    """The closest hit's geometric normal (shading mode 0 writes (n + 1) / 2) equals the normal
    traverseBVH returns, bit for bit."""
    m = meshgen.icosphere(5, seed=53)
    nodes, _, tree, mts = build(ctx, gpu, m, ctx.params(C.ALGO_LBVH))
    cam = auto_camera(nodes[0])
    w, h = 320, 200
    hts = [gpu.empty(w * h, dtype=gpu.float32, device="cuda")] + [gpu.empty(w * h, dtype=gpu.int32, device="cuda")
                                                               for _ in range(4)]
    ctx.trace_pinhole(tree.nodes, tree.n_nodes, [t.data_ptr() for t in mts], m.size(), cam, w, h,
                      [x.data_ptr() for x in hts], stream(gpu))
    rgb = gpu.empty(w * h * 3, dtype=gpu.float32, device="cuda")
    ctx.shade([t.data_ptr() for t in mts], m.size(), cam, w, h, [x.data_ptr() for x in hts], 0, 1.0,
              [0.0, 1.0, 0.0], rgb.data_ptr(), stream(gpu))
    gpu.cuda.synchronize()
    got = rgb.cpu().numpy().reshape(-1, 3)
    rro, rrd = R.generate_rays(_cam10(cam), w, h)
    ref = R.traverse(nodes, m.arrays(), rro, rrd)
    hit = ref[1] >= 0
    assert hit.sum() > 5000
    exp = ((ref[5][hit] + np.float32(1.0)) * np.float32(0.5)).astype(np.float32)
    assert np.array_equal(got[hit].view(np.uint32), exp.view(np.uint32))
