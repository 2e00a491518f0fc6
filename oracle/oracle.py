"""Python binding of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the
checker.  The product path (bvh_gb300/) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_float, c_int, c_uint32, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

NODE_DTYPE = np.dtype([
    ("min", "<f4", (3,)), ("pad0", "<f4"),
    ("max", "<f4", (3,)), ("pad1", "<f4"),
    ("left", "<i4"), ("right", "<i4"), ("aux0", "<i4"), ("aux1", "<i4"),
])
AABB_DTYPE = np.dtype([("min", "<f4", (3,)), ("pad0", "<f4"), ("max", "<f4", (3,)), ("pad1", "<f4")])


class OrcMesh(ctypes.Structure):
    _fields_ = [("v", c_void_p * 9), ("n", c_uint32)]


_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_lbvh.argtypes = [POINTER(OrcMesh), c_int, c_void_p, c_void_p, c_void_p]
        L.orc_lbvh_plus.argtypes = [POINTER(OrcMesh), c_int, c_int, c_void_p, c_void_p]
        L.orc_ploc.argtypes = [POINTER(OrcMesh), c_int, c_int, c_void_p, c_void_p, POINTER(c_uint32),
                               POINTER(c_int), POINTER(c_uint64)]
        L.orc_trace.argtypes = [c_void_p, c_uint32, POINTER(OrcMesh), c_void_p, c_void_p, c_uint32, c_void_p,
                                c_void_p, c_void_p, c_void_p, c_void_p]
        L.orc_pinhole_rays.argtypes = [c_void_p, c_void_p, c_void_p, c_float, c_int, c_int, c_void_p, c_void_p]
        L.orc_shade.argtypes = [POINTER(OrcMesh), c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_int, c_float,
                                c_void_p, c_void_p]
        L.orc_heatmap.argtypes = [c_void_p, c_uint32, c_void_p, c_float, c_void_p]
        L.orc_heatmap.restype = c_float
        L.orc_rgb8.argtypes = [c_void_p, c_uint32, c_void_p]
        L.orc_sah.argtypes = [c_void_p, c_uint32]
        L.orc_sah.restype = c_float
        L.orc_depth_stats.argtypes = [c_void_p, c_uint32, POINTER(c_int), POINTER(c_float), POINTER(c_uint32)]
        L.orc_tree_equal_canonical.argtypes = [c_void_p, c_uint32, c_void_p, c_uint32]
        L.orc_tri_bounds.argtypes = [POINTER(OrcMesh), c_void_p, c_void_p]
        L.orc_scene_bounds.argtypes = [c_void_p, c_uint32, c_void_p]
        L.orc_morton.argtypes = [c_void_p, c_uint32, c_int, c_void_p, c_void_p]
        L.orc_sort_pairs.argtypes = [c_void_p, c_void_p, c_uint32, c_int, c_int]
        L.orc_set_sa_form.argtypes = [c_int]
        L.orc_sa.argtypes = [c_void_p]
        L.orc_sa.restype = c_float
        L.orc_fmin.argtypes = [c_float, c_float]
        L.orc_fmin.restype = c_float
        L.orc_fmax.argtypes = [c_float, c_float]
        L.orc_fmax.restype = c_float
        L.orc_set_threads.argtypes = [c_int]
        L.orc_treelet.argtypes = [c_void_p, c_void_p, c_int]
        _lib = L
    return _lib


def _mesh(arrays):
    arrs = [np.ascontiguousarray(a, np.float32) for a in arrays]
    m = OrcMesh()
    for k, a in enumerate(arrs):
        m.v[k] = a.ctypes.data
    m.n = arrs[0].shape[0] if arrs else 0
    return m, arrs


def set_threads(t: int):
    lib().orc_set_threads(t)


def threads() -> int:
    return lib().orc_threads()


def lbvh(arrays, bits: int = 30):
    """(nodes, indices, sorted_keys) as LBVHBuilderCUDA (bits=30) or the 60/63-bit variant."""
    m, keep = _mesh(arrays)
    n = m.n
    nodes = np.zeros(max(2 * n - 1, 0), NODE_DTYPE)
    idx = np.zeros(n, np.uint32)
    keys = np.zeros(n, np.uint64)
    rc = lib().orc_lbvh(ctypes.byref(m), bits, nodes.ctypes.data, idx.ctypes.data, keys.ctypes.data)
    if rc:
        raise RuntimeError(f"orc_lbvh rc={rc}")
    return nodes, idx, keys


def lbvh_plus(arrays, bits: int = 60, rounds: int = 1):
    m, keep = _mesh(arrays)
    n = m.n
    nodes = np.zeros(max(2 * n - 1, 0), NODE_DTYPE)
    idx = np.zeros(n, np.uint32)
    rc = lib().orc_lbvh_plus(ctypes.byref(m), bits, rounds, nodes.ctypes.data, idx.ctypes.data)
    if rc:
        raise RuntimeError(f"orc_lbvh_plus rc={rc}")
    return nodes, idx


def ploc(arrays, radius: int = 25, max_iter: int = 0):
    """(nodes, indices, iterations, cluster_sum, rc)."""
    m, keep = _mesh(arrays)
    n = m.n
    nodes = np.zeros(max(2 * n - 1, 0), NODE_DTYPE)
    idx = np.zeros(n, np.uint32)
    nn = c_uint32(0)
    it = c_int(0)
    cs = c_uint64(0)
    rc = lib().orc_ploc(ctypes.byref(m), radius, max_iter, nodes.ctypes.data, idx.ctypes.data, ctypes.byref(nn),
                        ctypes.byref(it), ctypes.byref(cs))
    return nodes[: nn.value], idx, it.value, cs.value, rc


def tri_bounds(arrays):
    m, keep = _mesh(arrays)
    boxes = np.zeros(m.n, AABB_DTYPE)
    c4 = np.zeros((m.n, 4), np.float32)
    lib().orc_tri_bounds(ctypes.byref(m), boxes.ctypes.data, c4.ctypes.data)
    return boxes, c4


def trace(nodes, arrays, ro, rd):
    """Closest-hit traversal of explicit rays: (t, prim, visited, aabb_tests, tri_tests)."""
    m, keep = _mesh(arrays)
    ro = np.ascontiguousarray(ro, np.float32).reshape(-1, 3)
    rd = np.ascontiguousarray(rd, np.float32).reshape(-1, 3)
    nr = ro.shape[0]
    nodes = np.ascontiguousarray(nodes)
    t = np.zeros(nr, np.float32)
    prim = np.zeros(nr, np.int32)
    vis = np.zeros(nr, np.int32)
    at = np.zeros(nr, np.int32)
    tt = np.zeros(nr, np.int32)
    lib().orc_trace(nodes.ctypes.data, nodes.shape[0], ctypes.byref(m), ro.ctypes.data, rd.ctypes.data, nr,
                    t.ctypes.data, prim.ctypes.data, vis.ctypes.data, at.ctypes.data, tt.ctypes.data)
    return t, prim, vis, at, tt


def pinhole_rays(eye, look, up, fovy, width, height):
    eye = np.asarray(eye, np.float32)
    look = np.asarray(look, np.float32)
    up = np.asarray(up, np.float32)
    ro = np.zeros((width * height, 3), np.float32)
    rd = np.zeros((width * height, 3), np.float32)
    lib().orc_pinhole_rays(eye.ctypes.data, look.ctypes.data, up.ctypes.data, float(fovy), width, height,
                           ro.ctypes.data, rd.ctypes.data)
    return ro, rd


def shade(arrays, rd, t, prim, vis, mode, diag, light):
    """kRenderKernel's shading of traced pixels: float RGB (n, 3)."""
    m, keep = _mesh(arrays)
    rd = np.ascontiguousarray(rd, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(t, np.float32)
    prim = np.ascontiguousarray(prim, np.int32)
    vis = np.ascontiguousarray(vis, np.int32)
    light = np.ascontiguousarray(light, np.float32)
    rgb = np.zeros((t.shape[0], 3), np.float32)
    lib().orc_shade(ctypes.byref(m), rd.ctypes.data, t.ctypes.data, prim.ctypes.data, vis.ctypes.data, t.shape[0],
                    int(mode), float(diag), light.ctypes.data, rgb.ctypes.data)
    return rgb


def heatmap(vis, lut, fixed_max=0.0):
    """applyHeatmapColormap with a (256, 3) colormap: (rgb (n, 3), normalisation)."""
    vis = np.ascontiguousarray(vis, np.int32)
    lut = np.ascontiguousarray(lut, np.float32).reshape(256, 3)
    rgb = np.zeros((vis.shape[0], 3), np.float32)
    mx = lib().orc_heatmap(vis.ctypes.data, vis.shape[0], lut.ctypes.data, float(fixed_max), rgb.ctypes.data)
    return rgb, float(mx)


def rgb8(rgb):
    rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1)
    out = np.zeros(rgb.shape[0], np.uint8)
    lib().orc_rgb8(rgb.ctypes.data, rgb.shape[0], out.ctypes.data)
    return out


def sah(nodes) -> float:
    nodes = np.ascontiguousarray(nodes)
    return float(lib().orc_sah(nodes.ctypes.data, nodes.shape[0]))


def depth_stats(nodes):
    nodes = np.ascontiguousarray(nodes)
    md = c_int(0)
    avg = c_float(0)
    lc = c_uint32(0)
    lib().orc_depth_stats(nodes.ctypes.data, nodes.shape[0], ctypes.byref(md), ctypes.byref(avg), ctypes.byref(lc))
    return md.value, avg.value, lc.value


def canonical_equal(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return lib().orc_tree_equal_canonical(a.ctypes.data, a.shape[0], b.ctypes.data, b.shape[0]) == 0


def sa(box) -> float:
    b = np.array([box], AABB_DTYPE)
    return float(lib().orc_sa(b.ctypes.data))


def set_sa_form(form: int):
    lib().orc_set_sa_form(form)


def node_fields_equal(a, b) -> bool:
    """Bit-exact equality of the BVHNode fields (min, max, left, right); padding ignored."""
    if a.shape != b.shape:
        return False
    return (np.array_equal(a["min"].view(np.uint32), b["min"].view(np.uint32))
            and np.array_equal(a["max"].view(np.uint32), b["max"].view(np.uint32))
            and np.array_equal(a["left"], b["left"]) and np.array_equal(a["right"], b["right"]))
