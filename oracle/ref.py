"""Python access to oracle/_ref/ (TEST INFRASTRUCTURE): the reference's own code.

* ``RefEval`` -- the reference's BVHEvaluator (src/evaluator.cpp), host only; present where
  the reference sources were available at build time.
* ``RefRunner`` -- the reference's GPU kernels (fatbins) driven by oracle/ref_runner.cu.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_float, c_int, c_uint32, c_void_p

import numpy as np

from .oracle import NODE_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def loader_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_loader.so"))


def ref_load_obj(path: str):
    """The reference's loadOBJ on `path`: nine float32 arrays, or None when it throws."""
    lib = ctypes.CDLL(os.path.join(REF_DIR, "libref_loader.so"))
    out = (ctypes.POINTER(ctypes.c_float) * 9)()
    n = ctypes.c_uint32(0)
    if lib.ref_load_obj(path.encode(), out, ctypes.byref(n)):
        return None
    arrays = [np.ctypeslib.as_array(out[k], shape=(max(n.value, 1),))[: n.value].copy() for k in range(9)]
    lib.ref_free(out)
    return arrays


def eval_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_eval.so"))


def runner_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_runner.so")) and os.path.exists(
        os.path.join(REF_DIR, "ref_lbvh.fatbin"))


class RefEval:
    def __init__(self):
        self.lib = ctypes.CDLL(os.path.join(REF_DIR, "libref_eval.so"))
        self.lib.ref_evaluate.argtypes = [c_void_p, c_uint32, POINTER(c_float)]
        self.lib.ref_sizeof_node.restype = c_int

    def evaluate(self, nodes):
        """(sah, node_count, leaf_count, max_depth, avg_leaf_depth) from BVHEvaluator::evaluate."""
        nodes = np.ascontiguousarray(nodes)
        st = (c_float * 5)()
        self.lib.ref_evaluate(nodes.ctypes.data, nodes.shape[0], st)
        return float(st[0]), int(st[1]), int(st[2]), int(st[3]), float(st[4])


def _ptrs(arrays):
    arrs = [np.ascontiguousarray(a, np.float32) for a in arrays]
    arr = (c_void_p * 9)(*[a.ctypes.data for a in arrs])
    return arr, arrs


class RefRunner:
    def __init__(self, fast: bool = False):
        self.lib = ctypes.CDLL(os.path.join(REF_DIR, "libref_runner.so"))
        L = self.lib
        L.ref_error.restype = c_char_p
        L.ref_init.argtypes = [c_char_p, c_char_p]
        L.ref_lbvh.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]
        L.ref_lbvh_plus.argtypes = [c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]
        L.ref_ploc.argtypes = [c_void_p, c_uint32, c_int, c_int, c_void_p, c_void_p, POINTER(c_uint32), POINTER(c_int),
                               c_void_p]
        L.ref_render.argtypes = [c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_int, c_int, c_int, c_float, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        L.ref_ploc_nn.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p]
        L.ref_generate_rays.argtypes = [c_void_p, c_int, c_int, c_void_p]
        L.ref_traverse.argtypes = [c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_uint32, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        rc = L.ref_init(REF_DIR.encode(), b"_fast" if fast else b"")
        if rc:
            raise RuntimeError("ref_init: " + L.ref_error().decode())

    def _check(self, rc, what):
        if rc == 1:
            raise RuntimeError(f"{what}: " + self.lib.ref_error().decode())

    def lbvh(self, arrays):
        """(nodes, indices, ms[8]) from LBVHBuilderCUDA's kernels; ms[0] = getLastBuildTimeMS, ms[6] = wall."""
        p, keep = _ptrs(arrays)
        n = keep[0].shape[0]
        nodes = np.zeros(2 * n - 1, NODE_DTYPE)
        idx = np.zeros(n, np.uint32)
        ms = np.zeros(8, np.float32)
        self._check(self.lib.ref_lbvh(p, n, nodes.ctypes.data, idx.ctypes.data, ms.ctypes.data), "ref_lbvh")
        return nodes, idx, ms

    def lbvh_plus(self, arrays):
        """(nodes, indices, ms[8]); ms[0] = getLastBuildTimeMS, ms[7] = wall."""
        p, keep = _ptrs(arrays)
        n = keep[0].shape[0]
        nodes = np.zeros(2 * n - 1, NODE_DTYPE)
        idx = np.zeros(n, np.uint32)
        ms = np.zeros(8, np.float32)
        self._check(self.lib.ref_lbvh_plus(p, n, nodes.ctypes.data, idx.ctypes.data, ms.ctypes.data), "ref_lbvh_plus")
        return nodes, idx, ms

    def ploc(self, arrays, radius: int = 25, max_iter: int = 10000):
        """(nodes, indices, iterations, ms[8], rc); rc 2/3 = iteration cap / no progress."""
        p, keep = _ptrs(arrays)
        n = keep[0].shape[0]
        nodes = np.zeros(max(2 * n - 1, 1), NODE_DTYPE)
        idx = np.zeros(n, np.uint32)
        nn = c_uint32(0)
        it = c_int(0)
        ms = np.zeros(8, np.float32)
        rc = self.lib.ref_ploc(p, n, radius, max_iter, nodes.ctypes.data, idx.ctypes.data, ctypes.byref(nn),
                               ctypes.byref(it), ms.ctypes.data)
        self._check(rc, "ref_ploc")
        return nodes[: nn.value], idx, it.value, ms, rc

    def render(self, nodes, arrays, cam10, width, height, mode=1, scene_diag=1.0, light=(0.5, 0.8, 0.6)):
        """Per-pixel (visits, aabb_tests, tri_tests, rgb, kernel_ms) from kRenderKernel."""
        p, keep = _ptrs(arrays)
        n = keep[0].shape[0]
        nodes = np.ascontiguousarray(nodes)
        cam = np.asarray(cam10, np.float32)
        lt = np.asarray(light, np.float32)
        npx = width * height
        vis = np.zeros(npx, np.int32)
        at = np.zeros(npx, np.int32)
        tt = np.zeros(npx, np.int32)
        rgb = np.zeros(npx * 3, np.float32)
        ms = np.zeros(1, np.float32)
        self._check(self.lib.ref_render(nodes.ctypes.data, nodes.shape[0], p, n, cam.ctypes.data, width, height, mode,
                                        float(scene_diag), lt.ctypes.data, vis.ctypes.data, at.ctypes.data,
                                        tt.ctypes.data, rgb.ctypes.data, ms.ctypes.data), "ref_render")
        return vis, at, tt, rgb.reshape(-1, 3), float(ms[0])

    def generate_rays(self, cam10, width, height):
        """generateRay for every pixel (row-major): (origins (n, 3), directions (n, 3)) float32."""
        cam = np.asarray(cam10, np.float32)
        outs = [np.zeros(width * height, np.float32) for _ in range(6)]
        arr = (c_void_p * 6)(*[a.ctypes.data for a in outs])
        self._check(self.lib.ref_generate_rays(cam.ctypes.data, width, height, arr), "ref_generate_rays")
        return np.stack(outs[:3], axis=1), np.stack(outs[3:], axis=1)

    def traverse(self, nodes, arrays, ro, rd):
        """traverseBVH on given rays: (t, prim, visits, aabb_tests, tri_tests, normal (n, 3), kernel_ms)."""
        p, keep = _ptrs(arrays)
        n = keep[0].shape[0]
        nodes = np.ascontiguousarray(nodes)
        rays = [np.ascontiguousarray(a[:, k], np.float32) for a in (ro, rd) for k in range(3)]
        nr = rays[0].shape[0]
        rp = (c_void_p * 6)(*[a.ctypes.data for a in rays])
        t = np.zeros(nr, np.float32)
        ints = [np.zeros(nr, np.int32) for _ in range(4)]
        nrm = np.zeros(nr * 3, np.float32)
        ms = np.zeros(1, np.float32)
        self._check(self.lib.ref_traverse(nodes.ctypes.data, nodes.shape[0], p, n, rp, nr, t.ctypes.data,
                                          *[a.ctypes.data for a in ints], nrm.ctypes.data, ms.ctypes.data),
                    "ref_traverse")
        return (t, *ints, nrm.reshape(-1, 3), float(ms[0]))

    def trace_available(self) -> bool:
        return os.path.exists(os.path.join(REF_DIR, "ref_trace.fatbin"))

    def ploc_nn(self, boxes_aabb, radius):
        boxes_aabb = np.ascontiguousarray(boxes_aabb)
        n = boxes_aabb.shape[0]
        nb = np.zeros(n, np.int32)
        d = np.zeros(n, np.float32)
        self._check(self.lib.ref_ploc_nn(boxes_aabb.ctypes.data, n, radius, nb.ctypes.data, d.ctypes.data), "ref_ploc_nn")
        return nb, d
