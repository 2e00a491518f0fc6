"""ctypes binding of the C ABI declared in include/bvh_gb300.h (libbvh_gb300.so).

The shared library is built in-tree by ``bvh_gb300.build.build_library()``.  There is no
fallback: if the library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_float, c_int, c_int32, c_uint32, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbvh_gb300.so")

BVH_OK = 0
BVH_ERR_INVALID_ARG = 1
BVH_ERR_OUT_OF_MEMORY = 2
BVH_ERR_NO_PROGRESS = 3
BVH_ERR_DEVICE = 4
BVH_ERR_TIMEOUT = 5
BVH_ERR_UNSUPPORTED = 6

ALGO_LBVH = 0
ALGO_LBVH_PLUS = 1
ALGO_PLOC = 2

# BVHNode (include/bvh_node.h:8-31): 48 bytes.
NODE_DTYPE = np.dtype([
    ("min", "<f4", (3,)), ("pad0", "<f4"),
    ("max", "<f4", (3,)), ("pad1", "<f4"),
    ("left", "<i4"), ("right", "<i4"), ("aux0", "<i4"), ("aux1", "<i4"),
])
assert NODE_DTYPE.itemsize == 48

MESH_FIELDS = ("v0x", "v0y", "v0z", "v1x", "v1y", "v1z", "v2x", "v2y", "v2z")


class MeshSoA(ctypes.Structure):
    _fields_ = [(f, c_void_p) for f in MESH_FIELDS] + [("n", c_uint32)]


class Params(ctypes.Structure):
    _fields_ = [("algo", c_int32), ("morton_bits", c_int32), ("treelet_rounds", c_int32),
                ("ploc_radius", c_int32), ("max_iterations", c_int32), ("reserved", c_int32 * 3)]


class Tree(ctypes.Structure):
    _fields_ = [("nodes", c_void_p), ("indices", c_void_p), ("n_nodes", c_uint32), ("n_prims", c_uint32)]


class Timing(ctypes.Structure):
    _fields_ = [("total_ms", c_float), ("bounds_ms", c_float), ("morton_ms", c_float), ("sort_ms", c_float),
                ("emit_ms", c_float), ("optimize_ms", c_float), ("ploc_iterations", c_int32),
                ("tree_height", c_int32), ("ploc_cluster_sum", c_uint64), ("kernel_launches", c_int32),
                ("reserved", c_int32)]


class Hits(ctypes.Structure):
    _fields_ = [("t", c_void_p), ("prim", c_void_p), ("nodes_visited", c_void_p), ("aabb_tests", c_void_p),
                ("tri_tests", c_void_p)]


class Rays(ctypes.Structure):
    _fields_ = [(f, c_void_p) for f in ("ox", "oy", "oz", "dx", "dy", "dz")] + [("n", c_uint32)]


class Batch(ctypes.Structure):
    _fields_ = [("mesh", MeshSoA), ("offsets", c_void_p), ("count", c_uint32)]


BATCH_USE_GRAPH = 1
HOST_DRIVEN_LOOPS = 1  # bvh_params.reserved[1]: PLOC / LBVH+ loops driven from the host
NO_COOPERATIVE = 1  # bvh_params.reserved[2]: no cooperative kernels (their host-driven fallbacks)
SERVE_BATCHED = 1  # bvh_serve_config.reserved[0]: batched ticks


class Camera(ctypes.Structure):
    _fields_ = [("eye", c_float * 3), ("look_at", c_float * 3), ("up", c_float * 3), ("fov_y_deg", c_float)]


class EvalStats(ctypes.Structure):
    _fields_ = [("sah", ctypes.c_double), ("avg_leaf_depth", ctypes.c_double), ("node_count", c_uint64),
                ("leaf_count", c_uint64), ("max_depth", c_uint32), ("reserved", c_uint32)]


class ObjMesh(ctypes.Structure):
    _fields_ = [("v", POINTER(ctypes.c_float) * 9), ("n", c_uint32), ("pinned", c_uint32), ("vertices", c_uint64)]


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", c_uint64), ("slots", c_int32), ("morton_bits", c_int32), ("device", c_int32),
                ("max_triangles", c_uint32), ("max_rays", c_uint32), ("reserved", c_int32 * 3)]


class ServeRequest(ctypes.Structure):
    _fields_ = [("mesh", MeshSoA), ("rays", Rays), ("hits", Hits), ("tag", c_uint64)]


class ServeResult(ctypes.Structure):
    _fields_ = [("tag", c_uint64), ("status", c_int32), ("triangles", c_uint32), ("rays", c_uint32),
                ("reserved", c_uint32), ("t_submit_ns", c_uint64), ("t_admit_ns", c_uint64), ("t_done_ns", c_uint64)]


class ServeStats(ctypes.Structure):
    _fields_ = [(f, c_uint64) for f in ("submitted", "admitted", "completed", "rejected", "budget_waits", "triangles",
                                        "rays", "in_flight_bytes", "peak_in_flight_bytes", "queued")]


# Every symbol include/bvh_gb300.h declares, with its ctypes signature.
SIGNATURES = {
    "bvh_status_string": (c_char_p, [c_int]),
    "bvh_version": (c_char_p, []),
    "bvh_ctx_create": (c_int, [POINTER(c_void_p), c_int]),
    "bvh_ctx_destroy": (c_int, [c_void_p]),
    "bvh_ctx_reserve": (c_int, [c_void_p, c_uint32, c_int32]),
    "bvh_ctx_device_bytes": (c_int, [c_void_p, POINTER(c_uint64)]),
    "bvh_default_params": (Params, [c_int32]),
    "bvh_build_device": (c_int, [c_void_p, POINTER(MeshSoA), POINTER(Params), c_void_p, POINTER(Tree)]),
    "bvh_build_host": (c_int, [c_void_p, POINTER(MeshSoA), POINTER(Params), c_void_p, c_void_p, c_void_p,
                               POINTER(c_uint32)]),
    "bvh_tree_download": (c_int, [c_void_p, POINTER(Tree), c_void_p, c_void_p, c_void_p]),
    "bvh_last_timing": (c_int, [c_void_p, POINTER(Timing)]),
    "bvh_sync": (c_int, [c_void_p]),
    "bvh_selftest_bounded_wait": (c_int, [c_int, c_uint32]),
    "bvh_trace": (c_int, [c_void_p, c_void_p, c_uint32, POINTER(MeshSoA), POINTER(Rays), POINTER(Hits), c_void_p]),
    "bvh_trace_pinhole": (c_int, [c_void_p, c_void_p, c_uint32, POINTER(MeshSoA), POINTER(Camera), c_int32, c_int32,
                                  POINTER(Hits), c_void_p]),
    "bvh_pinhole_rays": (c_int, [POINTER(Camera), c_int32, c_int32] + [c_void_p] * 6 + [c_void_p]),
    "bvh_auto_camera": (c_int, [c_void_p, POINTER(Camera)]),
    "bvh_shade": (c_int, [c_void_p, POINTER(MeshSoA), POINTER(Camera), c_int32, c_int32, POINTER(Hits), c_int32,
                          ctypes.c_float, c_void_p, c_void_p, c_void_p]),
    "bvh_heatmap": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p, ctypes.c_float, c_void_p, c_void_p, c_void_p]),
    "bvh_rgb8": (c_int, [c_void_p, c_uint32, c_void_p, c_void_p]),
    "bvh_build_batched": (c_int, [c_void_p, POINTER(Batch), POINTER(Params), c_void_p, POINTER(Tree)]),
    "bvh_autotune": (c_int, [c_void_p, c_uint32, c_void_p, c_char_p, ctypes.c_size_t]),
    "bvh_tuning_get": (c_int, [c_void_p, POINTER(c_int32)]),
    "bvh_tuning_set": (c_int, [c_void_p, c_int32]),
    "bvh_autotune_build": (c_int, [c_void_p, POINTER(MeshSoA), POINTER(Params), c_void_p, c_char_p, ctypes.c_size_t]),
    "bvh_tuning_export": (c_int, [c_void_p, c_char_p, ctypes.c_size_t]),
    "bvh_tuning_import": (c_int, [c_void_p, c_char_p]),
    "bvh_build_lbvh_static": (c_int, [POINTER(MeshSoA), c_int32, c_void_p, c_void_p, c_void_p]),
    "bvh_evaluate": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p, POINTER(EvalStats)]),
    "bvh_load_obj": (c_int, [ctypes.c_char_p, c_int32, c_int32, POINTER(ObjMesh)]),
    "bvh_obj_free": (None, [POINTER(ObjMesh)]),
    "bvh_serve_default_config": (ServeConfig, []),
    "bvh_serve_open": (c_int, [POINTER(ServeConfig), POINTER(c_void_p)]),
    "bvh_serve_submit": (c_int, [c_void_p, POINTER(ServeRequest)]),
    "bvh_serve_poll": (c_int32, [c_void_p, POINTER(ServeResult), c_int32, c_int32]),
    "bvh_serve_stats_get": (c_int, [c_void_p, POINTER(ServeStats)]),
    "bvh_serve_close": (c_int, [c_void_p]),
}

_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libbvh_gb300.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class BVHError(RuntimeError):
    """Non-ok bvh_status from the library (the reference's callers catch std::exception)."""

    def __init__(self, status: int, what: str = ""):
        lib = load_library()
        msg = lib.bvh_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)
        self.status = status


def check(status: int, what: str = "") -> None:
    if status != BVH_OK:
        raise BVHError(status, what)


def mesh_struct(ptrs, n: int) -> MeshSoA:
    """MeshSoA from nine addresses (ints) in TriangleMesh order."""
    m = MeshSoA()
    for f, p in zip(MESH_FIELDS, ptrs):
        setattr(m, f, p)
    m.n = n
    return m
