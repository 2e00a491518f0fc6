"""Host-side mirror of the reference's builder interface.

``BVHBuilder`` follows include/bvh_builder.h:10-37 (getName, build, getNodes, getIndices,
getLastBuildTimeMS, getTimingBreakdown); ``TriangleMesh`` follows include/mesh.h:9-50 (nine
float32 SoA arrays).  The concrete builders stand in for LBVHBuilderCUDA
(src/cuda/lbvh_builder.cuh:16-64), LBVHPlusBuilderCUDA (src/cuda/lbvh_plus_builder.cuh:11-61)
and PLOCBuilderCUDA (src/cuda/ploc_builder.cuh:10-67) and run every step on the GPU through
the C ABI (include/bvh_gb300.h).  Errors raise ``BVHError`` (a RuntimeError), as the
reference's callers expect std::exception.

``Context.build_device`` is the device-resident path (inputs already in HBM, tree stays there).
"""
from __future__ import annotations

import abc
import ctypes
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _capi as C


@dataclass
class TriangleMesh:
    """SoA triangle mesh (include/mesh.h:9-50): v0x..v2z, float32, one entry per triangle."""
    v0x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v0y: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v0z: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v1x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v1y: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v1z: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v2x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v2y: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    v2z: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))

    def __post_init__(self):
        for f in C.MESH_FIELDS:
            a = np.ascontiguousarray(getattr(self, f), dtype=np.float32)
            setattr(self, f, a)
        n = {getattr(self, f).shape[0] for f in C.MESH_FIELDS}
        if len(n) != 1:
            raise ValueError("all nine SoA arrays must have the same length")

    @classmethod
    def from_vertices(cls, v0: np.ndarray, v1: np.ndarray, v2: np.ndarray) -> "TriangleMesh":
        """From three (n, 3) vertex arrays."""
        return cls(v0[:, 0], v0[:, 1], v0[:, 2], v1[:, 0], v1[:, 1], v1[:, 2], v2[:, 0], v2[:, 1], v2[:, 2])

    def arrays(self) -> Sequence[np.ndarray]:
        return [getattr(self, f) for f in C.MESH_FIELDS]

    def size(self) -> int:
        return int(self.v0x.shape[0])

    def __len__(self) -> int:
        return self.size()

    def getTriangleBounds(self, i: int):
        """mesh.h:36-49: (min, max) of triangle i."""
        v = np.array([[self.v0x[i], self.v0y[i], self.v0z[i]], [self.v1x[i], self.v1y[i], self.v1z[i]],
                      [self.v2x[i], self.v2y[i], self.v2z[i]]], np.float32)
        return v.min(0), v.max(0)


class Context:
    """A library context on one CUDA device (owns the workspace and the last tree)."""

    def __init__(self, device: int = 0):
        self.lib = C.load_library()
        h = ctypes.c_void_p()
        C.check(self.lib.bvh_ctx_create(ctypes.byref(h), int(device)), "bvh_ctx_create")
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.bvh_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self, algo: int, morton_bits: Optional[int] = None, treelet_rounds: Optional[int] = None,
               ploc_radius: Optional[int] = None, max_iterations: Optional[int] = None,
               host_loops: bool = False, no_cooperative: bool = False) -> C.Params:
        p = self.lib.bvh_default_params(algo)
        if host_loops:
            p.reserved[1] = C.HOST_DRIVEN_LOOPS
        if no_cooperative:
            p.reserved[2] = C.NO_COOPERATIVE
        if morton_bits is not None:
            p.morton_bits = morton_bits
        if treelet_rounds is not None:
            p.treelet_rounds = treelet_rounds
        if ploc_radius is not None:
            p.ploc_radius = ploc_radius
        if max_iterations is not None:
            p.max_iterations = max_iterations
        return p

    def reserve(self, n: int, algo: int = C.ALGO_LBVH):
        C.check(self.lib.bvh_ctx_reserve(self.handle, n, algo), "bvh_ctx_reserve")

    def build_device(self, ptrs: Sequence[int], n: int, params: C.Params, stream: int = 0) -> C.Tree:
        """Build from nine device addresses; asynchronous on `stream` (a cudaStream_t value)."""
        m = C.mesh_struct(ptrs, n)
        t = C.Tree()
        C.check(self.lib.bvh_build_device(self.handle, ctypes.byref(m), ctypes.byref(params),
                                          ctypes.c_void_p(stream), ctypes.byref(t)), "bvh_build_device")
        return t

    def build_batched(self, ptrs: Sequence[int], offsets: np.ndarray, params: C.Params, stream: int = 0,
                      use_graph: bool = False) -> C.Tree:
        """Build every mesh of a batch: nine device addresses of the concatenated SoA and the
        count+1 host offsets.  Mesh m's tree is nodes[2*offsets[m]-m : 2*offsets[m+1]-m-1]."""
        offsets = np.ascontiguousarray(offsets, np.uint32)
        count = offsets.shape[0] - 1
        b = C.Batch()
        b.mesh = C.mesh_struct(ptrs, int(offsets[-1]))
        b.offsets = offsets.ctypes.data
        b.count = count
        p = C.Params.from_buffer_copy(params)
        p.reserved[0] = C.BATCH_USE_GRAPH if use_graph else 0
        t = C.Tree()
        C.check(self.lib.bvh_build_batched(self.handle, ctypes.byref(b), ctypes.byref(p), ctypes.c_void_p(stream),
                                           ctypes.byref(t)), "bvh_build_batched")
        self._batch_keep = offsets
        return t

    def evaluate(self, nodes_ptr: int, n_nodes: int, stream: int = 0) -> dict:
        """BVHEvaluator statistics of a device node array, computed on the GPU (bvh_evaluate)."""
        st = C.EvalStats()
        C.check(self.lib.bvh_evaluate(self.handle, ctypes.c_void_p(nodes_ptr), n_nodes, ctypes.c_void_p(stream),
                                      ctypes.byref(st)), "bvh_evaluate")
        return {"sah": st.sah, "avg_leaf_depth": st.avg_leaf_depth, "node_count": st.node_count,
                "leaf_count": st.leaf_count, "max_depth": st.max_depth}

    def autotune(self, n: int, stream: int = 0) -> dict:
        """Time every radix-sort variant on n keys, keep the fastest (bvh_autotune); returns the table."""
        import json
        buf = ctypes.create_string_buffer(8192)
        C.check(self.lib.bvh_autotune(self.handle, n, ctypes.c_void_p(stream), buf, len(buf)), "bvh_autotune")
        return json.loads(buf.value.decode())

    def autotune_build(self, ptrs: Sequence[int], n: int, params: C.Params, stream: int = 0) -> dict:
        """bvh_autotune_build: time every launch shape on this mesh (device SoA), keep the fastest
        in the context's tuning table, report tree-changing choices with their SAH."""
        import json
        m = C.mesh_struct(ptrs, n)
        buf = ctypes.create_string_buffer(1 << 16)
        C.check(self.lib.bvh_autotune_build(self.handle, ctypes.byref(m), ctypes.byref(params), ctypes.c_void_p(stream),
                                            buf, len(buf)), "bvh_autotune_build")
        return json.loads(buf.value.decode())

    def tuning_export(self) -> str:
        """The context's tuning table as JSON (bvh_tuning_export), e.g. to write to a file."""
        buf = ctypes.create_string_buffer(1 << 16)
        C.check(self.lib.bvh_tuning_export(self.handle, buf, len(buf)), "bvh_tuning_export")
        return buf.value.decode()

    def tuning_import(self, text: str) -> None:
        """Replace the tuning table with one bvh_tuning_export wrote (bvh_tuning_import)."""
        C.check(self.lib.bvh_tuning_import(self.handle, text.encode()), "bvh_tuning_import")

    def tuning(self) -> int:
        """The sort variant this context uses (bvh_tuning_get)."""
        a = ctypes.c_int32()
        C.check(self.lib.bvh_tuning_get(self.handle, ctypes.byref(a)), "bvh_tuning_get")
        return a.value

    def set_tuning(self, variant: int):
        C.check(self.lib.bvh_tuning_set(self.handle, variant), "bvh_tuning_set")

    def build_host(self, mesh: TriangleMesh, params: C.Params, stream: int = 0):
        """Upload, build, download (BVHBuilder::build).  Returns (nodes, indices)."""
        n = mesh.size()
        arrs = mesh.arrays()
        m = C.mesh_struct([a.ctypes.data for a in arrs], n)
        nodes = np.zeros(max(2 * n - 1, 0), C.NODE_DTYPE)
        idx = np.zeros(n, np.uint32)
        nn = ctypes.c_uint32(0)
        C.check(self.lib.bvh_build_host(self.handle, ctypes.byref(m), ctypes.byref(params), ctypes.c_void_p(stream),
                                        nodes.ctypes.data if n else None, idx.ctypes.data if n else None,
                                        ctypes.byref(nn)), "bvh_build_host")
        return nodes[: nn.value], idx

    def download(self, tree: C.Tree, stream: int = 0):
        nodes = np.zeros(tree.n_nodes, C.NODE_DTYPE)
        idx = np.zeros(tree.n_prims, np.uint32)
        if tree.n_nodes:
            C.check(self.lib.bvh_tree_download(self.handle, ctypes.byref(tree), ctypes.c_void_p(stream),
                                               nodes.ctypes.data, idx.ctypes.data), "bvh_tree_download")
        return nodes, idx

    def sync(self):
        C.check(self.lib.bvh_sync(self.handle), "bvh_sync")

    def last_timing(self) -> C.Timing:
        t = C.Timing()
        C.check(self.lib.bvh_last_timing(self.handle, ctypes.byref(t)), "bvh_last_timing")
        return t

    def trace(self, nodes_ptr: int, n_nodes: int, mesh_ptrs: Sequence[int], n_tris: int, ray_ptrs: Sequence[int],
              n_rays: int, hit_ptrs: Sequence[int], stream: int = 0):
        m = C.mesh_struct(mesh_ptrs, n_tris)
        r = C.Rays(*ray_ptrs, n_rays)
        h = C.Hits(*hit_ptrs)
        C.check(self.lib.bvh_trace(self.handle, ctypes.c_void_p(nodes_ptr), n_nodes, ctypes.byref(m), ctypes.byref(r),
                                   ctypes.byref(h), ctypes.c_void_p(stream)), "bvh_trace")

    def trace_pinhole(self, nodes_ptr: int, n_nodes: int, mesh_ptrs: Sequence[int], n_tris: int, cam: C.Camera,
                      width: int, height: int, hit_ptrs: Sequence[int], stream: int = 0):
        m = C.mesh_struct(mesh_ptrs, n_tris)
        h = C.Hits(*hit_ptrs)
        C.check(self.lib.bvh_trace_pinhole(self.handle, ctypes.c_void_p(nodes_ptr), n_nodes, ctypes.byref(m),
                                           ctypes.byref(cam), width, height, ctypes.byref(h),
                                           ctypes.c_void_p(stream)), "bvh_trace_pinhole")

    def shade(self, mesh_ptrs: Sequence[int], n_tris: int, cam: C.Camera, width: int, height: int,
              hit_ptrs: Sequence[int], mode: int, scene_diag: float, light_dir, rgb_ptr: int, stream: int = 0):
        """kRenderKernel's shading of a trace_pinhole result into device float RGB (bvh_shade);
        mode 0 normal, 1 depth, 2 diffuse, 3 node visits."""
        m = C.mesh_struct(mesh_ptrs, n_tris)
        h = C.Hits(*hit_ptrs)
        light = (ctypes.c_float * 3)(*[float(x) for x in light_dir])
        C.check(self.lib.bvh_shade(self.handle, ctypes.byref(m), ctypes.byref(cam), width, height, ctypes.byref(h),
                                   int(mode), ctypes.c_float(scene_diag), ctypes.cast(light, ctypes.c_void_p),
                                   ctypes.c_void_p(rgb_ptr), ctypes.c_void_p(stream)), "bvh_shade")

    def heatmap(self, visits_ptr: int, n_pixels: int, colormap_ptr: int, rgb_ptr: int, fixed_max: float = 0.0,
                used_max_ptr: int = 0, stream: int = 0):
        """applyHeatmapColormap on device node-visit counts with a device 256 x 3 colormap (bvh_heatmap)."""
        C.check(self.lib.bvh_heatmap(self.handle, ctypes.c_void_p(visits_ptr), n_pixels, ctypes.c_void_p(colormap_ptr),
                                     ctypes.c_float(fixed_max), ctypes.c_void_p(rgb_ptr),
                                     ctypes.c_void_p(used_max_ptr or None), ctypes.c_void_p(stream)), "bvh_heatmap")

    def rgb8(self, rgb_ptr: int, n_values: int, out_ptr: int, stream: int = 0):
        """savePPM's float-to-byte conversion on the device (bvh_rgb8)."""
        C.check(self.lib.bvh_rgb8(ctypes.c_void_p(rgb_ptr), n_values, ctypes.c_void_p(out_ptr),
                                  ctypes.c_void_p(stream)), "bvh_rgb8")


def load_obj(path: str, threads: int = 0) -> "TriangleMesh":
    """loadOBJ (src/loader.cpp:10-74) as a multi-threaded parse straight to SoA (bvh_load_obj)."""
    lib = C.load_library()
    m = C.ObjMesh()
    C.check(lib.bvh_load_obj(str(path).encode(), int(threads), 0, ctypes.byref(m)), "bvh_load_obj")
    try:
        arrays = [np.ctypeslib.as_array(m.v[k], shape=(max(m.n, 1),))[: m.n].copy() for k in range(9)]
    finally:
        lib.bvh_obj_free(ctypes.byref(m))
    return TriangleMesh(*arrays)


def pinhole_rays(cam: C.Camera, width: int, height: int, ray_ptrs: Sequence[int], stream: int = 0):
    """generateRay (src/render_engine.cu:155-188) for every pixel into six device arrays
    (origin xyz, direction xyz; width * height floats each, row-major) -- bvh_pinhole_rays."""
    lib = C.load_library()
    C.check(lib.bvh_pinhole_rays(ctypes.byref(cam), width, height, *[ctypes.c_void_p(p) for p in ray_ptrs],
                                 ctypes.c_void_p(stream)), "bvh_pinhole_rays")


def auto_camera(root_node) -> C.Camera:
    """autoCamera (src/render_engine.cu:601-637) from a host root node (NODE_DTYPE record) or None."""
    lib = C.load_library()
    cam = C.Camera()
    if root_node is None:
        C.check(lib.bvh_auto_camera(None, ctypes.byref(cam)))
    else:
        rec = np.array([root_node], C.NODE_DTYPE)
        C.check(lib.bvh_auto_camera(ctypes.c_void_p(rec.ctypes.data), ctypes.byref(cam)))
    return cam


class BVHBuilder(abc.ABC):
    """include/bvh_builder.h:10-37."""

    @abc.abstractmethod
    def getName(self) -> str: ...

    @abc.abstractmethod
    def build(self, mesh: TriangleMesh) -> None: ...

    @abc.abstractmethod
    def getNodes(self) -> np.ndarray: ...

    @abc.abstractmethod
    def getIndices(self) -> np.ndarray: ...

    @abc.abstractmethod
    def getLastBuildTimeMS(self) -> float: ...

    def getTimingBreakdown(self) -> str:
        return ""


class _GpuBuilder(BVHBuilder):
    _algo = C.ALGO_LBVH

    def __init__(self, device: int = 0, **params):
        self._ctx = Context(device)
        self._params = self._ctx.params(self._algo, **params)
        self._nodes = np.zeros(0, C.NODE_DTYPE)
        self._indices = np.zeros(0, np.uint32)
        self._timing = C.Timing()

    def build(self, mesh: TriangleMesh) -> None:
        self._nodes, self._indices = self._ctx.build_host(mesh, self._params)
        self._timing = self._ctx.last_timing() if mesh.size() else C.Timing()

    def getNodes(self) -> np.ndarray:
        return self._nodes

    def getIndices(self) -> np.ndarray:
        return self._indices

    def getLastBuildTimeMS(self) -> float:
        """Device time of the build kernels (upload excluded), bvh_builder.h:29-31."""
        return float(self._timing.total_ms)

    def getTimingBreakdown(self) -> str:
        t = self._timing
        return (f"  Scene bounds:     {t.bounds_ms:.3f} ms\n"
                f"  Morton + boxes:   {t.morton_ms:.3f} ms\n"
                f"  Radix sort:       {t.sort_ms:.3f} ms\n"
                f"  Hierarchy+refit:  {t.emit_ms:.3f} ms\n"
                f"  Optimise/cluster: {t.optimize_ms:.3f} ms")


class LBVHBuilder(_GpuBuilder):
    """LBVHBuilderCUDA: 30-bit Morton by default (morton_bits=60 or 63 for longer keys)."""
    _algo = C.ALGO_LBVH

    def getName(self) -> str:
        return "LBVH" if self._params.morton_bits == 30 else f"LBVH-{self._params.morton_bits}"


class LBVHPlusBuilder(_GpuBuilder):
    """LBVHPlusBuilderCUDA: 60-bit Morton, one treelet pass by default."""
    _algo = C.ALGO_LBVH_PLUS

    def getName(self) -> str:
        return "LBVH+"


class PLOCBuilder(_GpuBuilder):
    """PLOCBuilderCUDA(r): radius-r nearest-neighbour clustering."""
    _algo = C.ALGO_PLOC

    def __init__(self, r: int = 25, device: int = 0, **params):
        super().__init__(device, ploc_radius=r, **params)

    def getName(self) -> str:
        return f"PLOC CUDA (r={self._params.ploc_radius})"

    def getTimingBreakdown(self) -> str:
        t = self._timing
        return (f"  Initialization:   {t.bounds_ms + t.morton_ms + t.sort_ms + t.emit_ms:.3f} ms\n"
                f"  Clustering:       {t.optimize_ms:.3f} ms ({t.ploc_iterations} iterations)")
