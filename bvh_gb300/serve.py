"""Python handle on the C ABI's build+trace server (bvh_serve_*, include/bvh_gb300.h).

Requests carry HOST arrays (pinned memory lets their copies overlap other requests); the
arrays must stay alive until the request's result has been polled, which this wrapper
guarantees by keeping a reference per tag.
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _capi as C


class Server:
    def __init__(self, budget_bytes: int = 40 << 30, slots: int = 8, morton_bits: int = 30, device: int = 0,
                 max_triangles: int = 0, max_rays: int = 0, batched: bool = False, batch_requests: int = 0,
                 batch_triangles: int = 0):
        """batched=True: batched ticks (one gather, build, trace and scatter launch sequence for all
        requests admitted together); otherwise one slot per request.  batch_requests and
        batch_triangles bound a batch (0: the library's defaults)."""
        self.lib = C.load_library()
        cfg = self.lib.bvh_serve_default_config()
        cfg.hbm_budget_bytes = int(budget_bytes)
        cfg.slots = int(slots)
        cfg.morton_bits = int(morton_bits)
        cfg.device = int(device)
        cfg.max_triangles = int(max_triangles)
        cfg.max_rays = int(max_rays)
        cfg.reserved[0] = C.SERVE_BATCHED if batched else 0
        cfg.reserved[1] = int(batch_requests)
        cfg.reserved[2] = int(batch_triangles)
        h = ctypes.c_void_p()
        C.check(self.lib.bvh_serve_open(ctypes.byref(cfg), ctypes.byref(h)), "bvh_serve_open")
        self.handle = h
        self._keep: Dict[int, tuple] = {}

    def submit(self, tag: int, mesh_arrays: Sequence, ray_arrays: Sequence, hit_arrays: Sequence) -> None:
        """mesh_arrays: nine host float32 arrays; ray_arrays: ox..dz; hit_arrays: t (float32), prim,
        visited, aabb, tri (int32), each len(rays) -- numpy arrays or pinned torch tensors."""
        def addr(a):
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        n = len(mesh_arrays[0])
        nr = len(ray_arrays[0]) if ray_arrays else 0
        req = C.ServeRequest()
        req.mesh = C.mesh_struct([addr(a) for a in mesh_arrays], n)
        req.rays = C.Rays(*[addr(a) for a in ray_arrays], nr)
        req.hits = C.Hits(*[addr(a) for a in hit_arrays])
        req.tag = tag
        C.check(self.lib.bvh_serve_submit(self.handle, ctypes.byref(req)), "bvh_serve_submit")
        self._keep[tag] = (mesh_arrays, ray_arrays, hit_arrays)

    def poll(self, max_results: int = 256, wait_ms: int = 0) -> List[dict]:
        buf = (C.ServeResult * max_results)()
        k = self.lib.bvh_serve_poll(self.handle, buf, max_results, wait_ms)
        out = []
        for i in range(k):
            r = buf[i]
            self._keep.pop(r.tag, None)
            out.append({"tag": r.tag, "status": r.status, "triangles": r.triangles, "rays": r.rays,
                        "t_submit_ns": r.t_submit_ns, "t_admit_ns": r.t_admit_ns, "t_done_ns": r.t_done_ns})
        return out

    def stats(self) -> dict:
        st = C.ServeStats()
        self.lib.bvh_serve_stats_get(self.handle, ctypes.byref(st))
        return {f: getattr(st, f) for f, _ in C.ServeStats._fields_}

    def close(self) -> None:
        if self.handle:
            C.check(self.lib.bvh_serve_close(self.handle), "bvh_serve_close")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
