"""bvh_gb300 -- GPU BVH construction (LBVH, LBVH+, PLOC) and traversal for GB300 (sm_103a).

The compute path is libbvh_gb300.so (hand-written CUDA behind the C ABI in
include/bvh_gb300.h); this package is its host-side mirror of the reference's BVHBuilder
interface.
"""
from ._capi import (ALGO_LBVH, ALGO_LBVH_PLUS, ALGO_PLOC, NODE_DTYPE, BVHError, load_library)  # noqa: F401
from .builders import (BVHBuilder, Context, LBVHBuilder, LBVHPlusBuilder, PLOCBuilder, TriangleMesh,  # noqa: F401
                       auto_camera, load_obj)

__all__ = ["ALGO_LBVH", "ALGO_LBVH_PLUS", "ALGO_PLOC", "NODE_DTYPE", "BVHError", "BVHBuilder", "Context",
           "LBVHBuilder", "LBVHPlusBuilder", "PLOCBuilder", "TriangleMesh", "auto_camera", "load_library",
           "load_obj"]
