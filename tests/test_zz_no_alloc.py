"""bvh_build_lbvh_static: the LBVH build for callers that cannot allocate device memory.

Such callers (a host application that forbids device allocations after start-up, a
real-time loop with a fixed memory budget) cannot create a context, so this entry point keeps
its scratch in a fixed array inside the library and takes only the caller's buffers.  Its
result must equal the context-based build bit for bit, on consecutive calls that reuse the
same array.  This file is collected last so that a failure here does not hide the others.
"""
import ctypes

import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C

pytestmark = pytest.mark.gpu

MAX_TRIS = 262_144


def _static_build(torch, lib, mesh, bits):
    n = mesh.size()
    ts = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in mesh.arrays()]
    m = C.mesh_struct([t.data_ptr() for t in ts], n)
    nodes = torch.empty((2 * n - 1) * 48, dtype=torch.uint8, device="cuda")
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    status = lib.bvh_build_lbvh_static(ctypes.byref(m), bits, ctypes.c_void_p(nodes.data_ptr()),
                                       ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(s))
    torch.cuda.synchronize()
    return status, nodes.cpu().numpy().view(C.NODE_DTYPE), idx.cpu().numpy().view(np.uint32)


def _ctx_build(torch, ctx, mesh, bits):
    ts = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in mesh.arrays()]
    s = torch.cuda.current_stream().cuda_stream
    tree = ctx.build_device([t.data_ptr() for t in ts], mesh.size(), ctx.params(C.ALGO_LBVH, morton_bits=bits), s)
    ctx.sync()
    return ctx.download(tree, s)


def _same(a, b):
    return (np.array_equal(a["min"].view(np.uint32), b["min"].view(np.uint32))
            and np.array_equal(a["max"].view(np.uint32), b["max"].view(np.uint32))
            and np.array_equal(a["left"], b["left"]) and np.array_equal(a["right"], b["right"]))


def test_static_build_equals_context_build_on_consecutive_calls(gpu):
    lib = C.load_library()
    ctx = Context(0)
    cases = [(meshgen.uniform_small(200_000, seed=21), 30), (meshgen.clustered(MAX_TRIS, seed=22), 63),
             (meshgen.uniform_small(1_000, seed=23), 60)]
    for mesh, bits in cases:  # consecutive calls share the library's scratch array
        status, nodes, idx = _static_build(gpu, lib, mesh, bits)
        assert status == C.BVH_OK
        ref_nodes, ref_idx = _ctx_build(gpu, ctx, mesh, bits)
        assert np.array_equal(idx, ref_idx)
        assert _same(nodes, ref_nodes)
    ctx.close()


@pytest.mark.parametrize("bits", [30, 60, 63])
def test_static_build_tiny_meshes(gpu, bits):
    """The static path keeps the 60/63-bit run fix-up's low bits and scratch inside the caller's
    node buffer, which is exactly 2n-1 nodes here: tiny meshes, and a dense cell (long runs of
    equal high halves), against the context build."""
    lib = C.load_library()
    ctx = Context(0)
    meshes = [meshgen.uniform_small(n, seed=30 + n) for n in (1, 2, 7, 9, 1025)]
    one = meshgen.uniform_small(1, seed=29)
    spread = meshgen.uniform_small(2000, seed=28)
    for copies in (600, 2999):  # runs of equal codes ranked by counting (<= 1024) or block-sorted
        same = [np.repeat(a, copies) for a in one.arrays()]
        meshes.append(type(one)(*[np.concatenate([s, b[:1]]) for s, b in zip(same, spread.arrays())]))
        meshes.append(type(one)(*[np.concatenate([s, b]) for s, b in zip(same, spread.arrays())]))
    for mesh in meshes:
        for _ in range(2):
            status, nodes, idx = _static_build(gpu, lib, mesh, bits)
            assert status == C.BVH_OK
            ref_nodes, ref_idx = _ctx_build(gpu, ctx, mesh, bits)
            assert np.array_equal(idx, ref_idx), mesh.size()
            assert _same(nodes, ref_nodes), mesh.size()
    ctx.close()


def test_static_build_rejects_more_than_its_maximum(gpu):
    lib = C.load_library()
    status, _, _ = _static_build(gpu, lib, meshgen.uniform_small(MAX_TRIS + 1, seed=24), 30)
    assert status == C.BVH_ERR_INVALID_ARG
