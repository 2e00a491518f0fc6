"""Device-memory helpers for GPU tests (torch is used only for allocation and streams)."""
import numpy as np


def to_device(torch, arrays):
    """Nine device tensors (16-byte aligned) from host arrays; returns (tensors, addresses)."""
    ts = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in arrays]
    return ts, [t.data_ptr() for t in ts]


def stream(torch) -> int:
    return torch.cuda.current_stream().cuda_stream


def build(ctx, torch, mesh, params):
    ts, ptrs = to_device(torch, mesh.arrays())
    tree = ctx.build_device(ptrs, mesh.size(), params, stream(torch))
    ctx.sync()
    nodes, idx = ctx.download(tree, stream(torch))
    return nodes, idx, tree, ts
