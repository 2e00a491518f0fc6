"""Edge-case meshes shared by the CPU and GPU tests."""
import numpy as np

from bvh_gb300.builders import TriangleMesh
from bvh_gb300 import meshgen


def identical(n):
    """Every triangle the same: all Morton codes equal, order by original index."""
    v = np.tile(np.array([[0.1, 0.2, 0.3]], np.float32), (n, 1))
    return TriangleMesh.from_vertices(v, v + np.float32(0.01), v + np.float32([0.0, 0.02, 0.0]))


def flat_z(n, seed=7):
    """All triangles in the plane z = 0.5 (zero scene extent along z)."""
    g = np.random.default_rng(seed)
    c = g.random((n, 3), dtype=np.float32)
    c[:, 2] = 0.5
    off = [(g.random((n, 3), dtype=np.float32) - 0.5) * np.float32(0.01) for _ in range(3)]
    for o in off:
        o[:, 2] = 0.0
    return TriangleMesh.from_vertices(c + off[0], c + off[1], c + off[2])


def clumped(n, seed=8):
    """Most triangles in a 1e-7 cube: many duplicate Morton codes."""
    g = np.random.default_rng(seed)
    c = g.random((n, 3), dtype=np.float32) * np.float32(1e-7) + np.float32(0.25)
    c[: n // 10] = g.random((n // 10, 3), dtype=np.float32)
    return TriangleMesh.from_vertices(c, c + np.float32(1e-8), c + np.float32([0, 2e-8, 0]))


def dense_cell(n, size=2e-4, spread=0.1, seed=10):
    """Most triangles in one small cube of a unit scene: with 60/63-bit codes they share the high
    32 code bits but differ below (long runs for the run fix-up after the high-half sort)."""
    g = np.random.default_rng(seed)
    c = g.random((n, 3), dtype=np.float32) * np.float32(size) + np.float32(0.3)
    k = int(n * spread)
    c[:k] = g.random((k, 3), dtype=np.float32)
    d = np.float32(size * 0.01)
    return TriangleMesh.from_vertices(c, c + d, c + np.float32([0, 1, 0]) * d)


def negative_scaled(n, seed=9):
    m = meshgen.uniform_small(n, seed=seed, scale=123.0, offset=(-400.0, 7.0, -0.001))
    return m


def small_cases():
    out = {}
    for n in (1, 2, 3, 5, 17, 64, 255, 256, 257, 1000, 3071, 3072, 3073, 4097):
        out[f"uniform{n}"] = meshgen.uniform_small(n, seed=n)
    out["identical100"] = identical(100)
    out["identical5000"] = identical(5000)                    # one run of equal codes > 1024
    out["identical1"] = identical(1)
    out["flat2000"] = flat_z(2000)
    out["clumped5000"] = clumped(5000)
    out["negscaled3000"] = negative_scaled(3000)
    out["clustered20000"] = meshgen.clustered(20000, seed=11)
    out["densecell6000"] = dense_cell(6000)                   # runs of thousands
    out["mediumcell3000"] = dense_cell(3000, size=4e-3)       # runs of about ten
    return out
