"""Seeded synthetic meshes and rays for the benchmark workloads.

The reference's random generator (src/loader.cpp:77-98) is seeded by wall-clock time and its
OBJ scenes are not shipped, so these seeded generators stand in for its inputs:

  uniform_small   n triangles: centroid ~ U[0,1]^3, each vertex = centroid + U[-0.005,0.005]^3
  clustered       64 Gaussian clusters (sigma 0.02, means ~ U[0,1]^3), vertices at distance
                  edge ~ logU[1e-4,1e-2] from the centroid in random directions
  icosphere       20*4^L triangles of a subdivided icosahedron displaced radially by
                  0.05 * fBm (4 octaves of value noise)
  strands         long thin triangles along random-walk strands in the unit cube
  batch_counts    mesh sizes ~ logU[lo, hi] for batched builds
  sphere_rays     origins uniform on a sphere of radius 1.5*(diag/2) around the scene box,
                  directions towards uniform points inside the box

Everything is numpy float32 from numpy's PCG64 generator, so a seed gives the same mesh on
x86-64 and aarch64.
"""
from __future__ import annotations

import numpy as np

from .builders import TriangleMesh


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def uniform_small(n: int, seed: int = 0, scale: float = 1.0, offset=(0.0, 0.0, 0.0)) -> TriangleMesh:
    g = _rng(seed)
    c = g.random((n, 3), dtype=np.float32)
    v = [c + (g.random((n, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.01) for _ in range(3)]
    off = np.asarray(offset, np.float32)
    v = [(x * np.float32(scale) + off).astype(np.float32) for x in v]
    return TriangleMesh.from_vertices(*v)


def _unit_dirs(g: np.random.Generator, n: int) -> np.ndarray:
    d = g.standard_normal((n, 3), dtype=np.float32)
    nrm = np.sqrt((d * d).sum(1, keepdims=True))
    nrm[nrm == 0] = 1.0
    return d / nrm


def clustered(n: int, seed: int = 1, clusters: int = 64, sigma: float = 0.02) -> TriangleMesh:
    g = _rng(seed)
    means = g.random((clusters, 3), dtype=np.float32)
    which = g.integers(0, clusters, n)
    c = means[which] + g.standard_normal((n, 3), dtype=np.float32) * np.float32(sigma)
    edge = np.exp(g.uniform(np.log(1e-4), np.log(1e-2), n)).astype(np.float32)[:, None]
    v = [(c + _unit_dirs(g, n) * edge).astype(np.float32) for _ in range(3)]
    return TriangleMesh.from_vertices(*v)


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint64) * np.uint64(0x9E3779B1) ^ iy.astype(np.uint64) * np.uint64(0x85EBCA77)
         ^ iz.astype(np.uint64) * np.uint64(0xC2B2AE3D) ^ np.uint64(seed * 0x27D4EB2F + 0x165667B1))
    h = (h ^ (h >> np.uint64(15))) * np.uint64(0x2C1B3C6D)
    h = (h ^ (h >> np.uint64(12))) * np.uint64(0x297A2D39)
    h = h ^ (h >> np.uint64(15))
    return ((h & np.uint64(0xFFFFFF)).astype(np.float64) / float(0xFFFFFF)) * 2.0 - 1.0


def _value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    f = np.floor(p)
    t = p - f
    t = t * t * (3.0 - 2.0 * t)
    i = f.astype(np.int64) & 0xFFFFF
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = ((t[:, 0] if dx else 1 - t[:, 0]) * (t[:, 1] if dy else 1 - t[:, 1])
                     * (t[:, 2] if dz else 1 - t[:, 2]))
                out += w * _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
    return out


def _fbm(p: np.ndarray, seed: int, octaves: int = 4) -> np.ndarray:
    acc = np.zeros(p.shape[0])
    amp, freq = 0.5, 4.0
    for o in range(octaves):
        acc += amp * _value_noise(p * freq, seed + o)
        amp *= 0.5
        freq *= 2.0
    return acc


def icosphere(levels: int = 8, seed: int = 2, displacement: float = 0.05) -> TriangleMesh:
    """20 * 4**levels triangles (levels=8 gives 1,310,720)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                      [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                      [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                      [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    tri = verts[faces]  # (F, 3, 3), vertices duplicated per triangle
    for _ in range(levels):
        a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tri = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                        np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    pts = tri.reshape(-1, 3)
    # displacement is a function of the (unit) position, so shared vertices stay shared
    r = 1.0 + displacement * _fbm(pts, seed)
    pts = (pts * r[:, None]).astype(np.float32).reshape(-1, 3, 3)
    return TriangleMesh.from_vertices(pts[:, 0], pts[:, 1], pts[:, 2])


def strands(n_strands: int = 20000, segments: int = 100, seed: int = 3, step: float = 0.01,
            width: float = 1e-4) -> TriangleMesh:
    """n_strands * segments long thin triangles (defaults: 2,000,000)."""
    g = _rng(seed)
    start = g.random((n_strands, 1, 3))
    steps = _unit_dirs(g, n_strands * segments).astype(np.float64).reshape(n_strands, segments, 3) * step
    pts = np.concatenate([start, start + np.cumsum(steps, axis=1)], axis=1)
    # reflect into the unit cube
    pts = np.abs(pts)
    pts = np.where(pts > 1.0, 2.0 - pts, pts)
    pts = np.clip(pts, 0.0, 1.0)
    a = pts[:, :-1].reshape(-1, 3)
    b = pts[:, 1:].reshape(-1, 3)
    side = _unit_dirs(g, a.shape[0]).astype(np.float64)
    d = b - a
    perp = np.cross(d, side)
    nrm = np.linalg.norm(perp, axis=1, keepdims=True)
    nrm[nrm == 0] = 1.0
    c = a + perp / nrm * width
    return TriangleMesh.from_vertices(a.astype(np.float32), b.astype(np.float32), c.astype(np.float32))


def batch_counts(meshes: int = 4096, lo: int = 64, hi: int = 262144, seed: int = 4) -> np.ndarray:
    g = _rng(seed)
    return np.exp(g.uniform(np.log(lo), np.log(hi), meshes)).astype(np.int64)


def batch_meshes(counts, seed: int = 5):
    """One uniform_small mesh per count, each with its own seed, scale and offset."""
    g = _rng(seed)
    out = []
    for k, n in enumerate(counts):
        s = float(np.exp(g.uniform(np.log(0.1), np.log(10.0))))
        off = g.uniform(-10, 10, 3)
        out.append(uniform_small(int(n), seed=seed * 100003 + k, scale=s, offset=off))
    return out


def batch(counts, seed: int = 5):
    """All meshes of a batch concatenated: (TriangleMesh, offsets[count+1]).  Mesh k is a
    uniform_small-style mesh (centroids ~ U[0,1]^3, vertex offsets ~ U[-0.005,0.005]^3) scaled
    by s_k ~ logU[0.1, 10] and moved by o_k ~ U[-10, 10]^3."""
    counts = np.asarray(counts, np.int64)
    g = _rng(seed)
    total = int(counts.sum())
    offsets = np.zeros(counts.shape[0] + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    scale = np.exp(g.uniform(np.log(0.1), np.log(10.0), counts.shape[0])).astype(np.float32)
    off = g.uniform(-10, 10, (counts.shape[0], 3)).astype(np.float32)
    mesh_id = np.repeat(np.arange(counts.shape[0]), counts)
    s = scale[mesh_id][:, None]
    o = off[mesh_id]
    c = g.random((total, 3), dtype=np.float32)
    arrs = []
    for _ in range(3):
        v = c + (g.random((total, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.01)
        v *= s
        v += o
        arrs.append(v)
    del c, s, o, mesh_id
    return TriangleMesh.from_vertices(*arrs), offsets.astype(np.uint32)


def batch_subset(counts, meshes, seed: int = 5):
    """The selected meshes of a batch, concatenated: (TriangleMesh, offsets[len(meshes)+1]).  Mesh k
    is drawn from its own generator (seed, k) as in batch() -- centroids U[0,1]^3, vertex offsets
    U[-0.005,0.005]^3, scale logU[0.1, 10], shift U[-10, 10]^3 -- so any subset (one rank's share)
    is reproducible on its own."""
    counts = np.asarray(counts, np.int64)
    meshes = np.asarray(meshes, np.int64)
    total = int(counts[meshes].sum())
    arrs = [np.empty((total, 3), np.float32) for _ in range(3)]
    offsets = np.zeros(len(meshes) + 1, np.int64)
    o = 0
    for j, k in enumerate(meshes):
        g = np.random.default_rng([seed, int(k)])
        c = int(counts[k])
        scale = np.float32(np.exp(g.uniform(np.log(0.1), np.log(10.0))))
        off = g.uniform(-10, 10, 3).astype(np.float32)
        cen = g.random((c, 3), dtype=np.float32)
        for a in arrs:
            v = cen + (g.random((c, 3), dtype=np.float32) - np.float32(0.5)) * np.float32(0.01)
            a[o:o + c] = v * scale + off
        o += c
        offsets[j + 1] = o
    return TriangleMesh.from_vertices(*arrs), offsets.astype(np.uint32)


def scene_box(mesh: TriangleMesh):
    lo = np.array([min(mesh.v0x.min(), mesh.v1x.min(), mesh.v2x.min()),
                   min(mesh.v0y.min(), mesh.v1y.min(), mesh.v2y.min()),
                   min(mesh.v0z.min(), mesh.v1z.min(), mesh.v2z.min())], np.float64)
    hi = np.array([max(mesh.v0x.max(), mesh.v1x.max(), mesh.v2x.max()),
                   max(mesh.v0y.max(), mesh.v1y.max(), mesh.v2y.max()),
                   max(mesh.v0z.max(), mesh.v1z.max(), mesh.v2z.max())], np.float64)
    return lo, hi


def sphere_rays(mesh: TriangleMesh, n: int, seed: int = 6):
    """(origins, directions), each (n, 3) float32."""
    g = _rng(seed)
    lo, hi = scene_box(mesh)
    center = (lo + hi) / 2
    radius = 1.5 * np.linalg.norm(hi - lo) / 2
    o = center + _unit_dirs(g, n).astype(np.float64) * radius
    target = lo + g.random((n, 3)) * (hi - lo)
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)
