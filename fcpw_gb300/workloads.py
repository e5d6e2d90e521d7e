"""Seeded synthetic scenes and queries for the benchmark and test workloads.

No dataset is involved; every mesh and query set is generated from
``numpy.random.Generator(PCG64(seed))``:

* ``geodesic_sphere(freq)``: icosahedron faces split into freq^2 triangles and
  projected to the unit sphere (freq = 2^k is the k-times subdivided icosphere:
  freq 32 gives 20,480 triangles / 10,242 vertices; freq 100 gives 200,000).
* ``perturbed_sphere``: vertex radius 1 + sigma*N(0,1), smoothed by
  ``smooth_passes`` uniform-Laplacian passes r <- (r + mean(neighbour r)) / 2.
* ``torus(nu, nv)``: R = 1, r = 0.3, nu x nv quads split into 2 triangles,
  minor radius scaled by 1 + noise*N(0,1) per vertex (1024 x 512 -> 1,048,576 triangles).
* ``star_polylines``: closed stars, radius 1 + 0.3 sin(k theta + phi),
  k ~ U{3..12}, phi ~ U[0, 2pi), scaled by ``scale`` and centred on a square
  grid covering [-extent, extent]^2.
* ``batched_meshes``: the uneven-batch workload, n meshes with triangle counts
  log-uniform in [1e3, 2e5] realised as the nearest perturbed geodesic sphere
  (20 freq^2) or torus (2 nu nv) count, kinds 50/50, and query counts
  log-uniform in [1e3, 1e6], queries uniform in each mesh's bounding cube
  grown by a quarter of its side on every side.
"""
from __future__ import annotations

import functools

import numpy as np

SEED_BASE = 20261203


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


@functools.lru_cache(maxsize=None)
def _geodesic_sphere_cached(freq: int):
    v, f = _geodesic_sphere(freq)
    v.setflags(write=False)
    f.setflags(write=False)
    return v, f


def geodesic_sphere(freq: int):
    """Unit geodesic sphere with 20*freq^2 triangles (shared vertices)."""
    v, f = _geodesic_sphere_cached(freq)
    return v.copy(), f.copy()


def _geodesic_sphere(freq: int):
    v0, f0 = _icosahedron()
    pts, tris = [], []
    base = 0
    # barycentric lattice per face: (i, j) with i + j <= freq
    ij = [(i, j) for i in range(freq + 1) for j in range(freq + 1 - i)]
    lid = {p: k for k, p in enumerate(ij)}
    local = []
    for i in range(freq):
        for j in range(freq - i):
            local.append((lid[(i, j)], lid[(i + 1, j)], lid[(i, j + 1)]))
            if i + j < freq - 1:
                local.append((lid[(i + 1, j)], lid[(i + 1, j + 1)], lid[(i, j + 1)]))
    local = np.array(local, np.int64)
    w = np.array(ij, np.float64) / freq
    for a, b, c in f0:
        p = v0[a] * (1 - w[:, :1] - w[:, 1:2]) + v0[b] * w[:, :1] + v0[c] * w[:, 1:2]
        pts.append(p)
        tris.append(local + base)
        base += len(ij)
    pts = np.concatenate(pts)
    tris = np.concatenate(tris)
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    # weld duplicated face-boundary vertices
    key = np.round(pts * 1e7).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)
    remap = np.empty_like(order)
    remap[order] = np.arange(len(order))
    verts = pts[first[order]]
    tris = remap[inv.reshape(-1)[tris]]
    return verts, tris.astype(np.int32)


def _vertex_neighbours(n_vertices: int, tris: np.ndarray):
    """Both directions of every mesh edge, each once, ordered by (src, dst)."""
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]).astype(np.int64)
    key = np.unique(np.concatenate([e[:, 0] * n_vertices + e[:, 1], e[:, 1] * n_vertices + e[:, 0]]))
    return key // n_vertices, key % n_vertices


@functools.lru_cache(maxsize=None)
def _sphere_neighbours(freq: int):
    verts, tris = _geodesic_sphere_cached(freq)
    src, dst = _vertex_neighbours(len(verts), tris)
    deg = np.bincount(src, minlength=len(verts)).astype(np.float64)
    for a in (src, dst, deg):
        a.setflags(write=False)
    return src, dst, deg


def perturbed_sphere(freq: int, seed: int, sigma: float = 0.1, smooth_passes: int = 2):
    verts, tris = geodesic_sphere(freq)
    g = rng(seed)
    r = 1.0 + sigma * g.standard_normal(len(verts))
    src, dst, deg = _sphere_neighbours(freq)
    for _ in range(smooth_passes):
        mean = np.bincount(src, weights=r[dst], minlength=len(verts)) / deg
        r = 0.5 * (r + mean)
    return (verts * r[:, None]).astype(np.float32), tris


def torus(nu: int, nv: int, seed: int, R: float = 1.0, r: float = 0.3, noise: float = 0.02):
    g = rng(seed)
    u = 2 * np.pi * np.arange(nu) / nu
    v = 2 * np.pi * np.arange(nv) / nv
    uu, vv = np.meshgrid(u, v, indexing="ij")
    rr = r * (1.0 + noise * g.standard_normal(uu.shape))
    x = (R + rr * np.cos(vv)) * np.cos(uu)
    y = (R + rr * np.cos(vv)) * np.sin(uu)
    z = rr * np.sin(vv)
    verts = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float32)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    t1 = np.stack([a, b, c], -1).reshape(-1, 3)
    t2 = np.stack([a, c, d], -1).reshape(-1, 3)
    tris = np.empty((2 * len(t1), 3), np.int64)
    tris[0::2] = t1
    tris[1::2] = t2
    return verts, tris.astype(np.int32)


def star_polylines(n_stars: int, segs_per_star: int, seed: int, extent: float = 3.0, scale: float = 0.14):
    g = rng(seed)
    side = int(np.ceil(np.sqrt(n_stars)))
    cell = 2 * extent / side
    verts, segs = [], []
    base = 0
    theta = 2 * np.pi * np.arange(segs_per_star) / segs_per_star
    for s in range(n_stars):
        k = g.integers(3, 13)
        phi = g.uniform(0, 2 * np.pi)
        rad = scale * (1 + 0.3 * np.sin(k * theta + phi))
        cx = -extent + cell * (s % side + 0.5)
        cy = -extent + cell * (s // side + 0.5)
        verts.append(np.stack([cx + rad * np.cos(theta), cy + rad * np.sin(theta)], -1))
        idx = np.arange(segs_per_star)
        segs.append(np.stack([base + idx, base + (idx + 1) % segs_per_star], -1))
        base += segs_per_star
    return np.concatenate(verts).astype(np.float32), np.concatenate(segs).astype(np.int32)


def uniform_points(n: int, dim: int, lo: float, hi: float, seed: int) -> np.ndarray:
    return rng(seed).uniform(lo, hi, size=(n, dim)).astype(np.float32)


def uniform_directions(n: int, dim: int, seed: int) -> np.ndarray:
    d = rng(seed).standard_normal((n, dim))
    return (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


def batched_meshes(n_meshes: int = 512, seed: int = SEED_BASE + 5, tri_range=(1e3, 2e5), query_range=(1e3, 1e6)):
    """Returns (meshes, query_counts, query_boxes): meshes[k] = (vertices, triangles),
    query_boxes[k] = (lo, hi) of the cube the queries of mesh k are drawn from."""
    g = rng(seed)
    tris = np.exp(g.uniform(np.log(tri_range[0]), np.log(tri_range[1]), n_meshes))
    counts = np.exp(g.uniform(np.log(query_range[0]), np.log(query_range[1]), n_meshes)).astype(np.int64)
    kinds = g.integers(0, 2, n_meshes)
    meshes, boxes = [], []
    for k in range(n_meshes):
        if kinds[k] == 0:
            freq = max(2, int(round(np.sqrt(tris[k] / 20.0))))
            v, f = perturbed_sphere(freq, seed + 1000 + k)
        else:
            nu = max(4, int(round(np.sqrt(tris[k]))))
            nv = max(3, int(round(tris[k] / (2.0 * nu))))
            v, f = torus(nu, nv, seed + 1000 + k)
        lo, hi = v.min(0), v.max(0)
        c, side = (lo + hi) / 2, float((hi - lo).max()) * 1.5
        meshes.append((v, f))
        boxes.append((c - side / 2, c + side / 2))
    return meshes, counts, boxes


def batched_queries(counts, boxes, seed: int) -> np.ndarray:
    """Queries of all meshes, grouped by mesh: uniform in each mesh's cube."""
    g = rng(seed)
    out = np.empty((int(np.sum(counts)), 3), np.float32)
    o = 0
    for nq, (lo, hi) in zip(counts, boxes):
        out[o:o + nq] = g.uniform(lo, hi, size=(int(nq), 3))
        o += int(nq)
    return out
