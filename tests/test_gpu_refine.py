"""Precise mode across conditioning regimes: queries from 1 down to 1e-8 edge
lengths off the faces, edges and vertices of large triangles (and segments),
sliver triangles, queries far from small primitives, and scenes scaled from
1e-3 to 1e9. The refinement runs in double-single arithmetic where the
projection is well conditioned and in FP64 elsewhere (Tri48Prim::refine);
every regime stays within 1e-6 of the FP64 brute-force distance. (Much
smaller scenes are out of reach of the FP32 traversal itself: products of
dot products in the closest-point routine, about edge^4, turn subnormal, so
the traversal can pick a wrong primitive that no refinement repairs.)"""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from helpers import build_scene, relative_error
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def cell_triangles(rng, sliver=False):
    """One triangle per cell of a 4x4x4 grid (spacing 3), edges about 1..2:
    a query near one triangle has no other one nearby."""
    tris = []
    for c in np.stack(np.meshgrid(*[np.arange(4)] * 3, indexing="ij"), -1).reshape(-1, 3):
        centre = 3.0 * c.astype(np.float64)
        a, b = rng.normal(size=3), rng.normal(size=3)
        a /= np.linalg.norm(a)
        b -= a * (a @ b)
        b /= np.linalg.norm(b)
        if sliver:  # aspect ratio 1e2..1e3
            w = 10.0 ** -rng.uniform(2, 3)
            t = np.array([-0.8 * a, 0.8 * a, w * b + rng.uniform(-0.5, 0.5) * a])
        else:
            ang = np.sort(rng.uniform(0, 2 * np.pi, 3))
            t = np.array([np.cos(q) * a + np.sin(q) * b for q in ang]) * rng.uniform(0.6, 1.0)
        tris.append(centre + t)
    v = np.concatenate(tris).astype(np.float32)
    return v, np.arange(len(v), dtype=np.int32).reshape(-1, 3)


def near_queries(rng, v, f, n, kmax):
    """Per query a triangle, a base point on its face, an edge or a vertex,
    and an outward offset of 10^-k edge lengths, k in [0, kmax]."""
    t = rng.integers(0, len(f), n)
    a, b, c = (v[f[t, j]].astype(np.float64) for j in range(3))
    nrm = np.cross(b - a, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    edge = np.linalg.norm(b - a, axis=1)
    kind = rng.integers(0, 3, n)
    u1, u2 = rng.uniform(0, 1, n), rng.uniform(0, 1, n)
    flip = u1 + u2 > 1
    u1[flip], u2[flip] = 1 - u1[flip], 1 - u2[flip]
    base = a + u1[:, None] * (b - a) + u2[:, None] * (c - a)
    lam = rng.uniform(0, 1, n)[:, None]
    on_edge = a + lam * (b - a)
    out_edge = np.cross(b - a, nrm)
    out_edge *= np.sign(np.sum(out_edge * (on_edge - c), 1))[:, None]
    out_edge /= np.linalg.norm(out_edge, axis=1, keepdims=True)
    phi = rng.uniform(-1.2, 1.2, n)[:, None]
    away = rng.normal(size=(n, 3))
    away /= np.linalg.norm(away, axis=1, keepdims=True)
    p0 = np.where((kind == 0)[:, None], base, np.where((kind == 1)[:, None], on_edge, a))
    u = np.where((kind == 0)[:, None], nrm * np.where(rng.uniform(0, 1, n) < 0.5, -1, 1)[:, None],
                 np.where((kind == 1)[:, None], np.cos(phi) * out_edge + np.sin(phi) * nrm, away))
    d = edge * 10.0 ** -rng.uniform(0, kmax, n)
    return (p0 + d[:, None] * u).astype(np.float32)


def precise_errors(dim, v, idx, pts, **cfg):
    s = build_scene(dim, v, idx)
    g = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    g.transfer_to_gpu(s)
    g.set_traversal(precise=True, **cfg)
    out = F.GPUInteractionList()
    g.find_closest_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    got = out.array()
    _, prims, _ = s.cpu_bvh.export()
    d64, _ = O.closest_points_brute_f64(dim, prims, R.make_spheres(pts, R.FLT_MAX))
    assert g.check_errors() == 0
    return relative_error(got["d"], d64)


@pytest.mark.parametrize("scale,kmax", [(1.0, 8), (1e4, 8), (1e9, 8), (1e-3, 6)])
@pytest.mark.parametrize("cfg", [dict(branching=4, bits=32, packet=True), dict(branching=4, bits=8, packet=False)])
def test_near_surface_queries_within_1e6(scale, kmax, cfg):
    rng = np.random.default_rng(71)
    v, f = cell_triangles(rng)
    pts = near_queries(rng, v, f, 12000, kmax)
    rel = precise_errors(3, (v * np.float32(scale)).astype(np.float32), f,
                         (pts * np.float32(scale)).astype(np.float32), **cfg)
    assert rel.max() <= 1e-6, f"scale {scale}: max relative error {rel.max():.3e}"


def test_sliver_triangles_within_1e6():
    """Slivers take the FP64 path near the surface (cond = s |ab| |ac| /
    (|n| d) grows with the aspect ratio). Much thinner ones are out of reach
    of the FP32 traversal: its barycentric terms cancel and a wrong
    primitive can win."""
    rng = np.random.default_rng(72)
    v, f = cell_triangles(rng, sliver=True)
    pts = near_queries(rng, v, f, 12000, 8)
    rel = precise_errors(3, v, f, pts, branching=4, bits=32, packet=True)
    assert rel.max() <= 1e-6, f"max relative error {rel.max():.3e}"


def test_far_queries_within_1e6():
    """Small triangles, queries 10 to 1e4 edge lengths away: the projection
    is well conditioned however small d is against the scene."""
    rng = np.random.default_rng(73)
    v, f = cell_triangles(rng)
    v = (v * np.float32(1e-3)).astype(np.float32)
    dirs = rng.normal(size=(8000, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    pts = (dirs * 10.0 ** rng.uniform(-2, 1, (8000, 1))).astype(np.float32)
    rel = precise_errors(3, v, f, pts, branching=4, bits=32, packet=True)
    assert rel.max() <= 1e-6, f"max relative error {rel.max():.3e}"


@pytest.mark.parametrize("scale", [1.0, 1e9])
def test_segments_near_queries_within_1e6(scale):
    rng = np.random.default_rng(74)
    cells = np.stack(np.meshgrid(np.arange(8), np.arange(8), indexing="ij"), -1).reshape(-1, 2) * 3.0
    ang = rng.uniform(0, 2 * np.pi, len(cells))
    half = np.stack([np.cos(ang), np.sin(ang)], 1) * rng.uniform(0.5, 1.0, (len(cells), 1))
    v = np.concatenate([cells - half, cells + half]).astype(np.float32)
    k = len(cells)
    sg = np.stack([np.arange(k), np.arange(k) + k], 1).astype(np.int32)
    n = 12000
    t = rng.integers(0, k, n)
    a, b = v[sg[t, 0]].astype(np.float64), v[sg[t, 1]].astype(np.float64)
    e = b - a
    L = np.linalg.norm(e, axis=1)
    nrm = np.stack([-e[:, 1], e[:, 0]], 1) / L[:, None]
    kind = rng.integers(0, 2, n)
    lam = rng.uniform(0, 1, n)[:, None]
    side = np.where(rng.uniform(0, 1, n) < 0.5, -1.0, 1.0)[:, None]
    ang2 = rng.uniform(-1.5, 1.5, n)
    tip = -e / L[:, None]
    away = np.cos(ang2)[:, None] * tip + np.sin(ang2)[:, None] * nrm
    p0 = np.where((kind == 0)[:, None], a + lam * e, a)
    u = np.where((kind == 0)[:, None], side * nrm, away)
    d = L * 10.0 ** -rng.uniform(0, 8, n)
    pts = ((p0 + d[:, None] * u) * scale).astype(np.float32)
    rel = precise_errors(2, (v * np.float32(scale)).astype(np.float32), sg, pts, branching=4, bits=32, packet=True)
    assert rel.max() <= 1e-6, f"scale {scale}: max relative error {rel.max():.3e}"
