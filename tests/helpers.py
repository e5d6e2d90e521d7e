"""Shared comparison logic for the parity tests.

Tolerances (written here once, used by every test):

* FP32 distance parity with the oracle (the reference CPU algorithm in FP32):
  ``|d_gpu - d_ref| <= 1e-6 * d_ref + 4 * eps32 * S`` with ``S = |x|_inf + |p|_inf``.
  The second term is the rounding floor of computing a distance from absolute
  FP32 coordinates (the reference forms ``x - p`` with ``p`` rounded to the
  ulp of its coordinates), so it is the least two correct FP32
  implementations can be expected to agree to.
* Index parity: indices are equal, or the two primitives are tied: their FP64
  distances to the query agree within twice the distance tolerance.
* Accuracy against FP64 for refined results: ``|d - d64| <= 1e-6 * d64``.
* Rays (compare_rays): hit flags equal except on grazing hits (the FP64 hit
  point within GRAZE * eps32 * (|o| + |x|) / cos of the primitive's
  boundary), hit distances within 1e-6 relative for equal indices, and every
  index mismatch an equidistant tie or a grazed nearer primitive.
"""
from __future__ import annotations

import numpy as np

from fcpw_gb300 import records as R
from oracle import oracle as O

EPS32 = float(np.finfo(np.float32).eps)
REL = 1e-6


def distance_tolerance(points, p, d):
    pts = np.asarray(points, np.float64)
    S = np.abs(pts).max(axis=1) + np.abs(np.asarray(p, np.float64)).max(axis=1)
    return REL * np.asarray(d, np.float64) + 4.0 * EPS32 * S


def leaf_positions(prims):
    """original primitive index -> position in the leaf-ordered primitive array"""
    pos = np.empty(len(prims), np.int64)
    pos[prims["index"].astype(np.int64)] = np.arange(len(prims))
    return pos


def compare_closest(dim, prims, points, got, ref, what="closest point"):
    """Asserts found-flags, distances within tolerance and tie-aware index parity.
    Returns a dict of statistics."""
    fg = got["index"] != R.UINT_MAX
    fr = ref["index"] != R.UINT_MAX
    assert np.array_equal(fg, fr), f"{what}: found/not-found differs for {np.count_nonzero(fg != fr)} queries"
    m = fr
    pts = np.asarray(points)[m]
    tol = distance_tolerance(pts, ref["p"][m][:, :pts.shape[1]], ref["d"][m])
    dd = np.abs(got["d"][m].astype(np.float64) - ref["d"][m].astype(np.float64))
    bad = dd > tol
    assert not bad.any(), (f"{what}: {np.count_nonzero(bad)} distances outside tolerance, worst "
                           f"|dd|={dd[bad].max():.3e} tol={tol[bad][np.argmax(dd[bad])]:.3e}")
    mism = got["index"][m] != ref["index"][m]
    n_ties = int(np.count_nonzero(mism))
    if n_ties:
        lp = leaf_positions(prims)
        gi = lp[got["index"][m][mism].astype(np.int64)]
        ri = lp[ref["index"][m][mism].astype(np.int64)]
        dg = O.prim_distance_f64(dim, prims, gi, pts[mism])
        dr = O.prim_distance_f64(dim, prims, ri, pts[mism])
        bad = np.abs(dg - dr) > 2.0 * tol[mism]
        assert not bad.any(), f"{what}: {np.count_nonzero(bad)} index mismatches that are not ties"
    return {"n": int(len(m)), "found": int(np.count_nonzero(m)), "index_ties": n_ties,
            "max_abs_dd": float(dd.max()) if len(dd) else 0.0}


GRAZE = 16.0  # grazing band, in units of the FP32 rounding of the hit point over the incidence cosine


def _prim_vertices(dim, prims, pos):
    """FP64 vertices (n, dim, 3) of the primitives at leaf positions pos."""
    if dim == 3:
        return np.stack([prims["pa"][pos], prims["pb"][pos], prims["pc"][pos]], axis=1).astype(np.float64)
    v = np.stack([prims["pa"][pos], prims["pb"][pos]], axis=1).astype(np.float64)
    v[..., 2] = 0.0
    return v


def ray_prim_f64(dim, verts, o, d):
    """FP64 ray-primitive geometry for rays o + t d against primitives verts
    (rows paired with the rays): the plane (3D) or line (2D) parameter t, the
    signed distance `margin` of that hit point from the primitive's boundary
    within the primitive's plane (positive inside; the triangle's edges, the
    segment's endpoints), the incidence cosine |n.d|/(|n||d|), and the
    grazing band of an FP32 test: GRAZE * eps32 * (|o|inf + |x|inf) / cos, x
    the hit point. A hit whose margin lies within that band of 0 is grazing:
    two correct FP32 evaluations may disagree on it."""
    o = np.asarray(o, np.float64)
    d = np.asarray(d, np.float64)
    if dim == 3:
        a, b, c = verts[:, 0], verts[:, 1], verts[:, 2]
        n = np.cross(b - a, c - a)
        nn = np.linalg.norm(n, axis=1)
        den = np.einsum("ij,ij->i", n, d)
        with np.errstate(divide="ignore", invalid="ignore"):
            t = np.einsum("ij,ij->i", n, a - o) / den
            x = o + t[:, None] * d
            nh = n / nn[:, None]
            m = np.full(len(o), np.inf)
            for p0, p1 in ((a, b), (b, c), (c, a)):
                e = p1 - p0
                m = np.minimum(m, np.einsum("ij,ij->i", np.cross(e, x - p0), nh) / np.linalg.norm(e, axis=1))
            cos = np.abs(den) / (nn * np.linalg.norm(d, axis=1))
    else:
        a, b = verts[:, 0, :2], verts[:, 1, :2]
        o2, d2 = o[:, :2], d[:, :2]
        v = b - a
        L = np.linalg.norm(v, axis=1)
        den = d2[:, 0] * v[:, 1] - d2[:, 1] * v[:, 0]
        u = a - o2
        with np.errstate(divide="ignore", invalid="ignore"):
            t = (u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0]) / den
            s = (u[:, 0] * d2[:, 1] - u[:, 1] * d2[:, 0]) / den
            x = o + t[:, None] * d
            m = np.minimum(s, 1.0 - s) * L
            cos = np.abs(den) / (L * np.linalg.norm(d2, axis=1))
    S = np.abs(o).max(axis=1) + np.abs(np.nan_to_num(x, nan=0.0, posinf=0.0, neginf=0.0)).max(axis=1)
    with np.errstate(divide="ignore"):
        band = GRAZE * EPS32 * S / np.maximum(cos, 1e-30)
    return t, m, cos, band


def _grazing(dim, prims, pos, o, d, tmax):
    """True where the ray's FP64 hit of that primitive lies within the grazing
    band of its boundary (and of the ray's [0, tMax] range)."""
    t, m, _, band = ray_prim_f64(dim, _prim_vertices(dim, prims, pos), o, d)
    near_edge = np.abs(m) <= band
    tol_t = band * np.linalg.norm(np.asarray(d, np.float64), axis=1)
    in_range = (t >= -tol_t) & (t <= np.asarray(tmax, np.float64) + tol_t)
    return near_edge & in_range, t, m >= -band


def _clear_hits_f64(dim, prims, o, d, tmax):
    """For each ray (few), whether some primitive is hit in FP64 with its hit
    point inside by more than the grazing band (a hit no FP32 evaluation may
    miss), by brute force over all primitives."""
    out = np.zeros(len(o), bool)
    allpos = np.arange(len(prims))
    V = _prim_vertices(dim, prims, allpos)
    for k in range(len(o)):
        ok = np.repeat(np.asarray(o[k], np.float64)[None], len(prims), 0)
        dk = np.repeat(np.asarray(d[k], np.float64)[None], len(prims), 0)
        t, m, _, band = ray_prim_f64(dim, V, ok, dk)
        out[k] = bool(np.any((m > band) & (t >= 0) & (t <= float(tmax[k]))))
    return out


def compare_rays(dim, prims, rays, got, ref, ref_hit, occl=False, floor=False, what="rays"):
    """Ray parity against the reference (the reference's own answers or the
    oracle's restatement of them), no percentage allowances:

    * a ray hits in both or in neither, except where the hit is grazing: the
      primitive that one side hit is grazed in FP64 (its hit point lies within
      GRAZE * eps32 * (|o| + |x|) / cos of the primitive's boundary); when the
      reference reports an occlusion the GPU did not, no primitive may be hit
      in FP64 clearly inside (brute force over the scene);
    * equal indices: hit distances within 1e-6 relative (floor=True adds the
      FP32 rounding floor 4 eps32 (|o| + |x|) of rays that went through a
      transform);
    * different indices: an equidistant tie (both primitives' FP64 hit
      parameters agree within the grazing band along the ray, both hit or
      grazed), or the nearer primitive is grazed (one side passed it by the
      grazing band and hit the next one behind).
    Returns counts of each kind."""
    rays = np.asarray(rays)
    rf = rays.view(np.float32).reshape(len(rays), 10).astype(np.float64)
    o, d, tmax = rf[:, 0:3], rf[:, 3:6], rf[:, 9]
    lp = leaf_positions(prims)
    g_hit = got["index"] != R.UINT_MAX
    r_hit = np.asarray(ref_hit, bool)
    stats = {"n": int(len(rays)), "hits": int(np.count_nonzero(r_hit)), "flips": 0, "ties": 0, "grazed": 0}
    flip = g_hit != r_hit
    if flip.any():
        k = np.nonzero(flip)[0]
        # the side that hit names its primitive (an occlusion answer of the reference names none)
        gk = k[g_hit[k]]
        if len(gk):
            gz, _, _ = _grazing(dim, prims, lp[got["index"][gk].astype(np.int64)], o[gk], d[gk], tmax[gk])
            assert gz.all(), f"{what}: {np.count_nonzero(~gz)} GPU hits the reference misses are not grazing"
        rk = k[r_hit[k]]
        if len(rk):
            if occl:
                clear = _clear_hits_f64(dim, prims, o[rk], d[rk], tmax[rk])
                assert not clear.any(), f"{what}: {np.count_nonzero(clear)} occlusions missed with a clear FP64 hit"
            else:
                gz, _, _ = _grazing(dim, prims, lp[ref["index"][rk].astype(np.int64)], o[rk], d[rk], tmax[rk])
                assert gz.all(), f"{what}: {np.count_nonzero(~gz)} reference hits the GPU misses are not grazing"
        stats["flips"] = int(len(k))
    if occl:
        return stats
    both = g_hit & r_hit
    same = both & (got["index"] == ref["index"])
    dr = ref["d"][same].astype(np.float64)
    tol = REL * dr
    if floor:
        x = ref["p"][same].astype(np.float64)
        tol = tol + 4.0 * EPS32 * (np.abs(o[same]).max(1) + np.abs(x).max(1))
    dd = np.abs(got["d"][same].astype(np.float64) - dr)
    assert np.all(dd <= tol), (f"{what}: {np.count_nonzero(dd > tol)} hit distances outside 1e-6 relative, "
                               f"worst {np.max(dd / np.maximum(dr, 1e-30)):.3e}")
    diff = np.nonzero(both & ~same)[0]
    if len(diff):
        pg = lp[got["index"][diff].astype(np.int64)]
        pr = lp[ref["index"][diff].astype(np.int64)]
        gz_g, tg, in_g = _grazing(dim, prims, pg, o[diff], d[diff], tmax[diff])
        gz_r, tr, in_r = _grazing(dim, prims, pr, o[diff], d[diff], tmax[diff])
        _, _, _, band_g = ray_prim_f64(dim, _prim_vertices(dim, prims, pg), o[diff], d[diff])
        _, _, _, band_r = ray_prim_f64(dim, _prim_vertices(dim, prims, pr), o[diff], d[diff])
        dn = np.linalg.norm(d[diff], axis=1)
        tie = (np.abs(tg - tr) * dn <= np.maximum(band_g, band_r)) & in_g & in_r
        nearer_grazed = np.where(got["d"][diff] < ref["d"][diff], gz_g, gz_r)
        ok = tie | nearer_grazed
        assert ok.all(), f"{what}: {np.count_nonzero(~ok)} index mismatches that are neither ties nor grazing"
        stats["ties"] = int(np.count_nonzero(tie))
        stats["grazed"] = int(np.count_nonzero(~tie))
    return stats


def edge_aimed_rays(verts, tris, o, seed):
    """Directions from the origins o towards edge midpoints and vertices of
    random triangles (half each): rays that graze edges and pass through
    vertices, where FP32 evaluations tie or disagree."""
    rng = np.random.default_rng(seed)
    m = len(o)
    tri = rng.integers(0, len(tris), m)
    k = rng.integers(0, 3, m)
    a = np.asarray(verts, np.float64)[tris[tri, k]]
    b = np.asarray(verts, np.float64)[tris[tri, (k + 1) % 3]]
    target = a + np.where(rng.random(m) < 0.5, 0.5, 0.0)[:, None] * (b - a)
    d = target - np.asarray(o, np.float64)
    return (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)


def relative_error(d, d64):
    d64 = np.asarray(d64, np.float64)
    m = np.isfinite(d64) & (d64 > 0)
    return np.abs(np.asarray(d, np.float64)[m] - d64[m]) / d64[m]


def build_scene(dim, verts, idx, silhouettes=False, aggregate=None):
    import fcpw_gb300 as F
    s = F.Scene3D() if dim == 3 else F.Scene2D()
    s.set_object_count(1)
    s.set_object_vertices(verts, 0)
    if dim == 3:
        s.set_object_triangles(idx, 0)
    else:
        s.set_object_line_segments(idx, 0)
    if silhouettes:
        s.compute_silhouettes()
    s.build(aggregate if aggregate is not None else F.AggregateType.Bvh_SurfaceArea, False)
    return s
