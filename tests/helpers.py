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


def compare_rays(got, ref_out, ref_hit, occl=False):
    """Ray parity: hit flags (grazing rays through shared edges or vertices
    may flip between two FP32 implementations: at most 1e-4 of the rays),
    hit distances within 1e-5 relative (absolute below 1), indices equal for
    99.9% of the common hits."""
    g_hit = got["index"] != R.UINT_MAX
    mism = g_hit != ref_hit
    assert mism.sum() <= max(2, int(1e-4 * len(got))), f"{mism.sum()} hit/miss disagreements"
    both = g_hit & ref_hit
    if not occl:
        tol = 1e-5 * np.maximum(ref_out["d"][both], 1.0)
        assert np.all(np.abs(got["d"][both] - ref_out["d"][both]) <= tol)
        same = got["index"][both] == ref_out["index"][both]
        assert same.mean() > 0.999


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
