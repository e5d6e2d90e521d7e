"""ctypes wrapper of the C oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as
the checker; the product never imports this module. Every function takes and
returns numpy arrays in the interop record layouts of fcpw_gb300.records.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import ORACLE_LIB, build_oracle

_lib = None
P = C.c_void_p


def _load():
    global _lib
    if _lib is None:
        path = build_oracle()
        _lib = C.CDLL(str(path))
        i, u, f = C.c_int, C.c_uint32, C.c_float
        sig = {
            "oracle_closest_points_bvh": [i, i, P, P, P, u, i, P, P, i],
            "oracle_closest_points_bvh_gpu_order": [i, i, P, P, P, u, P, P, i],
            "oracle_closest_points_brute": [i, P, u, P, u, P, i],
            "oracle_closest_points_brute_f64": [i, P, u, P, u, P, P, i],
            "oracle_intersect_rays_bvh": [i, i, P, P, P, u, i, P, P, i],
            "oracle_intersect_rays_brute_f64": [i, P, u, P, u, P, P, i],
            "oracle_silhouettes_bvh": [i, P, P, P, P, u, f, f, P, i],
            "oracle_sphere_sample_bvh": [i, i, P, P, P, P, u, P, P, i],
            "oracle_refit": [i, i, P, P, P],
            "oracle_prim_distance_f64": [i, P, u, P, P, u, P],
            "oracle_contains_bvh": [i, i, P, P, P, u, P, i],
            "oracle_line_of_sight_bvh": [i, i, P, P, P, P, u, P, i],
            "oracle_record_sizes": [P],
            "oracle_instanced_closest_points": [i, P, P, u, P, P, P, P, P, P, u, i, P, P],
            "oracle_instanced_rays": [i, P, P, u, P, P, P, P, P, P, u, i, P, P, P],
        }
        _lib.oracle_lbvh_build.restype = C.c_uint32
        _lib.oracle_lbvh_build.argtypes = [i, P, P, u, u, P, P, P]
        for name, args in sig.items():
            fn = getattr(_lib, name)
            fn.restype = C.c_int
            fn.argtypes = args
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def threads(n: int | None = None) -> int:
    return n if n else (os.cpu_count() or 1)


def _records():
    from fcpw_gb300 import records as R
    return R


def closest_points_bvh(dim, nodes, prims, spheres, record_normals=False, nthreads=None, visited=False,
                       gpu_order=False):
    """bvh.inl:1291-1418. With gpu_order the children are ordered as the
    reference's GPU traversal orders them (bvh.slang:458-470, by the smaller
    d2Min, the left child on ties), whose visit counts the GPU reference-order
    kernel's traversal statistics must match; the answers are the same."""
    R = _records()
    snch = nodes.dtype == R.SNCH_NODE
    out = R.default_interactions(len(spheres))
    nv = np.zeros(len(spheres), np.uint32) if visited else None
    if gpu_order:
        if record_normals:
            raise ValueError("gpu_order counts visits only; record_normals is not supported with it")
        _load().oracle_closest_points_bvh_gpu_order(dim, int(snch), _p(nodes), _p(prims), _p(spheres), len(spheres),
                                                    _p(out), _p(nv), threads(nthreads))
    else:
        _load().oracle_closest_points_bvh(dim, int(snch), _p(nodes), _p(prims), _p(spheres), len(spheres),
                                          int(record_normals), _p(out), _p(nv), threads(nthreads))
    return (out, nv) if visited else out


def closest_points_brute(dim, prims, spheres, nthreads=None):
    R = _records()
    out = R.default_interactions(len(spheres))
    _load().oracle_closest_points_brute(dim, _p(prims), len(prims), _p(spheres), len(spheres), _p(out),
                                        threads(nthreads))
    return out


def closest_points_brute_f64(dim, prims, spheres, nthreads=None):
    d = np.zeros(len(spheres), np.float64)
    idx = np.zeros(len(spheres), np.uint32)
    _load().oracle_closest_points_brute_f64(dim, _p(prims), len(prims), _p(spheres), len(spheres), _p(d), _p(idx),
                                            threads(nthreads))
    return d, idx


def _pts3(points):
    p = np.asarray(points, np.float32)
    out = np.zeros((len(p), 3), np.float32)
    out[:, : p.shape[1]] = p
    return out


def contains_bvh(dim, nodes, prims, points, nthreads=None):
    """Aggregate::contains for every point: 1 inside, 0 outside (2 if a ray had
    more hits than the oracle keeps)."""
    R = _records()
    snch = nodes.dtype == R.SNCH_NODE
    pts = _pts3(points)
    out = np.zeros(len(pts), np.uint32)
    _load().oracle_contains_bvh(dim, int(snch), _p(nodes), _p(prims), _p(pts), len(pts), _p(out), threads(nthreads))
    return out


def line_of_sight_bvh(dim, nodes, prims, points_a, points_b, nthreads=None):
    """Aggregate::hasLineOfSight for every pair: 1 visible, 0 occluded."""
    R = _records()
    snch = nodes.dtype == R.SNCH_NODE
    a, b = _pts3(points_a), _pts3(points_b)
    out = np.zeros(len(a), np.uint32)
    _load().oracle_line_of_sight_bvh(dim, int(snch), _p(nodes), _p(prims), _p(a), _p(b), len(a), _p(out),
                                     threads(nthreads))
    return out


def intersect_rays_bvh(dim, nodes, prims, rays, occlusion=False, nthreads=None):
    R = _records()
    snch = nodes.dtype == R.SNCH_NODE
    out = R.default_interactions(len(rays))
    hit = np.zeros(len(rays), np.int32)
    _load().oracle_intersect_rays_bvh(dim, int(snch), _p(nodes), _p(prims), _p(rays), len(rays), int(occlusion),
                                      _p(out), _p(hit), threads(nthreads))
    return out, hit.astype(bool)


def intersect_rays_brute_f64(dim, prims, rays, nthreads=None):
    t = np.zeros(len(rays), np.float64)
    idx = np.zeros(len(rays), np.uint32)
    _load().oracle_intersect_rays_brute_f64(dim, _p(prims), len(prims), _p(rays), len(rays), _p(t), _p(idx),
                                            threads(nthreads))
    return t, idx


def silhouettes_bvh(dim, snch_nodes, sils, spheres, flip, squared_min_radius=0.0, precision=1e-3, nthreads=None):
    R = _records()
    out = R.default_interactions(len(spheres))
    flip = np.ascontiguousarray(flip, np.uint32)
    _load().oracle_silhouettes_bvh(dim, _p(snch_nodes), _p(sils), _p(spheres), _p(flip), len(spheres),
                                   float(squared_min_radius), float(precision), _p(out), threads(nthreads))
    return out


def sphere_sample_bvh(dim, nodes, prims, spheres, rand_nums, nthreads=None):
    R = _records()
    snch = nodes.dtype == R.SNCH_NODE
    out = R.default_interactions(len(spheres))
    hit = np.zeros(len(spheres), np.int32)
    rn = np.ascontiguousarray(rand_nums, np.float32)
    _load().oracle_sphere_sample_bvh(dim, int(snch), _p(nodes), _p(prims), _p(spheres), _p(rn), len(spheres),
                                     _p(out), _p(hit), threads(nthreads))
    return out, hit.astype(bool)


def refit(dim, nodes, prims, sils=None):
    R = _records()
    nodes = nodes.copy()
    _load().oracle_refit(dim, int(nodes.dtype == R.SNCH_NODE), _p(nodes), _p(prims), _p(sils))
    return nodes


def prim_distance_f64(dim, prims, positions_in_array, points):
    """FP64 distance from points[q] to prims[positions_in_array[q]]."""
    pos = np.ascontiguousarray(positions_in_array, np.uint32)
    x = np.zeros((len(pos), 3), np.float32)
    pts = np.asarray(points, np.float32)
    x[:, : pts.shape[1]] = pts
    out = np.zeros(len(pos), np.float64)
    _load().oracle_prim_distance_f64(dim, _p(prims), len(prims), _p(pos), _p(x), len(pos), _p(out))
    return out


def lbvh_build(dim, positions, indices, max_leaf=4):
    """Sequential model of the device linear-BVH build: (nodes, primitives,
    prim_vertices) exactly as fcpwgb_gpu_scene_build must produce them."""
    R = _records()
    pos = np.ascontiguousarray(positions, np.float32)
    idx = np.ascontiguousarray(indices, np.int32)
    n = len(idx)
    nodes = np.zeros(max(2 * n - 1, 1), R.BVH_NODE)
    prims = np.zeros(n, R.TRIANGLE if dim == 3 else R.LINE_SEGMENT)
    pv = np.zeros((n, dim), np.int32)
    cnt = _load().oracle_lbvh_build(dim, _p(pos), _p(idx), n, int(max_leaf), _p(nodes), _p(prims), _p(pv))
    return nodes[:cnt], prims, pv


def _instanced_args(top_nodes, top_refs, mats, inst_object, inst_transformed, objects):
    k = len(objects)
    nodes = [np.ascontiguousarray(o[0]) for o in objects]
    prims = [np.ascontiguousarray(o[1]) for o in objects]
    np_ = (C.c_void_p * k)(*[a.ctypes.data for a in nodes])
    pp_ = (C.c_void_p * k)(*[a.ctypes.data for a in prims])
    keep = (nodes, prims, np_, pp_)
    tn = np.ascontiguousarray(top_nodes) if len(top_nodes) else None
    tr = np.ascontiguousarray(top_refs, np.uint32) if len(top_refs) else None
    return (keep, tn, tr, np.ascontiguousarray(mats, np.float32), np.ascontiguousarray(inst_object, np.uint32),
            np.ascontiguousarray(inst_transformed, np.uint32), np_, pp_)


def _chunked(n, nthreads, call):
    """Runs call(begin, end) over nthreads slices of [0, n) (the C calls release the GIL)."""
    k = max(1, min(threads(nthreads), n // 1024 or 1))
    bounds = [(n * t // k, n * (t + 1) // k) for t in range(k)]
    if k == 1:
        call(0, n)
        return
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(k) as ex:
        list(ex.map(lambda b: call(*b), bounds))


def instanced_closest_points(dim, top_nodes, top_refs, mats, inst_object, inst_transformed, objects, spheres,
                             record_normals=False, nthreads=None):
    """Closest points on a scene of several objects / instances (the
    reference's top-level walk with TransformedAggregate leaves). objects:
    per object (nodes, primitives) in the interop layouts; mats: (n, 24) as
    fcpwgb_cpu_instances_export gives them. Returns (interactions, instance)."""
    R = _records()
    keep, tn, tr, m, io, it, np_, pp_ = _instanced_args(top_nodes, top_refs, mats, inst_object, inst_transformed,
                                                        objects)
    out = R.default_interactions(len(spheres))
    inst = np.zeros(len(spheres), np.uint32)
    sp = np.ascontiguousarray(spheres)

    def call(b, e):
        _load().oracle_instanced_closest_points(dim, _p(tn), _p(tr), len(io), _p(m), _p(io), _p(it),
                                                C.cast(np_, C.c_void_p), C.cast(pp_, C.c_void_p),
                                                sp.ctypes.data + b * sp.itemsize, e - b, int(record_normals),
                                                out.ctypes.data + b * out.itemsize, inst.ctypes.data + 4 * b)

    _chunked(len(sp), nthreads, call)
    del keep
    return out, inst


def instanced_rays(dim, top_nodes, top_refs, mats, inst_object, inst_transformed, objects, rays, occlusion=False,
                   nthreads=None):
    """Ray queries on a scene of several objects / instances. Returns
    (interactions, hit, instance)."""
    R = _records()
    keep, tn, tr, m, io, it, np_, pp_ = _instanced_args(top_nodes, top_refs, mats, inst_object, inst_transformed,
                                                        objects)
    out = R.default_interactions(len(rays))
    hit = np.zeros(len(rays), np.int32)
    inst = np.zeros(len(rays), np.uint32)
    rr = np.ascontiguousarray(rays)

    def call(b, e):
        _load().oracle_instanced_rays(dim, _p(tn), _p(tr), len(io), _p(m), _p(io), _p(it), C.cast(np_, C.c_void_p),
                                      C.cast(pp_, C.c_void_p), rr.ctypes.data + b * rr.itemsize, e - b,
                                      int(occlusion), out.ctypes.data + b * out.itemsize, hit.ctypes.data + 4 * b,
                                      inst.ctypes.data + 4 * b)

    _chunked(len(rr), nthreads, call)
    del keep
    return out, hit.astype(bool), inst


def record_sizes():
    s = (C.c_int * 9)()
    _load().oracle_record_sizes(s)
    return list(s)
