"""ctypes wrapper of oracle/_ref/libfcpw_ref.so, the reference's own CPU Scene
compiled from its sources (TEST INFRASTRUCTURE ONLY; available where the
reference headers are staged, see build.py), and of oracle/_ref/libfcpw_ref_simd.so,
the same built with Enoki packets for the reference's vectorised Mbvh (timing only)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build import build_reference, build_reference_simd

_libs = {}
P = C.c_void_p


def available(simd: bool = False) -> bool:
    try:
        return (build_reference_simd() if simd else build_reference()) is not None
    except RuntimeError:
        return False


def _load(simd: bool = False):
    if simd not in _libs:
        path = build_reference_simd() if simd else build_reference()
        if path is None:
            raise RuntimeError("the reference headers are not staged on this machine")
        lib = C.CDLL(str(path))
        i, f = C.c_int, C.c_float
        lib.ref_scene_create.restype = P
        lib.ref_scene_create.argtypes = [i, P, i, P, i, i, i]
        lib.ref_scene_create_ex.restype = P
        lib.ref_scene_create_ex.argtypes = [i, P, i, P, i, i, i, i]
        lib.ref_scene_destroy.argtypes = [P]
        lib.ref_scene_create_multi.restype = P
        lib.ref_scene_create_multi.argtypes = [i, i, P, P, P, P, P, P, i]
        lib.ref_scene_create_multi_ex.restype = P
        lib.ref_scene_create_multi_ex.argtypes = [i, i, P, P, P, P, P, P, i, i]
        lib.ref_simd_width.restype = i
        lib.ref_simd_width.argtypes = []
        for name, args in {"ref_scene_closest_points_timed": [P, P, i, P],
                           "ref_scene_intersect_rays_timed": [P, P, i, i, P],
                           "ref_scene_silhouettes_timed": [P, P, P, i, P]}.items():
            fn = getattr(lib, name)
            fn.restype = C.c_double
            fn.argtypes = args
        for name, args in {"ref_export": [P, P, P, P, P], "ref_closest_points": [P, P, i, i, P, P],
                           "ref_intersect_rays": [P, P, i, i, P, P], "ref_silhouettes": [P, P, P, i, f, f, P],
                           "ref_sphere_sample": [P, P, P, i, P, P], "ref_update_and_refit": [P, P, i],
                           "ref_contains": [P, P, i, P], "ref_line_of_sight": [P, P, P, i, P],
                           "ref_closest_points_objects": [P, P, i, i, P, P],
                           "ref_intersect_rays_objects": [P, P, i, i, P, P, P],
                           "ref_export_top": [P, P, P],
                           "ref_silhouettes_objects": [P, P, P, i, f, f, P, P],
                           "ref_sphere_sample_objects": [P, P, P, i, P, P, P],
                           "ref_update_object_and_refit": [P, i, P, i]}.items():
            fn = getattr(lib, name)
            fn.restype = i
            fn.argtypes = args
        _libs[simd] = lib
    return _libs[simd]


def simd_width() -> int:
    """FCPW_SIMD_WIDTH of the vectorised build (0 when it is not available)."""
    return int(_load(True).ref_simd_width()) if available(True) else 0


def _p(a):
    return None if a is None else a.ctypes.data


class RefScene:
    """The reference Scene<DIM> with one object, built with vectorize=False, or
    with vectorize=True (the Mbvh; needs the Enoki build, timing calls only)."""
    _simd = False

    def __init__(self, dim, positions, indices, aggregate_type=3, silhouettes=False, vectorize=False):
        self.dim = dim
        self.silhouettes = bool(silhouettes)
        self._simd = bool(vectorize)
        self.positions = np.ascontiguousarray(positions, np.float32)
        self.indices = np.ascontiguousarray(indices, np.int32)
        self._h = _load(self._simd).ref_scene_create_ex(dim, _p(self.positions), len(self.positions),
                                                        _p(self.indices), len(self.indices), int(aggregate_type),
                                                        int(self.silhouettes), int(self._simd))

    def __del__(self):
        if getattr(self, "_h", None):
            _load(self._simd).ref_scene_destroy(self._h)
            self._h = None

    # ---- the reference's public bundled API (Scene::findClosestPoints / intersect /
    # findClosestSilhouettePoints over std::vector, its own std::thread split); each returns
    # (records, seconds inside that call)
    def closest_points_timed(self, spheres):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        sec = _load(self._simd).ref_scene_closest_points_timed(self._h, _p(self._sph(spheres)), len(spheres),
                                                               _p(out))
        return out, float(sec)

    def intersect_rays_timed(self, rays, occlusion=False):
        from fcpw_gb300 import records as R
        out = np.zeros(len(rays), R.INTERACTION)
        r = np.ascontiguousarray(rays).view(np.float32)
        sec = _load(self._simd).ref_scene_intersect_rays_timed(self._h, _p(r), len(rays), int(occlusion), _p(out))
        return out, float(sec)

    def silhouettes_timed(self, spheres, flip):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        fl = np.ascontiguousarray(flip, np.uint32)
        sec = _load(self._simd).ref_scene_silhouettes_timed(self._h, _p(self._sph(spheres)), _p(fl), len(spheres),
                                                            _p(out))
        return out, float(sec)

    def export(self):
        from fcpw_gb300 import records as R
        info = np.zeros(5, np.int32)
        _load().ref_export(self._h, None, None, None, _p(info))
        nodes = np.zeros(info[0], R.SNCH_NODE if self.silhouettes else R.BVH_NODE)
        prims = np.zeros(info[3], R.TRIANGLE if self.dim == 3 else R.LINE_SEGMENT)
        sils = np.zeros(info[4], R.EDGE if self.dim == 3 else R.VERTEX) if self.silhouettes else None
        _load().ref_export(self._h, _p(nodes), _p(prims), _p(sils), _p(info))
        return nodes, prims, sils, {"n_nodes": int(info[0]), "n_leaves": int(info[1]), "max_depth": int(info[2])}

    @staticmethod
    def _sph(spheres):
        return np.ascontiguousarray(spheres).view(np.float32)

    def closest_points(self, spheres, record_normals=False, visited=False):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        nv = np.zeros(len(spheres), np.int32) if visited else None
        _load().ref_closest_points(self._h, _p(self._sph(spheres)), len(spheres), int(record_normals), _p(out), _p(nv))
        return (out, nv) if visited else out

    def intersect_rays(self, rays, occlusion=False):
        from fcpw_gb300 import records as R
        out = np.zeros(len(rays), R.INTERACTION)
        hit = np.zeros(len(rays), np.int32)
        r = np.ascontiguousarray(rays).view(np.float32)
        _load().ref_intersect_rays(self._h, _p(r), len(rays), int(occlusion), _p(out), _p(hit))
        return out, hit.astype(bool)

    def silhouettes_query(self, spheres, flip, squared_min_radius=0.0, precision=1e-3):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        fl = np.ascontiguousarray(flip, np.uint32)
        _load().ref_silhouettes(self._h, _p(self._sph(spheres)), _p(fl), len(spheres), float(squared_min_radius),
                                float(precision), _p(out))
        return out

    def sphere_sample(self, spheres, rand_nums):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        hit = np.zeros(len(spheres), np.int32)
        rn = np.ascontiguousarray(rand_nums, np.float32)
        _load().ref_sphere_sample(self._h, _p(self._sph(spheres)), _p(rn), len(spheres), _p(out), _p(hit))
        return out, hit.astype(bool)

    @staticmethod
    def _pts3(points):
        p = np.asarray(points, np.float32)
        out = np.zeros((len(p), 3), np.float32)
        out[:, : p.shape[1]] = p
        return out

    def contains(self, points):
        pts = self._pts3(points)
        out = np.zeros(len(pts), np.uint32)
        _load().ref_contains(self._h, _p(pts), len(pts), _p(out))
        return out

    def line_of_sight(self, points_a, points_b):
        a, b = self._pts3(points_a), self._pts3(points_b)
        out = np.zeros(len(a), np.uint32)
        _load().ref_line_of_sight(self._h, _p(a), _p(b), len(a), _p(out))
        return out

    def update_and_refit(self, positions):
        pos = np.ascontiguousarray(positions, np.float32)
        _load().ref_update_and_refit(self._h, _p(pos), len(pos))


class RefMultiScene(RefScene):
    """The reference Scene<DIM> with several objects and instance transforms
    (setObjectCount / setObjectInstanceTransforms), built with vectorize=False.
    objects: list of (positions, indices); transforms: per object a list of
    (DIM+1)x(DIM+1) matrices (empty: one untransformed instance)."""

    def __init__(self, dim, objects, transforms, aggregate_type=3, silhouettes=False):
        self.dim = dim
        self.silhouettes = bool(silhouettes)
        self._pos = [np.ascontiguousarray(p, np.float32) for p, _ in objects]
        self._idx = [np.ascontiguousarray(f, np.int32) for _, f in objects]
        k = len(objects)
        pp = (C.c_void_p * k)(*[a.ctypes.data for a in self._pos])
        ip = (C.c_void_p * k)(*[a.ctypes.data for a in self._idx])
        nv = np.array([len(a) for a in self._pos], np.int32)
        npr = np.array([len(a) for a in self._idx], np.int32)
        nt = np.array([len(t) for t in transforms], np.int32)
        self._transforms = [list(t) for t in transforms]
        mats = [np.asarray(m, np.float32).reshape(dim + 1, dim + 1) for t in transforms for m in t]
        self._tm = np.ascontiguousarray(np.concatenate([m.reshape(-1) for m in mats]) if mats
                                        else np.zeros(1, np.float32))
        self._h = _load().ref_scene_create_multi_ex(dim, k, C.cast(pp, C.c_void_p), _p(nv), C.cast(ip, C.c_void_p),
                                                    _p(npr), _p(nt), _p(self._tm), int(aggregate_type),
                                                    int(self.silhouettes))

    def closest_points_objects(self, spheres, record_normals=False):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        obj = np.zeros(len(spheres), np.int32)
        _load().ref_closest_points_objects(self._h, _p(self._sph(spheres)), len(spheres), int(record_normals),
                                           _p(out), _p(obj))
        return out, obj

    def intersect_rays_objects(self, rays, occlusion=False):
        from fcpw_gb300 import records as R
        out = np.zeros(len(rays), R.INTERACTION)
        hit = np.zeros(len(rays), np.int32)
        obj = np.zeros(len(rays), np.int32)
        r = np.ascontiguousarray(rays).view(np.float32)
        _load().ref_intersect_rays_objects(self._h, _p(r), len(rays), int(occlusion), _p(out), _p(hit), _p(obj))
        return out, hit.astype(bool), obj

    def silhouettes_objects(self, spheres, flip, squared_min_radius=0.0, precision=1e-3):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        obj = np.zeros(len(spheres), np.int32)
        fl = np.ascontiguousarray(flip, np.uint32)
        _load().ref_silhouettes_objects(self._h, _p(self._sph(spheres)), _p(fl), len(spheres),
                                        float(squared_min_radius), float(precision), _p(out), _p(obj))
        return out, obj

    def sphere_sample_objects(self, spheres, rand_nums):
        from fcpw_gb300 import records as R
        out = np.zeros(len(spheres), R.INTERACTION)
        hit = np.zeros(len(spheres), np.int32)
        obj = np.zeros(len(spheres), np.int32)
        rn = np.ascontiguousarray(rand_nums, np.float32)
        _load().ref_sphere_sample_objects(self._h, _p(self._sph(spheres)), _p(rn), len(spheres), _p(out), _p(hit),
                                          _p(obj))
        return out, hit.astype(bool), obj

    def update_object_and_refit(self, object_index, positions):
        pos = np.ascontiguousarray(positions, np.float32)
        self._pos[object_index] = pos
        _load().ref_update_object_and_refit(self._h, int(object_index), _p(pos), len(pos))

    def export_top(self):
        """(nodes, aggregate index per leaf reference) of the top-level tree."""
        from fcpw_gb300 import records as R
        n = _load().ref_export_top(self._h, None, None)
        nodes = np.zeros(n, R.BVH_NODE)
        refs = np.zeros(sum(len(t) or 1 for t in self._transforms), np.int32)
        _load().ref_export_top(self._h, _p(nodes), _p(refs))
        return nodes, refs
