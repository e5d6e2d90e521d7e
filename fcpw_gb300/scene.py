"""Host-side scene description and BVH producer: the subset of the reference's
``fcpw.Scene2D/3D`` (python/fcpw_bindings.cpp:217-491) that the GPU path needs.

A scene holds one object (vertex positions + line segments or triangles). ``build``
runs the native binary SAH builder, which reproduces ``Scene<DIM>::build`` with
``vectorize=False`` for a single object (include/fcpw/fcpw.inl:1053-1126).
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np

from . import records as R
from ._lib import BvhInfo, check, lib, ptr


class AggregateType(IntEnum):
    """include/fcpw/utilities/scene_data.h:17-24"""
    Baseline = 0
    Bvh_LongestAxisCenter = 1
    Bvh_OverlapSurfaceArea = 2
    Bvh_SurfaceArea = 3
    Bvh_OverlapVolume = 4
    Bvh_Volume = 5


class PrimitiveType(IntEnum):
    LineSegment = 0
    Triangle = 1


class CpuBvh:
    """Owner of a native host-built BVH (fcpwgb_cpu_bvh)."""

    def __init__(self, dim: int, positions: np.ndarray, indices: np.ndarray, aggregate_type: int,
                 with_silhouettes: bool):
        positions = np.ascontiguousarray(positions, np.float32)
        indices = np.ascontiguousarray(indices, np.int32)
        if positions.ndim != 2 or positions.shape[1] != dim:
            raise ValueError(f"positions must have shape (V, {dim})")
        if indices.ndim != 2 or indices.shape[1] != dim:
            raise ValueError(f"indices must have shape (N, {dim})")
        handle = C.c_void_p()
        check(lib().fcpwgb_cpu_bvh_build(dim, ptr(positions), positions.shape[0], ptr(indices), indices.shape[0],
                                         int(aggregate_type), int(bool(with_silhouettes)), C.byref(handle)))
        self._h = handle
        self.dim = dim
        info = BvhInfo()
        check(lib().fcpwgb_cpu_bvh_info(self._h, C.byref(info)))
        self.info = info

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fcpwgb_cpu_bvh_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def snch(self) -> bool:
        return self.info.bvh_type in (R.LINE_SEGMENT_SNCH, R.TRIANGLE_SNCH)

    def export(self):
        """Flattened tree in the interop layouts: (nodes, primitives, silhouettes)."""
        i = self.info
        nodes = np.zeros(i.n_nodes, R.SNCH_NODE if self.snch else R.BVH_NODE)
        prims = np.zeros(i.n_primitives, R.TRIANGLE if self.dim == 3 else R.LINE_SEGMENT)
        sils = np.zeros(i.n_silhouettes, R.EDGE if self.dim == 3 else R.VERTEX) if self.snch else None
        check(lib().fcpwgb_cpu_bvh_export(self._h, ptr(nodes), ptr(prims), ptr(sils) if sils is not None and len(sils) else None))
        return nodes, prims, sils

    def topology(self):
        """(index_map, prim_vertices (leaf order, caller numbering), prim_index, sil_vertices)"""
        i = self.info
        index_map = np.zeros(i.n_vertices, np.int32)
        prim_vertices = np.zeros((i.n_primitives, self.dim), np.int32)
        prim_index = np.zeros(i.n_primitives, np.uint32)
        sil_vertices = np.zeros((i.n_silhouettes, self.dim + 1), np.int32) if self.snch else None
        check(lib().fcpwgb_cpu_bvh_export_topology(self._h, ptr(index_map), ptr(prim_vertices), ptr(prim_index),
                                                   ptr(sil_vertices) if sil_vertices is not None and len(sil_vertices) else None))
        return index_map, prim_vertices, prim_index, sil_vertices

    def export_wide(self, branching: int, bits: int, leaf_size: int = 0):
        """The wide / quantised tree of the GPU fast path: (raw records as an
        (n_nodes, node_bytes) uint8 array, child_binary (n_nodes, branching))."""
        n, nb = C.c_uint32(0), C.c_uint32(0)
        check(lib().fcpwgb_cpu_bvh_export_wide(self._h, branching, bits, leaf_size, None, None, C.byref(n),
                                               C.byref(nb)))
        nodes = np.zeros((n.value, nb.value), np.uint8)
        cb = np.zeros((n.value, branching), np.int32)
        check(lib().fcpwgb_cpu_bvh_export_wide(self._h, branching, bits, leaf_size, ptr(nodes), ptr(cb), C.byref(n),
                                               C.byref(nb)))
        return nodes, cb

    def save(self, path, wide=()) -> None:
        """Writes a scene file (fcpwgb_cpu_bvh_save): the tree, primitives,
        silhouettes, topology and the wide trees of the given
        (branching, bits, leaf_size) layouts."""
        from ._lib import TraversalConfig
        cfgs = (TraversalConfig * max(len(wide), 1))()
        for k, w in enumerate(wide):
            b, q = int(w[0]), int(w[1])
            leaf = int(w[2]) if len(w) > 2 else 0
            cfgs[k] = TraversalConfig(b, q, 128, 1, 0, 1, 0, leaf, 16, 1)
        check(lib().fcpwgb_cpu_bvh_save(self._h, str(path).encode(), cfgs, len(wide)))

    def update_positions(self, positions: np.ndarray) -> None:
        positions = np.ascontiguousarray(positions, np.float32)
        if positions.shape != (self.info.n_vertices, self.dim):
            raise ValueError("positions must keep the vertex count")
        check(lib().fcpwgb_cpu_bvh_update_positions(self._h, ptr(positions)))


class CpuInstances:
    """Owner of a native instanced structure (fcpwgb_cpu_instances): the
    objects' host trees, the instances and the top-level tree, as the
    reference's Scene::build makes them for several objects or instances
    (fcpw.inl:1053-1102)."""

    def __init__(self, dim: int, objects: list, instance_objects, transforms, aggregate_type: int):
        self.dim = dim
        self.objects = list(objects)            # CpuBvh per object (kept alive with this owner)
        self.instance_objects = np.ascontiguousarray(instance_objects, np.uint32)
        n = len(self.instance_objects)
        self.transformed = np.ascontiguousarray([t is not None for t in transforms], np.uint32)
        mats = np.zeros((n, dim, dim + 1), np.float32)
        for i, t in enumerate(transforms):
            if t is not None:
                m = np.asarray(t, np.float32)
                if m.shape not in ((dim + 1, dim + 1), (dim, dim + 1)):
                    raise ValueError(f"instance transforms must be ({dim + 1}, {dim + 1}) or ({dim}, {dim + 1})")
                mats[i] = m[:dim]
        self.matrices = np.ascontiguousarray(mats)
        handles = (C.c_void_p * len(self.objects))(*[o.handle.value for o in self.objects])
        h = C.c_void_p()
        check(lib().fcpwgb_cpu_instances_build(dim, int(aggregate_type), C.cast(handles, C.c_void_p),
                                               len(self.objects), ptr(self.instance_objects), ptr(self.matrices),
                                               ptr(self.transformed), n, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def __len__(self):
        return len(self.instance_objects)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fcpwgb_cpu_instances_destroy(h)
            except Exception:
                pass
            self._h = None

    def export(self):
        """(top-level nodes, leaf references (instance indices), (n, 24) float
        matrices: the 3x4 rows of each transform, then of its inverse)."""
        nn = C.c_uint32(0)
        check(lib().fcpwgb_cpu_instances_export(self._h, None, None, None, C.byref(nn)))
        nodes = np.zeros(nn.value, R.BVH_NODE)
        refs = np.zeros(len(self) if nn.value else 0, np.uint32)
        mats = np.zeros((len(self), 24), np.float32)
        check(lib().fcpwgb_cpu_instances_export(self._h, ptr(nodes) if nn.value else None,
                                                ptr(refs) if nn.value else None, ptr(mats), C.byref(nn)))
        return nodes, refs, mats


class _Scene:
    DIM = 3

    def __init__(self):
        self._positions: list = []
        self._indices: list = []
        self._silhouettes = False
        self._bvh: CpuBvh | None = None
        self._vectorized = False
        self._aggregate_type = None
        self._transforms: list = []
        self._instances: CpuInstances | None = None

    # -- geometry ---------------------------------------------------------
    def set_object_count(self, n_objects: int) -> None:
        self._positions = [None] * int(n_objects)
        self._indices = [None] * int(n_objects)
        self._transforms = [[] for _ in range(int(n_objects))]
        self._bvh = None
        self._instances = None

    def set_object_instance_transforms(self, transforms, object_index: int) -> None:
        """Scene::setObjectInstanceTransforms (fcpw.h:70, fcpw.inl:393-397):
        appends (DIM+1)x(DIM+1) affine matrices (uniform scale) for an object."""
        for t in transforms:
            m = np.asarray(t, np.float32)
            if m.shape != (self.DIM + 1, self.DIM + 1):
                raise ValueError(f"instance transforms must be ({self.DIM + 1}, {self.DIM + 1}) matrices")
            self._transforms[object_index].append(m.copy())

    def set_object_vertices(self, positions, object_index: int) -> None:
        p = np.asarray(positions, np.float32)
        if p.ndim != 2 or p.shape[1] != self.DIM:
            raise ValueError(f"positions must have shape (V, {self.DIM})")
        self._positions[object_index] = np.ascontiguousarray(p)

    def _set_indices(self, indices, object_index: int) -> None:
        ix = np.asarray(indices, np.int32)
        if ix.ndim != 2 or ix.shape[1] != self.DIM:
            raise ValueError(f"indices must have shape (N, {self.DIM})")
        self._indices[object_index] = np.ascontiguousarray(ix)

    def compute_silhouettes(self, ignore_silhouette=None) -> None:
        """Scene::computeSilhouettes (fcpw.inl:428-521). Custom ignore callbacks are not supported."""
        if ignore_silhouette is not None:
            raise NotImplementedError("ignore_silhouette callbacks are not supported by the GPU producer")
        self._silhouettes = True

    def build(self, aggregate_type, vectorize: bool, print_stats: bool = False,
              reduce_memory_footprint: bool = False) -> None:
        """Scene::build (fcpw.inl:1053-1126). One object without instance
        transforms gives one tree; several objects or instance transforms give
        a tree per object, the instances in the reference's order (objects in
        turn; an object without transforms is one untransformed instance) and
        a top-level tree over them."""
        if not self._positions or any(p is None for p in self._positions) or \
                any(i is None for i in self._indices):
            raise ValueError("every object needs vertices and primitives")
        self._vectorized = bool(vectorize)
        self._aggregate_type = AggregateType(int(aggregate_type))
        self._instances = None
        if len(self._positions) == 1 and not self._transforms[0]:
            self._bvh = CpuBvh(self.DIM, self._positions[0], self._indices[0], int(aggregate_type),
                               self._silhouettes)
        else:
            objs = [CpuBvh(self.DIM, p, f, int(aggregate_type), self._silhouettes)
                    for p, f in zip(self._positions, self._indices)]
            inst_obj, mats = [], []
            for k, ts in enumerate(self._transforms):
                if not ts:
                    inst_obj.append(k)
                    mats.append(None)
                for t in ts:
                    inst_obj.append(k)
                    mats.append(t)
            self._instances = CpuInstances(self.DIM, objs, inst_obj, mats, int(aggregate_type))
            self._bvh = None
            if print_stats:
                print(f"{len(objs)} objects, {len(inst_obj)} instances")
            return
        if print_stats:
            i = self._bvh.info
            print(f"BVH stats: {i.n_nodes} nodes, {i.n_leaves} leaves, {i.max_depth} max depth, "
                  f"{i.n_primitives} primitives, {i.n_silhouettes} silhouetteRefs")

    def update_object_vertex(self, position, vertex_index: int, object_index: int) -> None:
        self._positions[object_index][vertex_index] = np.asarray(position, np.float32)[: self.DIM]

    def update_object_vertices(self, positions, object_index: int) -> None:
        p = np.asarray(positions, np.float32)
        self._positions[object_index][: len(p)] = p

    # -- accessors used by GPUScene ---------------------------------------
    @property
    def cpu_bvh(self) -> CpuBvh:
        if self._bvh is None:
            if self._instances is not None:
                raise RuntimeError("a scene of several objects or instances has one tree per object "
                                   "(Scene.instances)")
            raise RuntimeError("Scene.build has not been called")
        return self._bvh

    @property
    def instances(self) -> CpuInstances | None:
        """The instanced structure of a scene of several objects or instances (None otherwise)."""
        return self._instances

    def positions(self, object_index: int = 0) -> np.ndarray:
        return self._positions[object_index]

    def indices(self, object_index: int = 0) -> np.ndarray:
        return self._indices[object_index]


class Scene2D(_Scene):
    DIM = 2

    def set_object_line_segments(self, indices, object_index: int) -> None:
        self._set_indices(indices, object_index)


class Scene3D(_Scene):
    DIM = 3

    def set_object_triangles(self, indices, object_index: int) -> None:
        self._set_indices(indices, object_index)


def scene_file_info(path) -> dict:
    """Header of a scene file (checksum verified)."""
    from ._lib import BvhInfo
    info, nw = BvhInfo(), C.c_uint32(0)
    check(lib().fcpwgb_scene_file_info(str(path).encode(), C.byref(info), C.byref(nw)))
    return {"dim": info.dim, "bvh_type": info.bvh_type, "n_nodes": info.n_nodes, "n_primitives": info.n_primitives,
            "n_silhouettes": info.n_silhouettes, "n_vertices": info.n_vertices, "n_wide": int(nw.value)}
