"""``GPUScene2D`` / ``GPUScene3D``: the reference's Python GPU classes
(python/fcpw_bindings.cpp:493-673) on top of the C ABI.

Method names, keyword names, defaults and overloads follow the reference:
``transfer_to_gpu``, ``refit``, ``intersect`` (rays or spheres, arrays or
lists), ``find_closest_points`` and ``find_closest_silhouette_points``. Results
land in a ``GPUInteractionList`` passed by the caller, as in the reference.
Tensor methods (``*_tensor``) take CUDA tensors and return device tensors
without host copies.
"""
from __future__ import annotations

import ctypes as C
from collections import namedtuple

import numpy as np

from . import records as R
from ._lib import check, lib, ptr
from .scene import Scene2D, Scene3D, _Scene


# ---------------------------------------------------------------- structs
class GPUFloat2:
    def __init__(self, x: float = 0.0, y: float = 0.0):
        self.x, self.y = float(x), float(y)


class GPUFloat3:
    def __init__(self, x: float = 0.0, y: float = 0.0, z: float = 0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)


def _f3(v) -> tuple:
    if isinstance(v, GPUFloat3):
        return (v.x, v.y, v.z)
    return tuple(float(a) for a in v)


class GPURay:
    def __init__(self, o=None, d=None, tMax: float = float(R.FLT_MAX)):
        self.o = o if o is not None else GPUFloat3()
        self.d = d if d is not None else GPUFloat3()
        dd = _f3(self.d)
        with np.errstate(divide="ignore"):
            inv = np.float32(1.0) / np.asarray(dd, np.float32)
        self.inv_d = GPUFloat3(*inv)
        self.t_max = float(tMax)


class GPUBoundingSphere:
    def __init__(self, c=None, r2: float = 0.0):
        self.c = c if c is not None else GPUFloat3()
        self.r2 = float(r2)


class GPUInteraction:
    def __init__(self, rec=None):
        rec = rec if rec is not None else R.default_interactions(1)[0]
        self.p = GPUFloat3(*rec["p"])
        self.n = GPUFloat3(*rec["n"])
        self.uv = GPUFloat2(*rec["uv"])
        self.d = float(rec["d"])
        self.index = int(rec["index"])


# ------------------------------------------------------------------ lists
class _RecordList:
    """A growable array of interop records with a list-like interface."""
    DTYPE = None

    def __init__(self, items=None):
        self._a = np.zeros(0, self.DTYPE)
        if items is not None:
            for it in items:
                self.append(it)

    @classmethod
    def from_array(cls, arr: np.ndarray):
        obj = cls()
        obj._a = np.ascontiguousarray(arr, cls.DTYPE)
        return obj

    def array(self) -> np.ndarray:
        return self._a

    def __len__(self):
        return len(self._a)

    def resize(self, n: int):
        a = np.zeros(n, self.DTYPE)
        m = min(n, len(self._a))
        a[:m] = self._a[:m]
        self._a = a

    def clear(self):
        self._a = np.zeros(0, self.DTYPE)

    def append(self, item):
        rec = np.zeros(1, self.DTYPE)
        self._fill(rec[0], item)
        self._a = np.concatenate([self._a, rec])


class GPUFloat3List(_RecordList):
    DTYPE = np.dtype(("<f4", (3,)))

    def _fill(self, rec, item):
        rec[...] = _f3(item)

    def __getitem__(self, i):
        return GPUFloat3(*self._a[i])


class GPURayList(_RecordList):
    DTYPE = R.RAY

    def _fill(self, rec, r: GPURay):
        rec["o"], rec["d"], rec["dInv"], rec["tMax"] = _f3(r.o), _f3(r.d), _f3(r.inv_d), r.t_max


class GPUBoundingSphereList(_RecordList):
    DTYPE = R.SPHERE

    def _fill(self, rec, s: GPUBoundingSphere):
        rec["c"], rec["r2"] = _f3(s.c), s.r2


class Uint32List(_RecordList):
    DTYPE = np.dtype("<u4")

    def _fill(self, rec, v):
        rec[...] = int(v)


class GPUInteractionList(_RecordList):
    DTYPE = R.INTERACTION

    def _fill(self, rec, it: GPUInteraction):
        rec["p"], rec["n"] = _f3(it.p), _f3(it.n)
        rec["uv"] = (it.uv.x, it.uv.y)
        rec["d"], rec["index"] = it.d, it.index

    def __getitem__(self, i):
        return GPUInteraction(self._a[i])

    # bulk extraction, python/fcpw_bindings.cpp:536-584
    def get_distances(self):
        return self._a["d"].copy()

    def get_positions(self):
        return self._a["p"].copy()

    def get_normals(self):
        return self._a["n"].copy()

    def get_uvs(self):
        return self._a["uv"].copy()

    def get_indices(self):
        return self._a["index"].copy()


TensorInteractions = namedtuple("TensorInteractions", "p n uv d index raw")


def _split_records(raw):
    """Views of a (N, 10) float32 tensor holding interaction records."""
    import torch
    return TensorInteractions(raw[:, 0:3], raw[:, 3:6], raw[:, 6:8], raw[:, 8], raw[:, 9].view(torch.int32), raw)


# ------------------------------------------------------------ GPU scenes
class _GPUScene:
    DIM = 3

    def __init__(self, fcpw_directory_path: str = "", print_logs: bool = False, device: int = 0):
        # the directory argument of the reference locates Slang shaders; kernels here are precompiled
        self.print_logs = bool(print_logs)
        self.device = int(device)
        handle = C.c_void_p()
        check(lib().fcpwgb_gpu_scene_create(self.DIM, self.device, C.byref(handle)))
        self._h = handle
        self._cpu_bvh = None
        self._instances = None
        self._n_vertices = 0
        self._n_nodes = 0
        self._snch = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fcpwgb_gpu_scene_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    # -- traversal variant -------------------------------------------------
    def set_traversal(self, branching: int = 0, bits: int = 32, sort_queries: bool = True,
                      persistent: bool = True, precise: bool = True, packet: bool = False, leaf_size: int = 0,
                      short_stack: int = 16, threads_per_query: int = 1) -> None:
        """Selects the closest point traversal (see fcpwgb_traversal_config):
        branching 0 is the reference-order binary traversal; 2/4/8 use a wide
        tree with 32-, 16- or 8-bit child boxes; packet walks the queries of a
        warp together; precise refines distances to within 1e-6 of FP64;
        leaf_size merges small subtrees into wide leaves; short_stack (0 or 16)
        is the per-thread stack depth kept in shared memory; threads_per_query
        (1, 2, 4 or 8) answers each query with that many cooperating lanes,
        which split each record's child boxes and each leaf's primitives. With branching
        > 0, silhouette queries use warp packets and contains and rays are
        sorted spatially (sort_queries)."""
        from ._lib import TraversalConfig
        cfg = TraversalConfig(int(branching), int(bits), 128, int(bool(sort_queries)), int(bool(persistent)),
                              int(bool(precise)), int(bool(packet)), int(leaf_size), int(short_stack),
                              int(threads_per_query))
        check(lib().fcpwgb_gpu_scene_set_traversal(self._h, C.byref(cfg)))

    def get_traversal(self) -> dict:
        from ._lib import TraversalConfig
        cfg = TraversalConfig()
        check(lib().fcpwgb_gpu_scene_get_traversal(self._h, C.byref(cfg)))
        return {f: getattr(cfg, f) for f, _ in TraversalConfig._fields_}

    # -- transfer / refit --------------------------------------------------
    def transfer_to_gpu(self, scene: _Scene, device_backend: str = "default") -> None:
        """GPUScene::transferToGPU (include/fcpw/fcpw_gpu.h:21)."""
        if device_backend not in ("default", "cuda"):
            raise ValueError(f"unsupported device backend {device_backend!r}: this build runs on CUDA only")
        if scene.DIM != self.DIM:
            raise ValueError("scene dimension does not match the GPU scene")
        if scene._vectorized:
            raise ValueError("transfer_to_gpu needs a scene built with vectorize=False "
                             "(include/fcpw/fcpw_gpu.h:17-20)")
        if scene.instances is not None:
            # several objects or instances (fcpwgb_gpu_scene_transfer_instanced)
            check(lib().fcpwgb_gpu_scene_transfer_instanced(self._h, scene.instances.handle))
            self._cpu_bvh = None
            self._instances = scene.instances
            self._n_vertices = 0
            self._n_nodes = 0
            self._snch = False
            return
        self._instances = None
        bvh = scene.cpu_bvh
        check(lib().fcpwgb_gpu_scene_transfer_cpu_bvh(self._h, bvh.handle))
        self._cpu_bvh = bvh
        self._n_vertices = bvh.info.n_vertices
        self._n_nodes = bvh.info.n_nodes
        self._snch = bvh.snch

    def load(self, path) -> None:
        """Uploads a scene file written by CpuBvh.save (fcpwgb_gpu_scene_load): no CPU
        build, and no wide collapse for the layouts the file holds."""
        check(lib().fcpwgb_gpu_scene_load(self._h, str(path).encode()))
        from .scene import scene_file_info
        info = scene_file_info(path)
        self._cpu_bvh = None
        self._n_vertices = info["n_vertices"]
        self._n_nodes = info["n_nodes"]
        self._snch = info["bvh_type"] in (R.LINE_SEGMENT_SNCH, R.TRIANGLE_SNCH)

    def build_on_gpu(self, positions, indices, max_leaf_size: int = 4, method: str = "lbvh",
                     aggregate_type: int = 3) -> None:
        """Builds the tree on the device and sets the scene up from it:
        positions (V, DIM) float32, indices (P, DIM) int32, as numpy arrays or
        contiguous CUDA tensors (built on the current torch stream). method
        "lbvh" (fcpwgb_gpu_scene_build): a linear BVH, distances agree with
        the host SAH build, the primitive chosen on an exact tie may differ;
        "sah" (fcpwgb_gpu_scene_build_sah): the reference's binned SAH tree
        for aggregate_type (a Bvh_* AggregateType), node for node the tree
        Scene.build makes. No silhouettes."""
        if method not in ("lbvh", "sah"):
            raise ValueError("method must be 'lbvh' or 'sah'")
        try:
            import torch
            on_device = isinstance(positions, torch.Tensor) and positions.is_cuda
        except ImportError:  # pragma: no cover
            on_device = False
        if on_device:
            if (positions.dtype != torch.float32 or indices.dtype != torch.int32 or not indices.is_cuda
                    or not positions.is_contiguous() or not indices.is_contiguous()):
                raise ValueError("positions (float32) and indices (int32) must be contiguous CUDA tensors")
            if positions.dim() != 2 or positions.shape[1] != self.DIM or indices.dim() != 2 \
                    or indices.shape[1] != self.DIM:
                raise ValueError(f"positions and indices must have {self.DIM} columns")
            stream = torch.cuda.current_stream(positions.device).cuda_stream
            if method == "sah":
                check(lib().fcpwgb_gpu_scene_build_sah_device(self._h, positions.data_ptr(), positions.shape[0],
                                                              indices.data_ptr(), indices.shape[0],
                                                              int(aggregate_type), C.c_void_p(stream)))
            else:
                check(lib().fcpwgb_gpu_scene_build_device(self._h, positions.data_ptr(), positions.shape[0],
                                                          indices.data_ptr(), indices.shape[0], int(max_leaf_size),
                                                          C.c_void_p(stream)))
            n_vertices = positions.shape[0]
        else:
            pos = np.ascontiguousarray(positions, np.float32)
            idx = np.ascontiguousarray(indices, np.int32)
            if pos.ndim != 2 or pos.shape[1] != self.DIM or idx.ndim != 2 or idx.shape[1] != self.DIM:
                raise ValueError(f"positions and indices must have {self.DIM} columns")
            if method == "sah":
                check(lib().fcpwgb_gpu_scene_build_sah(self._h, ptr(pos), len(pos), ptr(idx), len(idx),
                                                       int(aggregate_type)))
            else:
                check(lib().fcpwgb_gpu_scene_build(self._h, ptr(pos), len(pos), ptr(idx), len(idx),
                                                   int(max_leaf_size)))
            n_vertices = len(pos)
        self._cpu_bvh = None
        self._n_vertices = int(n_vertices)
        self._n_nodes = self.info()["n_nodes"]
        self._snch = False

    def info(self) -> dict:
        """Sizes of the scene's binary tree (fcpwgb_gpu_scene_info)."""
        from ._lib import BvhInfo
        info = BvhInfo()
        check(lib().fcpwgb_gpu_scene_info(self._h, C.byref(info)))
        return {f: getattr(info, f) for f, _ in BvhInfo._fields_}

    def transfer_arrays(self, bvh_type: int, nodes, primitives, silhouettes=None, prim_vertices=None,
                        n_vertices: int = 0) -> None:
        """Uploads an already flattened tree in the interop layouts."""
        nodes = np.ascontiguousarray(nodes)
        primitives = np.ascontiguousarray(primitives)
        sils = np.ascontiguousarray(silhouettes) if silhouettes is not None else None
        pv = np.ascontiguousarray(prim_vertices, np.int32) if prim_vertices is not None else None
        check(lib().fcpwgb_gpu_scene_transfer(self._h, int(bvh_type), ptr(nodes), len(nodes), ptr(primitives),
                                              len(primitives), ptr(sils) if sils is not None and len(sils) else None,
                                              len(sils) if sils is not None else 0, ptr(pv), int(n_vertices)))
        self._n_vertices = int(n_vertices)
        self._n_nodes = len(nodes)
        self._snch = nodes.dtype == R.SNCH_NODE

    def refit(self, scene: _Scene, update_geometry: bool = True) -> None:
        """GPUScene::refit (include/fcpw/fcpw_gpu.h:27): with update_geometry the moved
        primitives (and silhouettes) are re-extracted from the scene and uploaded. On
        a scene of several objects or instances every object is refit, then the
        top level (Scene::refit, fcpw.inl:1146-1158)."""
        if getattr(self, "_instances", None) is not None:
            for k, bvh in enumerate(scene.instances.objects):
                if not update_geometry:
                    check(lib().fcpwgb_gpu_scene_refit_object(self._h, k, None, None))
                    continue
                bvh.update_positions(scene.positions(k))
                _, prims, sils = bvh.export()
                check(lib().fcpwgb_gpu_scene_refit_object(self._h, k, ptr(prims),
                                                          ptr(sils) if sils is not None and len(sils) else None))
            return
        if not update_geometry:
            check(lib().fcpwgb_gpu_scene_refit(self._h, None, None))
            return
        bvh = scene.cpu_bvh
        bvh.update_positions(scene.positions(0))
        _, prims, sils = bvh.export()
        check(lib().fcpwgb_gpu_scene_refit(self._h, ptr(prims), ptr(sils) if sils is not None and len(sils) else None))

    def refit_arrays(self, primitives=None, silhouettes=None) -> None:
        """refit with already extracted records (interop layouts); None refits the
        device geometry as it is (update_geometry=False)."""
        p = np.ascontiguousarray(primitives) if primitives is not None else None
        s = np.ascontiguousarray(silhouettes) if silhouettes is not None and len(silhouettes) else None
        check(lib().fcpwgb_gpu_scene_refit(self._h, ptr(p), ptr(s)))

    def update_vertices_tensor(self, positions) -> None:
        """Moves the vertices to ``positions`` (a CUDA float32 tensor (V, DIM) in the
        caller's vertex order) and refits on the device, on the current torch stream."""
        import torch
        if positions.dtype != torch.float32 or not positions.is_cuda or not positions.is_contiguous():
            raise ValueError("positions must be a contiguous float32 CUDA tensor")
        stream = torch.cuda.current_stream(positions.device).cuda_stream
        check(lib().fcpwgb_gpu_scene_update_vertices_device(self._h, positions.data_ptr(), positions.shape[0],
                                                            C.c_void_p(stream)))

    # -- queries -----------------------------------------------------------
    def _out(self, interactions: GPUInteractionList, n: int) -> np.ndarray:
        if not isinstance(interactions, GPUInteractionList):
            raise TypeError("interactions must be a GPUInteractionList")
        interactions._a = R.default_interactions(n)
        return interactions._a

    def intersect(self, *args, **kwargs) -> None:
        """The four ``intersect`` overloads of python/fcpw_bindings.cpp:597-613."""
        a0 = args[0] if args else kwargs.get("rays", kwargs.get("ray_origins", kwargs.get(
            "bounding_spheres", kwargs.get("sphere_centers"))))
        if isinstance(a0, GPURayList):
            self._intersect_rays_list(*args, **kwargs)
        elif isinstance(a0, GPUBoundingSphereList):
            self._intersect_spheres_list(*args, **kwargs)
        elif ("ray_origins" in kwargs) or (len(args) >= 3 and np.asarray(args[1]).ndim == 2
                                           and np.asarray(args[2]).ndim == 1):
            self._intersect_rays_arrays(*args, **kwargs)
        else:
            self._intersect_spheres_arrays(*args, **kwargs)

    def _intersect_rays_arrays(self, ray_origins, ray_directions, ray_distance_bounds, interactions,
                               check_for_occlusion: bool = False):
        rays = R.make_rays(ray_origins, ray_directions, ray_distance_bounds)
        self._run_rays(rays, interactions, check_for_occlusion)

    def _intersect_rays_list(self, rays: GPURayList, interactions, check_for_occlusion: bool = False):
        self._run_rays(rays.array(), interactions, check_for_occlusion)

    def _run_rays(self, rays, interactions, occl):
        out = self._out(interactions, len(rays))
        check(lib().fcpwgb_intersect_rays(self._h, ptr(rays), ptr(out), len(rays), int(bool(occl))))

    def _intersect_spheres_arrays(self, sphere_centers, sphere_squared_radii, rand_nums, interactions):
        spheres = R.make_spheres(sphere_centers, sphere_squared_radii)
        rn = np.zeros((len(spheres), 3), np.float32)
        r = np.asarray(rand_nums, np.float32)
        rn[:, : r.shape[1]] = r
        self._run_spheres(spheres, rn, interactions)

    def _intersect_spheres_list(self, bounding_spheres: GPUBoundingSphereList, rand_nums: GPUFloat3List,
                                interactions):
        self._run_spheres(bounding_spheres.array(), np.ascontiguousarray(rand_nums.array(), np.float32),
                          interactions)

    def _run_spheres(self, spheres, rn, interactions):
        out = self._out(interactions, len(spheres))
        check(lib().fcpwgb_intersect_spheres(self._h, ptr(spheres), ptr(rn), ptr(out), len(spheres)))

    def find_closest_points(self, *args, **kwargs) -> None:
        """python/fcpw_bindings.cpp:614-621"""
        a0 = args[0] if args else kwargs.get("bounding_spheres", kwargs.get("query_points"))
        if isinstance(a0, GPUBoundingSphereList):
            return self._closest_list(*args, **kwargs)
        return self._closest_arrays(*args, **kwargs)

    def _closest_arrays(self, query_points, squared_max_radii, interactions, record_normals: bool = False):
        spheres = R.make_spheres(query_points, squared_max_radii)
        self._run_closest(spheres, interactions, record_normals)

    def _closest_list(self, bounding_spheres, interactions, record_normals: bool = False):
        self._run_closest(bounding_spheres.array(), interactions, record_normals)

    def _run_closest(self, spheres, interactions, record_normals):
        out = self._out(interactions, len(spheres))
        check(lib().fcpwgb_find_closest_points(self._h, ptr(spheres), ptr(out), len(spheres),
                                               int(bool(record_normals))))

    # -- scenes of several objects or instances ------------------------------
    def find_closest_points_instanced(self, query_points, squared_max_radii, interactions,
                                      record_normals: bool = False) -> np.ndarray:
        """find_closest_points on a scene of several objects or instances, also
        returning the instance of every answer (UINT_MAX where none); indices
        are primitive indices within the instance's object."""
        spheres = R.make_spheres(query_points, squared_max_radii)
        out = self._out(interactions, len(spheres))
        inst = np.zeros(len(spheres), np.uint32)
        check(lib().fcpwgb_find_closest_points_instanced(self._h, ptr(spheres), ptr(out), ptr(inst), len(spheres),
                                                         int(bool(record_normals))))
        return inst

    def intersect_rays_instanced(self, ray_origins, ray_directions, ray_distance_bounds, interactions,
                                 check_for_occlusion: bool = False) -> np.ndarray:
        """Ray queries on a scene of several objects or instances, returning
        the instance hit by every ray (UINT_MAX where none)."""
        rays = R.make_rays(ray_origins, ray_directions, ray_distance_bounds)
        out = self._out(interactions, len(rays))
        inst = np.zeros(len(rays), np.uint32)
        check(lib().fcpwgb_intersect_rays_instanced(self._h, ptr(rays), ptr(out), ptr(inst), len(rays),
                                                    int(bool(check_for_occlusion))))
        return inst

    def intersect_spheres_instanced(self, sphere_centers, sphere_squared_radii, rand_nums,
                                    interactions) -> np.ndarray:
        """Sphere sampling on a scene of several objects or instances, returning
        the instance of every sample (UINT_MAX where none)."""
        spheres = R.make_spheres(sphere_centers, sphere_squared_radii)
        rn = np.zeros((len(spheres), 3), np.float32)
        r = np.asarray(rand_nums, np.float32)
        rn[:, : r.shape[1]] = r
        out = self._out(interactions, len(spheres))
        inst = np.zeros(len(spheres), np.uint32)
        check(lib().fcpwgb_intersect_spheres_instanced(self._h, ptr(spheres), ptr(rn), ptr(out), ptr(inst),
                                                       len(spheres)))
        return inst

    def find_closest_silhouette_points_instanced(self, query_points, squared_max_radii, flip_normal_orientation,
                                                 interactions, squared_min_radius: float = 0.0,
                                                 precision: float = 1e-3) -> np.ndarray:
        """Closest silhouette points on a scene of several objects or instances
        (every object built with silhouettes), returning the instance of every
        answer (UINT_MAX where none)."""
        spheres = R.make_spheres(query_points, squared_max_radii)
        flip = np.ascontiguousarray(np.asarray(flip_normal_orientation).astype(np.uint32))
        if len(flip) != len(spheres):
            raise ValueError("flip_normal_orientation must have one entry per query")
        out = self._out(interactions, len(spheres))
        inst = np.zeros(len(spheres), np.uint32)
        check(lib().fcpwgb_find_closest_silhouette_points_instanced(self._h, ptr(spheres), ptr(flip), ptr(out),
                                                                    ptr(inst), len(spheres), float(squared_min_radius),
                                                                    float(precision)))
        return inst

    def refit_object(self, object_index: int, primitives=None, silhouettes=None) -> None:
        """Refits one object of a scene of several objects or instances from its
        records (interop layouts, its leaf order; None: its device geometry as
        it is), then the top-level tree (fcpwgb_gpu_scene_refit_object)."""
        p = np.ascontiguousarray(primitives) if primitives is not None else None
        s = np.ascontiguousarray(silhouettes) if silhouettes is not None and len(silhouettes) else None
        check(lib().fcpwgb_gpu_scene_refit_object(self._h, int(object_index), ptr(p), ptr(s)))

    def update_object_vertices_tensor(self, object_index: int, positions) -> None:
        """Moves one object's vertices to ``positions`` (a CUDA float32 tensor (V, DIM)
        in the object's vertex order) and refits it and the top level on the
        device, on the current torch stream."""
        import torch
        if positions.dtype != torch.float32 or not positions.is_cuda or not positions.is_contiguous():
            raise ValueError("positions must be a contiguous float32 CUDA tensor")
        stream = torch.cuda.current_stream(positions.device).cuda_stream
        check(lib().fcpwgb_gpu_scene_update_object_vertices_device(self._h, int(object_index), positions.data_ptr(),
                                                                   positions.shape[0], C.c_void_p(stream)))

    def export_top_nodes(self) -> np.ndarray:
        """The device's top-level tree of a scene of several objects or instances
        (32 B interop nodes; empty for a single instance)."""
        n = C.c_uint32(0)
        check(lib().fcpwgb_gpu_scene_export_top_nodes(self._h, None, C.byref(n)))
        nodes = np.zeros(n.value, R.BVH_NODE)
        if n.value:
            check(lib().fcpwgb_gpu_scene_export_top_nodes(self._h, ptr(nodes), C.byref(n)))
        return nodes

    def instance_objects(self) -> np.ndarray:
        """Object of every instance of the transferred scene."""
        if getattr(self, "_instances", None) is None:
            raise RuntimeError("no scene of several objects or instances was transferred")
        return self._instances.instance_objects.copy()

    def find_closest_silhouette_points(self, *args, **kwargs) -> None:
        """python/fcpw_bindings.cpp:622-629"""
        a0 = args[0] if args else kwargs.get("bounding_spheres", kwargs.get("query_points"))
        if isinstance(a0, GPUBoundingSphereList):
            return self._silhouette_list(*args, **kwargs)
        return self._silhouette_arrays(*args, **kwargs)

    def _silhouette_arrays(self, query_points, squared_max_radii, flip_normal_orientation, interactions,
                           squared_min_radius: float = 0.0, precision: float = 1e-3):
        spheres = R.make_spheres(query_points, squared_max_radii)
        flip = np.ascontiguousarray(np.asarray(flip_normal_orientation).astype(np.uint32))
        self._run_silhouette(spheres, flip, interactions, squared_min_radius, precision)

    def _silhouette_list(self, bounding_spheres, flip_normal_orientation, interactions,
                         squared_min_radius: float = 0.0, precision: float = 1e-3):
        flip = flip_normal_orientation.array() if isinstance(flip_normal_orientation, Uint32List) else \
            np.ascontiguousarray(np.asarray(flip_normal_orientation).astype(np.uint32))
        self._run_silhouette(bounding_spheres.array(), flip, interactions, squared_min_radius, precision)

    def _run_silhouette(self, spheres, flip, interactions, sq_min_r, precision):
        if len(flip) != len(spheres):
            raise ValueError("flip_normal_orientation must have one entry per query")
        out = self._out(interactions, len(spheres))
        check(lib().fcpwgb_find_closest_silhouette_points(self._h, ptr(spheres), ptr(flip), ptr(out), len(spheres),
                                                          float(sq_min_r), float(precision)))

    # -- zero-copy tensor entry points ---------------------------------------
    @staticmethod
    def _stream(t):
        import torch
        return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)

    def _check_tensor(self, t, cols):
        import torch
        if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous() or t.dim() != 2 or t.shape[1] != cols:
            raise ValueError(f"expected a contiguous float32 CUDA tensor of shape (N, {cols})")

    def find_closest_points_tensor(self, spheres, record_normals: bool = False, out=None) -> TensorInteractions:
        """``spheres``: (N, 4) float32 CUDA tensor of (x, y, z, r2). Returns device views."""
        import torch
        self._check_tensor(spheres, 4)
        n = spheres.shape[0]
        raw = out if out is not None else torch.empty((n, 10), dtype=torch.float32, device=spheres.device)
        check(lib().fcpwgb_find_closest_points_device(self._h, spheres.data_ptr(), raw.data_ptr(), n,
                                                      int(bool(record_normals)), self._stream(spheres)))
        return _split_records(raw)

    def intersect_tensor(self, rays, check_for_occlusion: bool = False, out=None) -> TensorInteractions:
        """``rays``: (N, 10) float32 CUDA tensor of (o, d, 1/d, tMax) records."""
        import torch
        self._check_tensor(rays, 10)
        n = rays.shape[0]
        raw = out if out is not None else torch.empty((n, 10), dtype=torch.float32, device=rays.device)
        check(lib().fcpwgb_intersect_rays_device(self._h, rays.data_ptr(), raw.data_ptr(), n,
                                                 int(bool(check_for_occlusion)), self._stream(rays)))
        return _split_records(raw)

    # -- inside / line of sight (Scene::contains / hasLineOfSight, CPU-only in the reference)
    @staticmethod
    def _points3(points) -> np.ndarray:
        p = np.asarray(points, np.float32)
        if p.ndim != 2 or p.shape[1] not in (2, 3):
            raise ValueError("points must have shape (N, 2) or (N, 3)")
        out = np.zeros((len(p), 3), np.float32)
        out[:, : p.shape[1]] = p
        return out

    def contains(self, points) -> np.ndarray:
        """1 where a point is inside the (watertight) boundary, else 0 (fcpw.inl:1443-1460)."""
        pts = self._points3(points)
        res = np.zeros(len(pts), np.uint32)
        check(lib().fcpwgb_contains(self._h, ptr(pts), len(pts), ptr(res)))
        return res

    def has_line_of_sight(self, points_a, points_b) -> np.ndarray:
        """1 where the segment between the paired points hits no primitive (fcpw.inl:1501-1520)."""
        a, b = self._points3(points_a), self._points3(points_b)
        if len(a) != len(b):
            raise ValueError("points_a and points_b must have the same length")
        res = np.zeros(len(a), np.uint32)
        check(lib().fcpwgb_has_line_of_sight(self._h, ptr(a), ptr(b), len(a), ptr(res)))
        return res

    def contains_tensor(self, points, out=None):
        """points: (N, 3) float32 CUDA tensor; returns an int32 CUDA tensor of 0/1."""
        import torch
        self._check_tensor(points, 3)
        res = out if out is not None else torch.empty(points.shape[0], dtype=torch.int32, device=points.device)
        check(lib().fcpwgb_contains_device(self._h, points.data_ptr(), points.shape[0], res.data_ptr(),
                                           self._stream(points)))
        return res

    def has_line_of_sight_tensor(self, points_a, points_b, out=None):
        import torch
        self._check_tensor(points_a, 3)
        self._check_tensor(points_b, 3)
        res = out if out is not None else torch.empty(points_a.shape[0], dtype=torch.int32, device=points_a.device)
        check(lib().fcpwgb_has_line_of_sight_device(self._h, points_a.data_ptr(), points_b.data_ptr(),
                                                    points_a.shape[0], res.data_ptr(), self._stream(points_a)))
        return res

    def closest_distances_f64_tensor(self, spheres):
        """FP64 brute-force closest distances of the (N, 4) query tensor's centres over
        all primitives (an accuracy probe, O(N x primitives)). Returns a float64 tensor."""
        import torch
        self._check_tensor(spheres, 4)
        out = torch.empty(spheres.shape[0], dtype=torch.float64, device=spheres.device)
        check(lib().fcpwgb_closest_distances_f64_device(self._h, spheres.data_ptr(), spheres.shape[0],
                                                        out.data_ptr(), self._stream(spheres)))
        return out

    def export_nodes(self) -> np.ndarray:
        """The device tree (after any refit) in the interop node layout."""
        nodes = np.zeros(self._n_nodes, R.SNCH_NODE if self._snch else R.BVH_NODE)
        check(lib().fcpwgb_gpu_scene_export_nodes(self._h, ptr(nodes)))
        return nodes

    def check_errors(self) -> int:
        w = C.c_uint32(0)
        check(lib().fcpwgb_gpu_scene_check_errors(self._h, C.byref(w)))
        return int(w.value)


class GPUScene2D(_GPUScene):
    DIM = 2


class GPUScene3D(_GPUScene):
    DIM = 3
