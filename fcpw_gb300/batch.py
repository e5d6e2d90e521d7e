"""Batches of scenes: many meshes of uneven size, each with its own query set,
answered by one persistent launch over a forest of wide trees, replayed from a
captured CUDA graph (fcpwgb_gpu_batch_* in include/fcpw_gb300.h). The
reference has no batched API; a batch answers what one GPUScene per mesh and
one findClosestPoints call per mesh would."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import records as R
from ._lib import check, lib, ptr
from .gpu_scene import GPUInteractionList, TensorInteractions, _split_records


def _offsets(query_offsets, n_scenes: int) -> np.ndarray:
    off = np.ascontiguousarray(query_offsets, dtype=np.uint32)
    if off.ndim != 1 or off.shape[0] != n_scenes + 1:
        raise ValueError(f"query_offsets must hold {n_scenes + 1} entries (one per scene plus one)")
    return off


class _GPUSceneBatch:
    DIM = 3

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().fcpwgb_gpu_batch_create(self.DIM, int(device), C.byref(h)))
        self._h = h
        self._n_scenes = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().fcpwgb_gpu_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def n_scenes(self) -> int:
        return self._n_scenes

    def set_scenes(self, scenes) -> None:
        """``scenes``: built Scene2D/3D objects (single object each) or CpuBvh handles.
        Their trees and primitives are copied."""
        bvhs = [s.cpu_bvh if hasattr(s, "cpu_bvh") else s for s in scenes]
        arr = (C.c_void_p * max(len(bvhs), 1))(*[b.handle.value for b in bvhs])
        check(lib().fcpwgb_gpu_batch_set_scenes(self._h, arr, len(bvhs)))
        self._n_scenes = len(bvhs)

    def set_traversal(self, branching: int = 8, bits: int = 8, persistent: bool = False,
                      precise: bool = True, packet: bool = False, leaf_size: int = 0, short_stack: int = 16,
                      threads_per_query: int = 1) -> None:
        from ._lib import TraversalConfig
        cfg = TraversalConfig(int(branching), int(bits), 128, 1, int(bool(persistent)), int(bool(precise)),
                              int(bool(packet)), int(leaf_size), int(short_stack), int(threads_per_query))
        check(lib().fcpwgb_gpu_batch_set_traversal(self._h, C.byref(cfg)))

    def get_traversal(self) -> dict:
        from ._lib import TraversalConfig
        cfg = TraversalConfig()
        check(lib().fcpwgb_gpu_batch_get_traversal(self._h, C.byref(cfg)))
        return {f: getattr(cfg, f) for f, _ in TraversalConfig._fields_}

    def use_graph(self, on: bool = True) -> None:
        check(lib().fcpwgb_gpu_batch_use_graph(self._h, int(bool(on))))

    def find_closest_points_tensor(self, spheres, query_offsets, record_normals: bool = False,
                                   out=None) -> TensorInteractions:
        """``spheres``: (N, 4) float32 CUDA tensor, grouped by scene as ``query_offsets``
        says. Asynchronous on the current torch stream; returns device views."""
        import torch
        if (spheres.dtype != torch.float32 or not spheres.is_cuda or not spheres.is_contiguous()
                or spheres.dim() != 2 or spheres.shape[1] != 4):
            raise ValueError("spheres must be a contiguous float32 CUDA tensor of shape (N, 4)")
        off = _offsets(query_offsets, self._n_scenes)
        n = spheres.shape[0]
        if int(off[-1]) != n:
            raise ValueError("query_offsets[-1] must equal the number of queries")
        raw = out if out is not None else torch.empty((n, 10), dtype=torch.float32, device=spheres.device)
        stream = C.c_void_p(torch.cuda.current_stream(spheres.device).cuda_stream)
        check(lib().fcpwgb_gpu_batch_find_closest_points_device(self._h, spheres.data_ptr(), ptr(off), len(off),
                                                                raw.data_ptr(), int(bool(record_normals)), stream))
        return _split_records(raw)

    def find_closest_points(self, query_points, squared_max_radii, query_offsets,
                            interactions: GPUInteractionList, record_normals: bool = False) -> None:
        """Host arrays, synchronous (the shape of GPUScene.find_closest_points)."""
        pts = np.ascontiguousarray(query_points, np.float32)
        if pts.ndim != 2 or pts.shape[1] != self.DIM:
            raise ValueError(f"query_points must have shape (N, {self.DIM})")
        spheres = R.make_spheres(pts, np.asarray(squared_max_radii, np.float32))
        off = _offsets(query_offsets, self._n_scenes)
        if int(off[-1]) != len(spheres):
            raise ValueError("query_offsets[-1] must equal the number of queries")
        if not isinstance(interactions, GPUInteractionList):
            raise TypeError("interactions must be a GPUInteractionList")
        interactions._a = R.default_interactions(len(spheres))
        check(lib().fcpwgb_gpu_batch_find_closest_points(self._h, ptr(spheres), ptr(off), len(off),
                                                         ptr(interactions._a), int(bool(record_normals))))

    def traversal_stats(self, spheres, query_offsets, out=None) -> dict:
        """Per-batch traversal counts of the current variant (device tensors)."""
        import torch
        off = _offsets(query_offsets, self._n_scenes)
        n = spheres.shape[0]
        raw = out if out is not None else torch.empty((n, 10), dtype=torch.float32, device=spheres.device)
        st = (C.c_uint64 * 8)()
        check(lib().fcpwgb_gpu_batch_traversal_stats(self._h, spheres.data_ptr(), ptr(off), len(off),
                                                     raw.data_ptr(), st))
        return {"queries": int(st[0]), "expanded": int(st[2]), "prim_tests": int(st[3]),
                "warp_record_loads": int(st[4]), "warp_prim_loads": int(st[5])}

    def info(self) -> dict:
        v = [C.c_uint32(0) for _ in range(4)]
        check(lib().fcpwgb_gpu_batch_info(self._h, *[C.byref(x) for x in v]))
        return dict(zip(["scenes", "wide_nodes", "primitives", "sort_cells"], [int(x.value) for x in v]))

    def check_errors(self) -> int:
        w = C.c_uint32(0)
        check(lib().fcpwgb_gpu_batch_check_errors(self._h, C.byref(w)))
        return int(w.value)


class GPUSceneBatch3D(_GPUSceneBatch):
    DIM = 3


class GPUSceneBatch2D(_GPUSceneBatch):
    DIM = 2


def autotune_batch(batch: _GPUSceneBatch, spheres, query_offsets, space=None, reps: int = 3,
                   precise: bool = True):
    """Times the batched closest point launch (graph replay) for the candidates
    of fcpw_gb300.autotune.staged_search on the caller's queries and keeps the
    fastest. Returns (best config, [(config, ms per call)])."""
    import torch
    from .autotune import staged_search
    out = torch.empty((spheres.shape[0], 10), dtype=torch.float32, device=spheres.device)
    stream = torch.cuda.current_stream(spheres.device)

    def set_cfg(cfg):
        batch.set_traversal(cfg["branching"], cfg["bits"], cfg["persistent"], precise, cfg["packet"],
                            cfg["leaf_size"], cfg["short_stack"], cfg.get("threads_per_query", 1))

    def measure(cfg):
        set_cfg(cfg)
        batch.find_closest_points_tensor(spheres, query_offsets, out=out)  # forest build + graph capture
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(reps):
            batch.find_closest_points_tensor(spheres, query_offsets, out=out)
        end.record(stream)
        end.synchronize()
        return start.elapsed_time(end) / reps

    best, table = staged_search(measure, space, precise=precise)
    set_cfg(best)
    return best, table
