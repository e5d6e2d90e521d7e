"""ctypes binding of the C ABI declared in include/fcpw_gb300.h.

The library is loaded from ``fcpw_gb300/lib/libfcpw_gb300.so`` (built in-tree by
``fcpw_gb300.build.build()``). There is no fallback: when the library is missing
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libfcpw_gb300.so"
_lib = None

c_void_p, c_int, c_uint32, c_float = C.c_void_p, C.c_int, C.c_uint32, C.c_float
P = C.c_void_p

# name -> (restype, argtypes); mirrors include/fcpw_gb300.h
SIGNATURES = {
    "fcpwgb_last_error": (C.c_char_p, []),
    "fcpwgb_version": (C.c_char_p, []),
    "fcpwgb_device_count": (c_int, []),
    "fcpwgb_debug_fail_allocations": (c_int, [c_int, c_int]),
    "fcpwgb_cpu_bvh_build": (c_int, [c_int, P, c_uint32, P, c_uint32, c_int, c_int, C.POINTER(c_void_p)]),
    "fcpwgb_cpu_bvh_destroy": (None, [P]),
    "fcpwgb_cpu_bvh_info": (c_int, [P, P]),
    "fcpwgb_cpu_bvh_export": (c_int, [P, P, P, P]),
    "fcpwgb_cpu_bvh_export_topology": (c_int, [P, P, P, P, P]),
    "fcpwgb_cpu_bvh_update_positions": (c_int, [P, P]),
    "fcpwgb_cpu_bvh_export_wide": (c_int, [P, c_int, c_int, c_int, P, P, C.POINTER(c_uint32),
                                           C.POINTER(c_uint32)]),
    "fcpwgb_gpu_scene_create": (c_int, [c_int, c_int, C.POINTER(c_void_p)]),
    "fcpwgb_gpu_scene_destroy": (None, [P]),
    "fcpwgb_gpu_scene_transfer": (c_int, [P, c_int, P, c_uint32, P, c_uint32, P, c_uint32, P, c_uint32]),
    "fcpwgb_gpu_scene_transfer_cpu_bvh": (c_int, [P, P]),
    "fcpwgb_gpu_scene_build": (c_int, [P, P, c_uint32, P, c_uint32, c_uint32]),
    "fcpwgb_gpu_scene_build_sah": (c_int, [P, P, c_uint32, P, c_uint32, c_int]),
    "fcpwgb_gpu_scene_build_sah_device": (c_int, [P, P, c_uint32, P, c_uint32, c_int, P]),
    "fcpwgb_cpu_instances_build": (c_int, [c_int, c_int, P, c_uint32, P, P, P, c_uint32, P]),
    "fcpwgb_cpu_instances_destroy": (None, [P]),
    "fcpwgb_cpu_instances_export": (c_int, [P, P, P, P, P]),
    "fcpwgb_gpu_scene_transfer_instanced": (c_int, [P, P]),
    "fcpwgb_find_closest_points_instanced": (c_int, [P, P, P, P, c_uint32, c_int]),
    "fcpwgb_find_closest_points_instanced_device": (c_int, [P, P, P, P, c_uint32, c_int, P]),
    "fcpwgb_intersect_rays_instanced": (c_int, [P, P, P, P, c_uint32, c_int]),
    "fcpwgb_intersect_rays_instanced_device": (c_int, [P, P, P, P, c_uint32, c_int, P]),
    "fcpwgb_intersect_spheres_instanced": (c_int, [P, P, P, P, P, c_uint32]),
    "fcpwgb_intersect_spheres_instanced_device": (c_int, [P, P, P, P, P, c_uint32, P]),
    "fcpwgb_find_closest_silhouette_points_instanced": (c_int, [P, P, P, P, P, c_uint32, c_float, c_float]),
    "fcpwgb_find_closest_silhouette_points_instanced_device": (c_int, [P, P, P, P, P, c_uint32, c_float, c_float,
                                                                       P]),
    "fcpwgb_gpu_scene_refit_object": (c_int, [P, c_uint32, P, P]),
    "fcpwgb_gpu_scene_update_object_vertices_device": (c_int, [P, c_uint32, P, c_uint32, P]),
    "fcpwgb_gpu_scene_export_top_nodes": (c_int, [P, P, C.POINTER(c_uint32)]),
    "fcpwgb_gpu_scene_build_device": (c_int, [P, P, c_uint32, P, c_uint32, c_uint32, P]),
    "fcpwgb_gpu_scene_info": (c_int, [P, P]),
    "fcpwgb_gpu_scene_refit": (c_int, [P, P, P]),
    "fcpwgb_gpu_scene_update_vertices_device": (c_int, [P, P, c_uint32, P]),
    "fcpwgb_gpu_scene_update_vertices_device_static": (c_int, [P, P, c_uint32, P]),
    "fcpwgb_debug_fill_static_scratch": (c_int, [P, c_uint32, c_uint32]),
    "fcpwgb_find_closest_points": (c_int, [P, P, P, c_uint32, c_int]),
    "fcpwgb_intersect_rays": (c_int, [P, P, P, c_uint32, c_int]),
    "fcpwgb_intersect_spheres": (c_int, [P, P, P, P, c_uint32]),
    "fcpwgb_find_closest_silhouette_points": (c_int, [P, P, P, P, c_uint32, c_float, c_float]),
    "fcpwgb_find_closest_points_device": (c_int, [P, P, P, c_uint32, c_int, P]),
    "fcpwgb_intersect_rays_device": (c_int, [P, P, P, c_uint32, c_int, P]),
    "fcpwgb_intersect_spheres_device": (c_int, [P, P, P, P, c_uint32, P]),
    "fcpwgb_find_closest_silhouette_points_device": (c_int, [P, P, P, P, c_uint32, c_float, c_float, P]),
    "fcpwgb_closest_points_traversal_stats": (c_int, [P, P, P, c_uint32, P]),
    "fcpwgb_silhouette_traversal_stats": (c_int, [P, P, P, P, c_uint32, c_float, c_float, P]),
    "fcpwgb_gpu_scene_export_nodes": (c_int, [P, P]),
    "fcpwgb_closest_point_backward_device": (c_int, [P, P, P, P, c_uint32, P, P, P]),
    "fcpwgb_ray_backward_device": (c_int, [P, P, P, P, c_uint32, P, P, P, P]),
    "fcpwgb_gpu_scene_enable_kernel_timing": (c_int, [P, c_int]),
    "fcpwgb_gpu_scene_kernel_time": (c_int, [P, C.POINTER(C.c_double), C.POINTER(c_uint32)]),
    "fcpwgb_gpu_scene_set_traversal": (c_int, [P, P]),
    "fcpwgb_gpu_scene_get_traversal": (c_int, [P, P]),
    "fcpwgb_gpu_scene_check_errors": (c_int, [P, C.POINTER(c_uint32)]),
    "fcpwgb_closest_distances_f64_device": (c_int, [P, P, c_uint32, P, P]),
    "fcpwgb_cpu_bvh_save": (c_int, [P, C.c_char_p, P, c_uint32]),
    "fcpwgb_gpu_scene_load": (c_int, [P, C.c_char_p]),
    "fcpwgb_scene_file_info": (c_int, [C.c_char_p, P, C.POINTER(c_uint32)]),
    "fcpwgb_contains": (c_int, [P, P, c_uint32, P]),
    "fcpwgb_contains_device": (c_int, [P, P, c_uint32, P, P]),
    "fcpwgb_has_line_of_sight": (c_int, [P, P, P, c_uint32, P]),
    "fcpwgb_has_line_of_sight_device": (c_int, [P, P, P, c_uint32, P, P]),
    "fcpwgb_gpu_batch_create": (c_int, [c_int, c_int, C.POINTER(c_void_p)]),
    "fcpwgb_gpu_batch_destroy": (None, [P]),
    "fcpwgb_gpu_batch_set_scenes": (c_int, [P, P, c_uint32]),
    "fcpwgb_gpu_batch_set_traversal": (c_int, [P, P]),
    "fcpwgb_gpu_batch_get_traversal": (c_int, [P, P]),
    "fcpwgb_gpu_batch_use_graph": (c_int, [P, c_int]),
    "fcpwgb_gpu_batch_find_closest_points_device": (c_int, [P, P, P, c_uint32, P, c_int, P]),
    "fcpwgb_gpu_batch_find_closest_points": (c_int, [P, P, P, c_uint32, P, c_int]),
    "fcpwgb_gpu_batch_traversal_stats": (c_int, [P, P, P, c_uint32, P, P]),
    "fcpwgb_gpu_batch_info": (c_int, [P, C.POINTER(c_uint32), C.POINTER(c_uint32), C.POINTER(c_uint32),
                                      C.POINTER(c_uint32)]),
    "fcpwgb_gpu_batch_check_errors": (c_int, [P, C.POINTER(c_uint32)]),
}


class BvhInfo(C.Structure):
    _fields_ = [("dim", c_int), ("bvh_type", c_int), ("n_nodes", c_uint32), ("n_leaves", c_uint32),
                ("max_depth", c_uint32), ("n_primitives", c_uint32), ("n_silhouettes", c_uint32),
                ("n_vertices", c_uint32)]


class TraversalConfig(C.Structure):
    _fields_ = [("branching", c_int), ("bits", c_int), ("block_size", c_int), ("sort_queries", c_int),
                ("persistent", c_int), ("precise", c_int), ("packet", c_int), ("leaf_size", c_int),
                ("short_stack", c_int), ("threads_per_query", c_int)]


class FcpwError(RuntimeError):
    """A non-zero status returned by the native library."""

    def __init__(self, code: int, message: str):
        super().__init__(f"fcpw_gb300 error {code}: {message}")
        self.code = code


def library_path() -> Path:
    return _LIB_PATH


def lib():
    """Loads the native library (once) and declares every entry point."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"fcpw_gb300 native library not built: {_LIB_PATH} is missing "
                               "(run `python -c 'import fcpw_gb300.build as b; b.build()'`)")
        handle = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        msg = lib().fcpwgb_last_error()
        raise FcpwError(rc, msg.decode() if msg else "")


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
