"""fcpw_gb300 — GB300-native GPU query path for FCPW scenes.

Drop-in for the reference's ``fcpw.GPUScene2D/3D`` path: a host-side scene and
SAH BVH producer (``Scene2D/3D``), the GPU scene classes and their record and
list types, all on top of the C ABI in include/fcpw_gb300.h.
"""
from ._lib import FcpwError, library_path
from .batch import GPUSceneBatch2D, GPUSceneBatch3D
from .gpu_scene import (GPUBoundingSphere, GPUBoundingSphereList, GPUFloat2, GPUFloat3, GPUFloat3List,
                        GPUInteraction, GPUInteractionList, GPURay, GPURayList, GPUScene2D, GPUScene3D,
                        TensorInteractions, Uint32List)
from .scene import AggregateType, CpuBvh, PrimitiveType, Scene2D, Scene3D, scene_file_info

__all__ = [
    "AggregateType", "PrimitiveType", "Scene2D", "Scene3D", "CpuBvh", "GPUScene2D", "GPUScene3D",
    "GPUFloat2", "GPUFloat3", "GPURay", "GPUBoundingSphere", "GPUInteraction", "GPUFloat3List", "GPURayList",
    "GPUBoundingSphereList", "GPUInteractionList", "Uint32List", "TensorInteractions", "FcpwError",
    "library_path", "GPUSceneBatch2D", "GPUSceneBatch3D", "scene_file_info",
]
