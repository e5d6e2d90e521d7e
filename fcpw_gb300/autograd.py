"""Differentiable closest-point distance and ray-hit distance behind
``torch.autograd.Function`` (no counterpart in the reference, which has no
backward).

Forward runs the GPU query once and keeps its interaction records; backward
reads them back (nothing is traversed again) through
fcpwgb_closest_point_backward_device / fcpwgb_ray_backward_device, giving
d/dquery and d/dvertex with a deterministic vertex reduction. With
``refit=True`` the forward first moves the scene's vertices to ``vertices``
on the device and refits the tree, so gradients refer to that geometry.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import records as R
from ._lib import check, lib


def _stream(t):
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _check(t, name, cols=None):
    if t.dtype != torch.float32 or not t.is_cuda:
        raise ValueError(f"{name} must be a float32 CUDA tensor")
    if cols is not None and (t.dim() != 2 or t.shape[1] != cols):
        raise ValueError(f"{name} must have shape (N, {cols})")


class ClosestPointDistance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, vertices, gpu, refit: bool):
        dim = gpu.DIM
        _check(x, "x", dim)
        _check(vertices, "vertices", dim)
        if refit:
            gpu.update_vertices_tensor(vertices.detach().contiguous())
        n = x.shape[0]
        spheres = torch.zeros((n, 4), dtype=torch.float32, device=x.device)
        spheres[:, :dim] = x.detach()
        spheres[:, 3] = float(R.FLT_MAX)
        rec = gpu.find_closest_points_tensor(spheres)
        ctx.save_for_backward(spheres, rec.raw)
        ctx.gpu = gpu
        ctx.n_vertices = vertices.shape[0]
        d = rec.d.clone()
        d[rec.index == -1] = float("inf")
        return d

    @staticmethod
    def backward(ctx, grad_d):
        spheres, raw = ctx.saved_tensors
        gpu = ctx.gpu
        dim = gpu.DIM
        n = spheres.shape[0]
        g = grad_d.contiguous().to(torch.float32)
        grad_x = torch.empty((n, dim), dtype=torch.float32, device=spheres.device)
        grad_v = torch.empty((ctx.n_vertices, dim), dtype=torch.float32, device=spheres.device)
        check(lib().fcpwgb_closest_point_backward_device(gpu.handle, spheres.data_ptr(), raw.data_ptr(), g.data_ptr(),
                                                         n, grad_x.data_ptr(), grad_v.data_ptr(), _stream(g)))
        return grad_x, grad_v, None, None


class RayHitDistance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, origins, directions, vertices, gpu, refit: bool):
        dim = gpu.DIM
        _check(origins, "origins", dim)
        _check(directions, "directions", dim)
        _check(vertices, "vertices", dim)
        if refit:
            gpu.update_vertices_tensor(vertices.detach().contiguous())
        n = origins.shape[0]
        rays = torch.zeros((n, 10), dtype=torch.float32, device=origins.device)
        rays[:, 0:dim] = origins.detach()
        rays[:, 3:3 + dim] = directions.detach()
        rays[:, 6:9] = 1.0 / rays[:, 3:6]
        rays[:, 9] = float(R.FLT_MAX)
        rec = gpu.intersect_tensor(rays)
        ctx.save_for_backward(rays, rec.raw)
        ctx.gpu = gpu
        ctx.n_vertices = vertices.shape[0]
        t = rec.d.clone()
        t[rec.index == -1] = float("inf")
        return t

    @staticmethod
    def backward(ctx, grad_t):
        rays, raw = ctx.saved_tensors
        gpu = ctx.gpu
        dim = gpu.DIM
        n = rays.shape[0]
        g = grad_t.contiguous().to(torch.float32)
        grad_o = torch.empty((n, dim), dtype=torch.float32, device=rays.device)
        grad_d = torch.empty((n, dim), dtype=torch.float32, device=rays.device)
        grad_v = torch.empty((ctx.n_vertices, dim), dtype=torch.float32, device=rays.device)
        check(lib().fcpwgb_ray_backward_device(gpu.handle, rays.data_ptr(), raw.data_ptr(), g.data_ptr(), n,
                                               grad_o.data_ptr(), grad_d.data_ptr(), grad_v.data_ptr(), _stream(g)))
        return grad_o, grad_d, grad_v, None, None


def closest_point_distance(gpu, x, vertices, refit: bool = True):
    """Unsigned distance from every row of ``x`` to the scene, differentiable in
    ``x`` and ``vertices`` (caller vertex order of the transferred scene)."""
    return ClosestPointDistance.apply(x, vertices, gpu, refit)


def ray_hit_distance(gpu, origins, directions, vertices, refit: bool = True):
    """First-hit distance t along each ray (inf on a miss), differentiable in the
    ray origins, directions and ``vertices``."""
    return RayHitDistance.apply(origins, directions, vertices, gpu, refit)
