"""The traversal statistics behind the benchmark's algorithmic bytes. The
reference counts a closest-point query's work as nodesVisited: one per
expanded inner node and one per primitive test (bvh.inl:1312,1385). The
counting launch of the reference-order kernel (k_binary.cu, stats mode of
fcpwgb_closest_points_traversal_stats) must give the same totals as the
oracle's restatement counted with the GPU traversal's child order
(bvh.slang:458-470), up to the queries whose pruning differs by the last
bit of a box or primitive distance (the kernel may fuse multiply-adds where
the oracle rounds every step)."""
import ctypes as C

import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from fcpw_gb300._lib import check, lib
from helpers import build_scene
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(name):
    if name == "torus":
        v, f = W.torus(256, 128, W.SEED_BASE + 2)
        return 3, v, f, W.uniform_points(200_000, 3, -2.0, 2.0, 81)
    if name == "icosphere":
        v, f = W.perturbed_sphere(32, W.SEED_BASE + 1)
        return 3, v, f, W.uniform_points(200_000, 3, -1.5, 1.5, 82)
    v, sg = W.star_polylines(64, 256, W.SEED_BASE + 3)
    return 2, v, sg, W.uniform_points(200_000, 2, -3.0, 3.0, 83)


@pytest.mark.parametrize("name", ["torus", "icosphere", "stars2d"])
def test_binary_kernel_counts_equal_reference_visits(name):
    import torch
    dim, v, idx, pts = _case(name)
    s = build_scene(dim, v, idx)
    g = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    g.transfer_to_gpu(s)
    g.set_traversal(0)
    n = len(pts)
    sph = R.make_spheres(pts, R.FLT_MAX)
    t = torch.from_numpy(sph.view(np.float32).reshape(n, 4).copy()).cuda()
    out = torch.empty((n, 10), dtype=torch.float32, device="cuda")
    stats = (C.c_uint64 * 8)()
    check(lib().fcpwgb_closest_points_traversal_stats(g.handle, t.data_ptr(), out.data_ptr(), n, stats))
    assert stats[0] == n
    nodes, prims, _ = s.cpu_bvh.export()
    ref, nv = O.closest_points_bvh(dim, nodes, prims, sph, visited=True, gpu_order=True)
    got = int(stats[2]) + int(stats[3])
    want = int(nv.astype(np.int64).sum())
    assert abs(got - want) <= 1e-4 * want, f"{name}: kernel counts {got}, oracle {want}"
    # the counting launch answers the queries too
    d = out[:, 8].cpu().numpy()
    assert np.allclose(d, ref["d"], rtol=1e-5, atol=1e-6)
    assert g.check_errors() == 0


@pytest.mark.parametrize("dim", [2, 3])
def test_silhouette_packet_counts(dim):
    """The silhouette packets' counting launch (fcpwgb_silhouette_traversal_stats)
    returns the same records as the timed launch, and its counts are those of
    warps of 32 lanes: every lane test belongs to a warp step that loaded the
    record; it refuses a configuration that does not run the packets."""
    import torch
    from fcpw_gb300._lib import FcpwError
    if dim == 2:
        v, idx = W.star_polylines(64, 128, W.SEED_BASE + 3)
        pts = W.uniform_points(60_000, 2, -3, 3, 84)
    else:
        v, idx = W.torus(64, 32, W.SEED_BASE + 2)
        pts = W.uniform_points(40_000, 3, -2, 2, 85)
    s = build_scene(dim, v, idx, silhouettes=True)
    g = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    g.transfer_to_gpu(s)
    n = len(pts)
    sph = torch.from_numpy(R.make_spheres(pts, R.FLT_MAX).view(np.float32).reshape(n, 4).copy()).cuda()
    flip = torch.from_numpy((W.rng(86).uniform(0, 1, n) < 0.5).astype(np.uint32)).cuda()
    a = torch.empty((n, 10), dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    g.set_traversal(4, 32)
    check(lib().fcpwgb_find_closest_silhouette_points_device(g.handle, sph.data_ptr(), flip.data_ptr(), a.data_ptr(), n,
                                                             C.c_float(0.0), C.c_float(1e-3), None))
    # the counting call runs on the scene's own stream and shares its scratch arrays
    # with the call above: that one must have finished (one stream per scene at a time)
    torch.cuda.synchronize()
    stats = (C.c_uint64 * 8)()
    check(lib().fcpwgb_silhouette_traversal_stats(g.handle, sph.data_ptr(), flip.data_ptr(), b.data_ptr(), n,
                                                  C.c_float(0.0), C.c_float(1e-3), stats))
    torch.cuda.synchronize()
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    n_q, w_in, w_leaf, w_sil, t_child, t_sil = [int(x) for x in stats[:6]]
    assert n_q == n and w_in > 0 and w_leaf > 0 and w_sil > 0
    assert 0 < t_child <= 2 * 32 * w_in and 0 < t_sil <= 32 * w_sil
    g.set_traversal(0)
    with pytest.raises(FcpwError):
        check(lib().fcpwgb_silhouette_traversal_stats(g.handle, sph.data_ptr(), flip.data_ptr(), b.data_ptr(), n,
                                                      C.c_float(0.0), C.c_float(1e-3), stats))
    assert g.check_errors() == 0
