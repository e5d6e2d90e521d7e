"""GPU parity tests of the binary-tree kernels through the C ABI, against the C
oracle (the reference CPU algorithms restated) and an FP64 brute force."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import EPS32, build_scene, compare_closest, compare_rays, distance_tolerance
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sphere20k():
    v, f = W.perturbed_sphere(32, W.SEED_BASE + 1)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    return s, g


@pytest.fixture(scope="module")
def stars2d():
    v, sg = W.star_polylines(64, 128, W.SEED_BASE + 3)
    s = build_scene(2, v, sg, silhouettes=True)
    g = F.GPUScene2D()
    g.transfer_to_gpu(s)
    return s, g


def _closest(g, pts, r2, record_normals=False):
    out = F.GPUInteractionList()
    g.find_closest_points(pts, np.broadcast_to(np.float32(r2), (len(pts),)).copy(), out, record_normals)
    return out.array()


def test_closest_point_icosphere_infinite_radius(sphere20k):
    s, g = sphere20k
    pts = W.uniform_points(1 << 18, 3, -1.5, 1.5, 11)
    got = _closest(g, pts, R.FLT_MAX)
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    st = compare_closest(3, prims, pts, got, ref)
    assert st["found"] == len(pts)
    assert g.check_errors() == 0


def test_closest_point_against_fp64_brute_force(sphere20k):
    s, g = sphere20k
    pts = W.uniform_points(2048, 3, -1.5, 1.5, 12)
    got = _closest(g, pts, R.FLT_MAX)
    _, prims, _ = s.cpu_bvh.export()
    d64, _ = O.closest_points_brute_f64(3, prims, R.make_spheres(pts, R.FLT_MAX))
    tol = distance_tolerance(pts, got["p"], d64)
    assert np.all(np.abs(got["d"] - d64) <= tol)


def test_closest_point_finite_radius_and_normals(sphere20k):
    s, g = sphere20k
    pts = W.uniform_points(50000, 3, -1.5, 1.5, 13)
    r2 = (0.1 * W.rng(14).uniform(0, 1, len(pts)) * 3.0).astype(np.float32)  # 0.1*U*|extent| as in tests/gpu_tests.cpp:65
    out = F.GPUInteractionList()
    g.find_closest_points(pts, r2, out, True)
    got = out.array()
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, r2), record_normals=True)
    compare_closest(3, prims, pts, got, ref)
    m = ref["index"] != R.UINT_MAX
    assert 0 < m.sum() < len(pts)
    same = got["index"] == ref["index"]
    assert np.allclose(got["n"][same], ref["n"][same], atol=1e-6)
    assert np.allclose(np.linalg.norm(got["n"][m], axis=1), 1.0, atol=1e-5)
    # misses keep the reference defaults
    miss = ~m
    assert np.all(got["d"][miss] == R.FLT_MAX) and np.all(got["index"][miss] == R.UINT_MAX)


def test_closest_point_device_tensor_matches_host(sphere20k):
    import torch
    s, g = sphere20k
    pts = W.uniform_points(100000, 3, -1.5, 1.5, 15)
    host = _closest(g, pts, R.FLT_MAX)
    sph = torch.zeros((len(pts), 4), dtype=torch.float32, device="cuda")
    sph[:, :3] = torch.from_numpy(pts).cuda()
    sph[:, 3] = float(R.FLT_MAX)
    res = g.find_closest_points_tensor(sph)
    torch.cuda.synchronize()
    raw = res.raw.cpu().numpy().view(R.INTERACTION).reshape(-1)
    assert np.array_equal(raw["index"], host["index"])
    assert np.array_equal(raw["d"], host["d"])


def test_closest_point_2d_segments(stars2d):
    s, g = stars2d
    pts = W.uniform_points(100000, 2, -3, 3, 16)
    got = _closest(g, pts, R.FLT_MAX)
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(2, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    compare_closest(2, prims, pts, got, ref)
    assert np.all(got["p"][:, 2] == 0.0)


def test_rays_torus():
    v, f = W.torus(128, 64, W.SEED_BASE + 2)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    n = 100000
    o = W.uniform_points(n, 3, -2, 2, 17)
    d = W.uniform_directions(n, 3, 18)
    tmax = np.full(n, R.FLT_MAX, np.float32)
    out = F.GPUInteractionList()
    g.intersect(o, d, tmax, out)
    got = out.array()
    nodes, prims, _ = s.cpu_bvh.export()
    rays = R.make_rays(o, d, tmax)
    ref, hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    compare_rays(3, prims, rays, got, ref, hit)
    assert 0.05 < hit.mean() < 0.9
    # occlusion variant
    out2 = F.GPUInteractionList()
    g.intersect(o, d, tmax, out2, True)
    ref2, hit2 = O.intersect_rays_bvh(3, nodes, prims, rays, occlusion=True)
    compare_rays(3, prims, rays, out2.array(), ref2, hit2, occl=True)


def test_rays_2d(stars2d):
    s, g = stars2d
    n = 50000
    o = W.uniform_points(n, 2, -3, 3, 19)
    d = W.uniform_directions(n, 2, 20)
    tmax = np.full(n, R.FLT_MAX, np.float32)
    out = F.GPUInteractionList()
    g.intersect(o, d, tmax, out)
    nodes, prims, _ = s.cpu_bvh.export()
    rays = R.make_rays(o, d, tmax)
    ref, hit = O.intersect_rays_bvh(2, nodes, prims, rays)
    compare_rays(2, prims, rays, out.array(), ref, hit)
    occ = F.GPUInteractionList()
    g.intersect(o, d, tmax, occ, True)
    ref2, hit2 = O.intersect_rays_bvh(2, nodes, prims, rays, occlusion=True)
    compare_rays(2, prims, rays, occ.array(), ref2, hit2, occl=True)


def test_silhouettes_2d(stars2d):
    s, g = stars2d
    n = 50000
    pts = W.uniform_points(n, 2, -3, 3, 21)
    flip = (W.rng(22).uniform(0, 1, n) < 0.5).astype(np.uint32)
    out = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(n, R.FLT_MAX, np.float32), flip, out, 0.0, 1e-3)
    got = out.array()
    nodes, _, sils = s.cpu_bvh.export()
    ref = O.silhouettes_bvh(2, nodes, sils, R.make_spheres(pts, R.FLT_MAX), flip)
    fg, fr = got["index"] != R.UINT_MAX, ref["index"] != R.UINT_MAX
    assert (fg != fr).sum() <= max(2, int(1e-4 * n))
    both = fg & fr
    tol = distance_tolerance(pts[both], ref["p"][both][:, :2], ref["d"][both])
    assert np.all(np.abs(got["d"][both] - ref["d"][both]) <= 1e-3 * ref["d"][both] + tol)


def test_silhouettes_3d():
    v, f = W.torus(64, 32, W.SEED_BASE + 2)
    s = build_scene(3, v, f, silhouettes=True)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    n = 20000
    pts = W.uniform_points(n, 3, -2, 2, 23)
    flip = np.zeros(n, np.uint32)
    out = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(n, R.FLT_MAX, np.float32), flip, out)
    got = out.array()
    nodes, _, sils = s.cpu_bvh.export()
    ref = O.silhouettes_bvh(3, nodes, sils, R.make_spheres(pts, R.FLT_MAX), flip)
    fg, fr = got["index"] != R.UINT_MAX, ref["index"] != R.UINT_MAX
    assert (fg != fr).sum() <= max(2, int(1e-4 * n))
    both = fg & fr
    # silhouette test uses a precision threshold (1e-3), as in tests/aggregate_tests.cpp:610
    assert np.all(np.abs(got["d"][both] - ref["d"][both]) <= 1e-3 * np.maximum(ref["d"][both], 1e-3))
    # closest point queries still work on an SNCH tree
    cp = _closest(g, pts, R.FLT_MAX)
    nodes, prims, _ = s.cpu_bvh.export()
    compare_closest(3, prims, pts, cp, O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, R.FLT_MAX)))


def test_sphere_sampling(sphere20k):
    s, g = sphere20k
    n = 50000
    c = W.uniform_points(n, 3, -1.2, 1.2, 24)
    r2 = (W.rng(25).uniform(0.01, 0.3, n) ** 2).astype(np.float32)
    rn = W.rng(26).uniform(0, 1, (n, 3)).astype(np.float32)
    out = F.GPUInteractionList()
    g.intersect(c, r2, rn, out)
    got = out.array()
    nodes, prims, _ = s.cpu_bvh.export()
    ref, hit = O.sphere_sample_bvh(3, nodes, prims, R.make_spheres(c, r2), rn)
    gh = got["index"] != R.UINT_MAX
    assert (gh != hit).sum() <= max(2, int(1e-4 * n))
    both = gh & hit
    same = got["index"][both] == ref["index"][both]
    assert same.mean() > 0.999
    assert np.allclose(got["d"][both][same], ref["d"][both][same], rtol=1e-4)
    assert np.allclose(got["p"][both][same], ref["p"][both][same], atol=1e-5)


def _moved(v, seed, amp=0.02):
    return (v + amp * W.rng(seed).standard_normal(v.shape)).astype(np.float32)


def test_refit_host_update_matches_oracle():
    v, f = W.perturbed_sphere(16, W.SEED_BASE + 5)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    v2 = _moved(v, 27)
    s.update_object_vertices(v2, 0)
    g.refit(s, True)
    nodes, prims, _ = s.cpu_bvh.export()  # prims re-extracted from the moved positions
    ref_nodes = O.refit(3, nodes, prims)
    pts = W.uniform_points(20000, 3, -1.5, 1.5, 28)
    got = _closest(g, pts, R.FLT_MAX)
    ref = O.closest_points_bvh(3, ref_nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    compare_closest(3, prims, pts, got, ref)


def test_update_vertices_device_matches_host_refit():
    import torch
    v, f = W.perturbed_sphere(16, W.SEED_BASE + 6)
    s = build_scene(3, v, f)
    g_host, g_dev = F.GPUScene3D(), F.GPUScene3D()
    g_host.transfer_to_gpu(s)
    g_dev.transfer_to_gpu(s)
    v2 = _moved(v, 29)
    g_dev.update_vertices_tensor(torch.from_numpy(v2).cuda())
    torch.cuda.synchronize()
    s.update_object_vertices(v2, 0)
    g_host.refit(s, True)
    pts = W.uniform_points(20000, 3, -1.5, 1.5, 30)
    a, b = _closest(g_host, pts, R.FLT_MAX), _closest(g_dev, pts, R.FLT_MAX)
    assert np.array_equal(a["index"], b["index"]) and np.array_equal(a["d"], b["d"])


def test_refit_snch_keeps_silhouette_results():
    v, sg = W.star_polylines(16, 64, W.SEED_BASE + 7)
    s = build_scene(2, v, sg, silhouettes=True)
    g = F.GPUScene2D()
    g.transfer_to_gpu(s)
    v2 = _moved(v, 31, amp=0.002)
    s.update_object_vertices(v2, 0)
    g.refit(s, True)
    nodes, prims, sils = s.cpu_bvh.export()
    ref_nodes = O.refit(2, nodes, prims, sils)
    n = 20000
    pts = W.uniform_points(n, 2, -3, 3, 32)
    flip = np.zeros(n, np.uint32)
    out = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(n, R.FLT_MAX, np.float32), flip, out)
    ref = O.silhouettes_bvh(2, ref_nodes, sils, R.make_spheres(pts, R.FLT_MAX), flip)
    got = out.array()
    fg, fr = got["index"] != R.UINT_MAX, ref["index"] != R.UINT_MAX
    assert (fg != fr).sum() <= 2
    both = fg & fr
    assert np.all(np.abs(got["d"][both] - ref["d"][both]) <= 1e-3 * np.maximum(ref["d"][both], 1e-3))


def test_empty_query_batches(sphere20k):
    s, g = sphere20k
    out = F.GPUInteractionList()
    g.find_closest_points(np.zeros((0, 3), np.float32), np.zeros(0, np.float32), out)
    assert len(out) == 0
    g.intersect(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.float32), out)
    assert len(out) == 0


def test_queries_before_transfer_raise():
    g = F.GPUScene3D()
    with pytest.raises(F.FcpwError):
        g.find_closest_points(np.zeros((4, 3), np.float32), np.ones(4, np.float32), F.GPUInteractionList())


@pytest.mark.parametrize("dim", [3, 2])
def test_fp64_brute_force_probe_matches_oracle(sphere20k, stars2d, dim):
    """fcpwgb_closest_distances_f64_device (the accuracy probe) against the C
    oracle's FP64 brute force: the same FP64 formulas, so agreement to 1e-12."""
    import torch
    s, g = sphere20k if dim == 3 else stars2d
    _, prims, _ = s.cpu_bvh.export()
    lo, hi = (-1.5, 1.5) if dim == 3 else (-3.0, 3.0)
    pts = W.uniform_points(700, dim, lo, hi, 33)
    sph = R.make_spheres(pts, R.FLT_MAX)
    d_ref, _ = O.closest_points_brute_f64(dim, prims, sph)
    t = torch.from_numpy(sph.view(np.float32).reshape(-1, 4).copy()).cuda()
    d_gpu = g.closest_distances_f64_tensor(t).cpu().numpy()
    assert np.allclose(d_gpu, d_ref, rtol=1e-12, atol=1e-14)


def test_fast_path_silhouettes_agree_with_binary_kernel(stars2d):
    """With a fast-path configuration silhouette queries are sorted spatially
    and answered by warp packets (k_sil_packet.cu). The same tests prune the
    same subtrees, so against the binary kernel (reference order) the found
    flags are equal and the distances agree to the rounding floor; the
    silhouette differs only on exact ties."""
    s, g = stars2d
    n = 50000
    pts = W.uniform_points(n, 2, -3, 3, 61)
    flip = (W.rng(62).uniform(0, 1, n) < 0.5).astype(np.uint32)
    r2 = np.full(n, R.FLT_MAX, np.float32)
    g.set_traversal(0)
    a = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, r2, flip, a, 0.0, 1e-3)
    g.set_traversal(4, 8, sort_queries=True)
    b = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, r2, flip, b, 0.0, 1e-3)
    g.set_traversal(0)
    a, b = a.array(), b.array()
    fa, fb = a["index"] != R.UINT_MAX, b["index"] != R.UINT_MAX
    assert np.array_equal(fa, fb)
    tol = distance_tolerance(pts[fa], a["p"][fa][:, :2], a["d"][fa])
    assert np.all(np.abs(a["d"][fa].astype(np.float64) - b["d"][fa]) <= tol)


@pytest.mark.parametrize("dim", [3, 2])
def test_contains_and_line_of_sight_match_oracle(dim):
    """Larger seeded cases against the oracle (which equals the reference on the
    golden fixtures); the device-tensor entry points agree with the host ones."""
    import torch
    if dim == 3:
        v, f = W.torus(96, 48, W.SEED_BASE + 63)
        lo, hi = -2.0, 2.0
    else:
        v, f = W.star_polylines(36, 96, W.SEED_BASE + 64)
        lo, hi = -3.0, 3.0
    s = build_scene(dim, v, f)
    g = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    g.transfer_to_gpu(s)
    nodes, prims, _ = s.cpu_bvh.export()
    a = W.uniform_points(60000, dim, lo, hi, 65)
    b = W.uniform_points(60000, dim, lo, hi, 66)
    inside = g.contains(a)
    assert np.array_equal(inside, O.contains_bvh(dim, nodes, prims, a))
    assert 0 < inside.sum() < len(a)
    los = g.has_line_of_sight(a, b)
    assert np.array_equal(los, O.line_of_sight_bvh(dim, nodes, prims, a, b))
    pa = torch.zeros((len(a), 3), dtype=torch.float32, device="cuda")
    pb = torch.zeros((len(a), 3), dtype=torch.float32, device="cuda")
    pa[:, :dim] = torch.from_numpy(a).cuda()
    pb[:, :dim] = torch.from_numpy(b).cuda()
    t_in = g.contains_tensor(pa)
    t_los = g.has_line_of_sight_tensor(pa, pb)
    torch.cuda.synchronize()
    assert np.array_equal(t_in.cpu().numpy().astype(np.uint32), inside)
    assert np.array_equal(t_los.cpu().numpy().astype(np.uint32), los)
    # with a fast-path configuration the points are sorted spatially first:
    # the same answers, in the caller's order, from the host and device entries
    g.set_traversal(4, 32, sort_queries=True)
    assert np.array_equal(g.contains(a), inside)
    t_in2 = g.contains_tensor(pa)
    torch.cuda.synchronize()
    assert np.array_equal(t_in2.cpu().numpy().astype(np.uint32), inside)
    g.set_traversal(0)
    assert g.check_errors() == 0
