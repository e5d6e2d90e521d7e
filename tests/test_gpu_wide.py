"""GPU parity of the wide / quantised closest-point kernels against the oracle
(reference CPU order) and FP64, for every branching factor and box precision."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import build_scene, compare_closest, compare_rays, edge_aimed_rays, leaf_positions, relative_error
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torus():
    v, f = W.torus(256, 128, W.SEED_BASE + 2)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    pts = W.uniform_points(120000, 3, -2, 2, 41)
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    return s, g, pts, ref, prims


def _run(g, pts, r2=None):
    out = F.GPUInteractionList()
    r2 = np.full(len(pts), R.FLT_MAX, np.float32) if r2 is None else r2
    g.find_closest_points(pts, r2, out)
    return out.array()


@pytest.mark.parametrize("branching", [2, 4, 8])
@pytest.mark.parametrize("bits", [32, 16, 8])
def test_wide_variants_match_oracle(torus, branching, bits):
    s, g, pts, ref, prims = torus
    g.set_traversal(branching, bits, sort_queries=True, persistent=True, precise=False)
    got = _run(g, pts)
    compare_closest(3, prims, pts, got, ref, f"wide {branching}/{bits}")
    assert g.check_errors() == 0


@pytest.mark.parametrize("sort_queries,persistent", [(False, False), (True, False), (False, True)])
def test_wide_scheduling_options_agree(torus, sort_queries, persistent):
    s, g, pts, ref, prims = torus
    g.set_traversal(4, 8, sort_queries=sort_queries, persistent=persistent, precise=False)
    got = _run(g, pts)
    compare_closest(3, prims, pts, got, ref, "wide scheduling")


@pytest.mark.parametrize("branching", [2, 4, 8])
@pytest.mark.parametrize("bits", [32, 16, 8])
def test_packet_traversal_matches_oracle(torus, branching, bits):
    """Warp packets: each query still prunes with its own radius."""
    s, g, pts, ref, prims = torus
    g.set_traversal(branching, bits, sort_queries=True, precise=False, packet=True)
    got = _run(g, pts)
    compare_closest(3, prims, pts, got, ref, f"packet {branching}/{bits}")
    assert g.check_errors() == 0


def test_packet_unsorted_finite_radius_and_normals(torus):
    """Packets of unsorted queries with finite, different radii per lane."""
    s, g, pts, ref, prims = torus
    r2 = (0.05 * W.rng(43).uniform(0, 1, len(pts))).astype(np.float32)
    nodes, _, _ = s.cpu_bvh.export()
    ref2 = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, r2), record_normals=True)
    g.set_traversal(4, 8, sort_queries=False, precise=False, packet=True)
    out = F.GPUInteractionList()
    g.find_closest_points(pts, r2, out, True)
    got = out.array()
    compare_closest(3, prims, pts, got, ref2, "packet finite radius")
    same = (got["index"] == ref2["index"]) & (ref2["index"] != R.UINT_MAX)
    assert np.allclose(got["n"][same], ref2["n"][same], atol=1e-6)


def test_precise_mode_within_1e6_of_fp64(torus):
    s, g, pts, ref, prims = torus
    g.set_traversal(4, 8, precise=True)
    sub = pts[:3000]
    got = _run(g, sub)
    d64, _ = O.closest_points_brute_f64(3, prims, R.make_spheres(sub, R.FLT_MAX))
    rel = relative_error(got["d"], d64)
    assert rel.max() <= 1e-6, f"max relative error {rel.max():.3e}"
    # plain FP32 (reference arithmetic) for comparison: larger near the surface
    g.set_traversal(0)
    plain = _run(g, sub)
    assert relative_error(plain["d"], d64).max() >= rel.max()


def test_wide_finite_radius_and_normals(torus):
    s, g, pts, ref, prims = torus
    r2 = (0.05 * W.rng(42).uniform(0, 1, len(pts))).astype(np.float32)
    nodes, _, _ = s.cpu_bvh.export()
    ref2 = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, r2), record_normals=True)
    g.set_traversal(8, 16, precise=False)
    out = F.GPUInteractionList()
    g.find_closest_points(pts, r2, out, True)
    got = out.array()
    compare_closest(3, prims, pts, got, ref2, "wide finite radius")
    same = (got["index"] == ref2["index"]) & (ref2["index"] != R.UINT_MAX)
    assert np.allclose(got["n"][same], ref2["n"][same], atol=1e-6)


@pytest.mark.parametrize("cfg", [dict(branching=4, bits=32, packet=True), dict(branching=4, bits=8, persistent=False),
                                 dict(branching=2, bits=16, persistent=True)])
def test_precise_mode_finite_radius_and_normals(torus, cfg):
    """Precise mode on triangles writes its records in the refinement pass:
    the face normal of the primitive it keeps, the caller's radius respected
    by the winner and the runner-up, and FP64-accurate distances."""
    s, g, pts, ref, prims = torus
    sub = pts[:40000]
    r2 = (0.05 * W.rng(45).uniform(0, 1, len(sub))).astype(np.float32)
    nodes, _, _ = s.cpu_bvh.export()
    ref2 = O.closest_points_bvh(3, nodes, prims, R.make_spheres(sub, r2), record_normals=True)
    g.set_traversal(precise=True, **cfg)
    out = F.GPUInteractionList()
    g.find_closest_points(sub, r2, out, True)
    got = out.array()
    g.set_traversal(0)
    compare_closest(3, prims, sub, got, ref2, f"precise finite radius {cfg}")
    found = got["index"] != R.UINT_MAX
    assert np.all(got["d"][found].astype(np.float64) ** 2 <= r2[found].astype(np.float64) * (1 + 1e-6))
    same = (got["index"] == ref2["index"]) & found
    assert np.allclose(got["n"][same], ref2["n"][same], atol=1e-6)
    # the normal is the kept primitive's own face normal
    pos = leaf_positions(prims)[got["index"][found].astype(np.int64)]
    p = prims[pos]
    n = np.cross(p["pb"][:, :3].astype(np.float64) - p["pa"][:, :3], p["pc"][:, :3].astype(np.float64) - p["pa"][:, :3])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    assert np.allclose(got["n"][found], n, atol=1e-5)
    d64, _ = O.closest_points_brute_f64(3, prims, R.make_spheres(sub[found], R.FLT_MAX))
    assert relative_error(got["d"][found], d64).max() <= 1e-6


def test_wide_after_refit(torus):
    v, f = W.perturbed_sphere(24, W.SEED_BASE + 8)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    g.set_traversal(4, 8, precise=False)
    pts = W.uniform_points(30000, 3, -1.5, 1.5, 43)
    _run(g, pts)  # builds the wide tree
    v2 = (v * 1.1 + 0.01 * W.rng(44).standard_normal(v.shape)).astype(np.float32)
    s.update_object_vertices(v2, 0)
    g.refit(s, True)
    got = _run(g, pts)
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(3, O.refit(3, nodes, prims), prims, R.make_spheres(pts, R.FLT_MAX))
    compare_closest(3, prims, pts, got, ref, "wide after refit")


def test_wide_2d_segments():
    v, sg = W.star_polylines(64, 128, W.SEED_BASE + 3)
    s = build_scene(2, v, sg)
    g = F.GPUScene2D()
    g.transfer_to_gpu(s)
    pts = W.uniform_points(60000, 2, -3, 3, 45)
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(2, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    for b, q in [(4, 8), (8, 16), (2, 32)]:
        g.set_traversal(b, q, precise=False)
        compare_closest(2, prims, pts, _run(g, pts), ref, f"2D wide {b}/{q}")


@pytest.mark.parametrize("branching", [2, 4, 8])
@pytest.mark.parametrize("bits", [32, 16, 8])
@pytest.mark.parametrize("schedule", ["thread", "refill", "packet"])
def test_wide_rays_match_oracle(torus, branching, bits, schedule):
    """Rays on the wide trees (sorted by direction octant and origin), one
    thread per ray, lanes refilled from a counter (persistent), or warp
    packets, against the reference CPU order."""
    packet = schedule == "packet"
    s, g, pts, ref, prims = torus
    n = 60000
    o = W.uniform_points(n, 3, -2, 2, 51)
    d = W.uniform_directions(n, 3, 52)
    tmax = np.full(n, R.FLT_MAX, np.float32)
    nodes, _, _ = s.cpu_bvh.export()
    rays = R.make_rays(o, d, tmax)
    ref_out, ref_hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    g.set_traversal(branching, bits, sort_queries=True, packet=packet, persistent=schedule == "refill")
    out = F.GPUInteractionList()
    g.intersect(o, d, tmax, out)
    compare_rays(3, prims, rays, out.array(), ref_out, ref_hit)
    out2 = F.GPUInteractionList()
    g.intersect(o, d, tmax, out2, True)
    ref2, hit2 = O.intersect_rays_bvh(3, nodes, prims, rays, occlusion=True)
    compare_rays(3, prims, rays, out2.array(), ref2, hit2, occl=True)
    assert g.check_errors() == 0


@pytest.mark.parametrize("cfg", [dict(branching=0), dict(branching=2, bits=32, sort_queries=True),
                                 dict(branching=4, bits=8, sort_queries=True, packet=True),
                                 dict(branching=8, bits=16, sort_queries=False, persistent=False),
                                 dict(branching=4, bits=32, sort_queries=True, persistent=False),
                                 dict(branching=4, bits=32, sort_queries=False, persistent=True)])
def test_rays_aimed_at_edges_and_vertices(torus, cfg):
    """Rays through edge midpoints and vertices (grazing hits, equidistant
    ties between the faces of an edge or a vertex): every kernel passes the
    tie-aware ray check against the reference order, first hit and
    occlusion."""
    s, g, pts, ref, prims = torus
    v, f = s.positions(0), s.indices(0)
    n = 40000
    o = W.uniform_points(n, 3, -2, 2, 57)
    d = edge_aimed_rays(v, f, o, 58)
    tmax = np.full(n, R.FLT_MAX, np.float32)
    nodes, _, _ = s.cpu_bvh.export()
    rays = R.make_rays(o, d, tmax)
    ref_out, ref_hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    g.set_traversal(**cfg)
    out = F.GPUInteractionList()
    g.intersect(o, d, tmax, out)
    compare_rays(3, prims, rays, out.array(), ref_out, ref_hit, what=f"edge rays {cfg}")
    occ = F.GPUInteractionList()
    g.intersect(o, d, tmax, occ, True)
    ref2, hit2 = O.intersect_rays_bvh(3, nodes, prims, rays, occlusion=True)
    compare_rays(3, prims, rays, occ.array(), ref2, hit2, occl=True, what=f"edge occlusion {cfg}")
    g.set_traversal(0)
    assert g.check_errors() == 0


def test_coherent_rays_keep_the_callers_order(torus):
    """Camera rays from one eye, in pixel order: the sort sees that consecutive
    rays point alike and leaves them in the caller's order (the traversal
    then reads the caller's array); the records equal those of the unsorted
    configuration and match the oracle."""
    s, g, pts, ref, prims = torus
    h, w = 192, 256
    ys, xs = np.mgrid[0:h, 0:w]
    u = ((xs.ravel() + 0.5) / w * 2 - 1) * 0.45
    v = ((ys.ravel() + 0.5) / h * 2 - 1) * 0.45 - 0.3
    d = np.stack([u, np.ones_like(u), v], 1)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    o = np.broadcast_to(np.array([0.0, -5.0, 1.5], np.float32), d.shape).copy()
    tmax = np.full(len(d), R.FLT_MAX, np.float32)
    nodes, _, _ = s.cpu_bvh.export()
    rays = R.make_rays(o, d, tmax)
    ref_out, ref_hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    outs = []
    for cfg in [dict(sort_queries=False), dict(sort_queries=True), dict(sort_queries=True, packet=True)]:
        g.set_traversal(4, 32, **cfg)
        out = F.GPUInteractionList()
        g.intersect(o, d, tmax, out)
        outs.append(out.array())
        compare_rays(3, prims, rays, outs[-1], ref_out, ref_hit)
    g.set_traversal(0)
    assert outs[1].tobytes() == outs[0].tobytes()
    assert g.check_errors() == 0


def test_wide_rays_finite_tmax_unsorted_and_2d():
    v, sg = W.star_polylines(16, 64, W.SEED_BASE + 53)
    s = build_scene(2, v, sg)
    g = F.GPUScene2D()
    g.transfer_to_gpu(s)
    n = 30000
    o = W.uniform_points(n, 2, -3, 3, 54)
    d = W.uniform_directions(n, 2, 55)
    tmax = W.rng(56).uniform(0.1, 3.0, n).astype(np.float32)
    nodes, prims, _ = s.cpu_bvh.export()
    rays = R.make_rays(o, d, tmax)
    ref_out, ref_hit = O.intersect_rays_bvh(2, nodes, prims, rays)
    for cfg in [(4, 8, True, False), (8, 16, False, False), (2, 32, True, False), (4, 32, True, True),
                (8, 8, False, True)]:
        g.set_traversal(cfg[0], cfg[1], sort_queries=cfg[2], packet=cfg[3])
        out = F.GPUInteractionList()
        g.intersect(o, d, tmax, out)
        compare_rays(2, prims, rays, out.array(), ref_out, ref_hit)
        occ = F.GPUInteractionList()
        g.intersect(o, d, tmax, occ, True)
        ref2, hit2 = O.intersect_rays_bvh(2, nodes, prims, rays, occlusion=True)
        compare_rays(2, prims, rays, occ.array(), ref2, hit2, occl=True)
    assert g.check_errors() == 0


@pytest.mark.parametrize("packet", [False, True])
def test_precise_mode_near_ties_2d_within_1e6(packet):
    """2D polylines: adjacent segments tie within FP32 rounding near shared
    vertices; the precise mode refines the winner and the runner-up in FP64."""
    v, sg = W.star_polylines(64, 256, W.SEED_BASE + 57)
    s = build_scene(2, v, sg)
    g = F.GPUScene2D()
    g.transfer_to_gpu(s)
    pts = W.uniform_points(30000, 2, -3, 3, 58)
    g.set_traversal(4, 32, sort_queries=True, precise=True, packet=packet)
    got = _run(g, pts)
    _, prims, _ = s.cpu_bvh.export()
    d64, _ = O.closest_points_brute_f64(2, prims, R.make_spheres(pts, R.FLT_MAX))
    rel = relative_error(got["d"], d64)
    assert rel.max() <= 1e-6, f"max relative error {rel.max():.3e}"


@pytest.mark.parametrize("leaf_size,short_stack,packet", [(8, 16, False), (12, 0, False), (6, 16, False),
                                                          (8, 16, True), (0, 0, False)])
def test_leaf_size_and_stack_placement_match_oracle(torus, leaf_size, short_stack, packet):
    s, g, pts, ref, prims = torus
    g.set_traversal(4, 16, sort_queries=True, precise=False, packet=packet, leaf_size=leaf_size,
                    short_stack=short_stack)
    got = _run(g, pts)
    compare_closest(3, prims, pts, got, ref, f"leaf {leaf_size} stack {short_stack} packet {packet}")
    assert g.check_errors() == 0
    g.set_traversal(0)


def test_warp_cooperative_results_repeat_exactly(torus):
    """Exact distance ties go to the earlier leaf position, so the packet
    kernel's answer does not depend on which queries share a warp, although
    the order inside a sort cell changes from run to run."""
    s, g, pts, ref, prims = torus
    g.set_traversal(4, 32, sort_queries=True, precise=True, packet=True)
    clustered = np.repeat(pts[:4000], 30, axis=0)  # many queries per sort cell
    first = _run(g, clustered).tobytes()
    for _ in range(3):
        assert _run(g, clustered).tobytes() == first
    g.set_traversal(0)


@pytest.mark.parametrize("precise", [False, True])
@pytest.mark.parametrize("scale", [1.0, 25.0])
def test_every_wide_layout_and_schedule_agrees_exactly(torus, precise, scale):
    """The winner (and in precise mode the runner-up) is the first primitive
    in leaf order among those at the smallest distance, which every layout
    and schedule visits (boxes are visited within the winner's distance plus
    the rounding band): results are byte-identical across all of them, also
    for queries far from the mesh (scale 25), where box distances round
    coarser than the box padding."""
    s, g, pts, ref, prims = torus
    sub = (pts[:40000] * np.float32(scale)).astype(np.float32)
    outs = {}
    for cfg in [dict(branching=4, bits=32, packet=True), dict(branching=4, bits=32, persistent=False),
                dict(branching=4, bits=32, persistent=True), dict(branching=2, bits=16),
                dict(branching=8, bits=8), dict(branching=4, bits=8, leaf_size=8, short_stack=0),
                dict(branching=8, bits=32, packet=True), dict(branching=4, bits=16, sort_queries=False),
                dict(branching=4, bits=32, threads_per_query=4), dict(branching=8, bits=8, threads_per_query=8),
                dict(branching=2, bits=32, threads_per_query=2), dict(branching=8, bits=16, threads_per_query=2),
                dict(branching=4, bits=8, leaf_size=12, threads_per_query=8),
                dict(branching=4, bits=32, packet=True, persistent=False),
                dict(branching=8, bits=16, packet=True, persistent=True)]:
        g.set_traversal(precise=precise, **cfg)
        outs[str(cfg)] = _run(g, sub).tobytes()
    g.set_traversal(0)
    first = next(iter(outs.values()))
    differ = [k for k, v in outs.items() if v != first]
    assert not differ, f"configurations that differ from the first: {differ}"


@pytest.mark.parametrize("lanes", [2, 4, 8])
@pytest.mark.parametrize("branching,bits", [(2, 32), (4, 16), (8, 8), (8, 32)])
def test_cooperative_lanes_match_oracle(torus, lanes, branching, bits):
    """Groups of 2, 4 or 8 lanes per query (child boxes and leaf primitives
    split over the lanes) against the reference CPU order, with and without
    the precise refinement and merged leaves."""
    s, g, pts, ref, prims = torus
    for precise, leaf in ((False, 0), (True, 0), (True, 8)):
        g.set_traversal(branching, bits, sort_queries=True, precise=precise, leaf_size=leaf, threads_per_query=lanes)
        compare_closest(3, prims, pts, _run(g, pts), ref, f"coop{lanes} {branching}/{bits} leaf {leaf}")
    g.set_traversal(0)
    assert g.check_errors() == 0


def test_cooperative_lanes_2d_and_finite_radius():
    v, sg = W.star_polylines(16, 64, W.SEED_BASE + 59)
    s = build_scene(2, v, sg)
    g = F.GPUScene2D()
    g.transfer_to_gpu(s)
    pts = W.uniform_points(30000, 2, -3, 3, 60)
    r2 = W.rng(61).uniform(0.0, 0.5, len(pts)).astype(np.float32)
    nodes, prims, _ = s.cpu_bvh.export()
    ref = O.closest_points_bvh(2, nodes, prims, R.make_spheres(pts, r2))
    for lanes in (2, 4, 8):
        g.set_traversal(4, 16, sort_queries=True, precise=True, threads_per_query=lanes)
        compare_closest(2, prims, pts, _run(g, pts, r2), ref, f"2D coop{lanes}")
    with pytest.raises(F.FcpwError):
        g.set_traversal(4, 32, packet=True, threads_per_query=4)
    with pytest.raises(F.FcpwError):
        g.set_traversal(4, 32, threads_per_query=3)
    g.set_traversal(0)
    assert g.check_errors() == 0


@pytest.mark.parametrize("dim", [3, 2])
def test_scene_file_load_matches_transfer(tmp_path, dim):
    """A scene loaded from a file (no CPU build, preloaded wide trees) answers
    exactly like the scene transferred from the host BVH, on the binary and the
    wide paths, and refits from device vertices like it."""
    import torch
    if dim == 3:
        v, f = W.torus(96, 48, W.SEED_BASE + 72)
        lo, hi = -2.0, 2.0
    else:
        v, f = W.star_polylines(16, 64, W.SEED_BASE + 73)
        lo, hi = -3.0, 3.0
    s = build_scene(dim, v, f, silhouettes=True)
    path = tmp_path / "scene.fcpwgb"
    s.cpu_bvh.save(path, wide=[(4, 32), (4, 8, 8)])
    a = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    b = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    a.transfer_to_gpu(s)
    b.load(path)
    pts = W.uniform_points(30000, dim, lo, hi, 74)
    for cfg in [dict(branching=0), dict(branching=4, bits=32, packet=True), dict(branching=4, bits=8, leaf_size=8),
                dict(branching=8, bits=16)]:
        a.set_traversal(**cfg)
        b.set_traversal(**cfg)
        ra, rb = _run(a, pts), _run(b, pts)
        assert ra.tobytes() == rb.tobytes(), cfg
    assert np.array_equal(a.export_nodes().tobytes(), b.export_nodes().tobytes())
    flip = np.zeros(len(pts), np.uint32)
    sa, sb = F.GPUInteractionList(), F.GPUInteractionList()
    a.find_closest_silhouette_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), flip, sa)
    b.find_closest_silhouette_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), flip, sb)
    assert sa.array().tobytes() == sb.array().tobytes()
    moved = torch.from_numpy((v * 1.01).astype(np.float32)).cuda()
    a.update_vertices_tensor(moved)
    b.update_vertices_tensor(moved)
    torch.cuda.synchronize()
    assert np.array_equal(a.export_nodes().tobytes(), b.export_nodes().tobytes())
