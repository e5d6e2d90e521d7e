"""Scenes of several objects and instances on the GPU: closest points and
rays through the C ABI against the reference's own answers
(tests/golden/instanced*.npz) and, on a larger seeded scene, against the
oracle's restatement of the reference's instanced traversal; the regular and
the _instanced entry points agree; single-tree operations refuse such a
scene."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import compare_rays, distance_tolerance, ray_prim_f64, _prim_vertices
from oracle import oracle as O
from test_cpu_instanced import NAMES, SIL_NAMES, load, oracle_inputs, scene_of

pytestmark = pytest.mark.gpu


def world_prims(s):
    """Per instance, its object's primitives mapped to world space (FP64 map, FP32 records)."""
    inst = s.instances
    _, _, mats = inst.export()
    dim = s.DIM
    out = []
    for i, k in enumerate(inst.instance_objects):
        v = s.positions(int(k)).astype(np.float64)
        f = s.indices(int(k))
        if inst.transformed[i]:
            t = mats[i, :12].reshape(3, 4).astype(np.float64)
            v = v @ t[:dim, :dim].T + t[:dim, 3]
        v = v.astype(np.float32)
        p = np.zeros(len(f), R.TRIANGLE if dim == 3 else R.LINE_SEGMENT)
        for j, c in enumerate(("pa", "pb", "pc")[:dim]):
            p[c][:, :dim] = v[f[:, j]]
        p["index"] = np.arange(len(f))
        out.append(p)
    return out


def compare_instanced(s, pts, got, got_inst, ref, ref_obj, what):
    """Found flags equal, distances within the parity tolerance of helpers.py,
    and (object, primitive) equal unless tied in FP64: the reference reports
    the object only, so its candidate's FP64 distance is the minimum over
    that object's instances."""
    dim = s.DIM
    inst = s.instances
    fg = got_inst != R.UINT_MAX
    fr = np.asarray(ref_obj) >= 0
    assert np.array_equal(fg, fr), f"{what}: found/not-found differs for {np.count_nonzero(fg != fr)} queries"
    m = np.nonzero(fr)[0]
    tol = distance_tolerance(pts[m], ref["p"][m][:, :dim], ref["d"][m])
    dd = np.abs(got["d"][m].astype(np.float64) - ref["d"][m].astype(np.float64))
    assert (dd <= tol).all(), f"{what}: worst |dd| {dd.max():.3e}"
    gobj = inst.instance_objects[got_inst[m]].astype(np.int64)
    mism = (gobj != ref_obj[m]) | (got["index"][m] != ref["index"][m])
    if mism.any():
        wp = world_prims(s)
        for j in np.nonzero(mism)[0]:
            q = m[j]
            x = pts[q:q + 1]
            dg = O.prim_distance_f64(dim, wp[got_inst[q]], [got["index"][q]], x)[0]
            dr = min(O.prim_distance_f64(dim, wp[i], [ref["index"][q]], x)[0]
                     for i in np.nonzero(inst.instance_objects == ref_obj[q])[0])
            assert abs(dg - dr) <= 2 * tol[j], f"{what}: query {q} is not a tie"
    return int(mism.sum())


def gpu_of(s, **cfg):
    g = F.GPUScene3D() if s.DIM == 3 else F.GPUScene2D()
    if cfg:
        g.set_traversal(**cfg)
    g.transfer_to_gpu(s)
    return g


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("bits", [32, 8])
def test_closest_points_match_reference(name, bits):
    gd = load(name)
    s = scene_of(gd)
    g = gpu_of(s, branching=4, bits=bits)
    pts = gd["cp_points"]
    for r2, key, normals in ((R.FLT_MAX, "cp", True), (gd["cpr_r2"], "cpr", False)):
        out = F.GPUInteractionList()
        which = g.find_closest_points_instanced(pts, np.broadcast_to(np.float32(r2), (len(pts),)).copy(), out,
                                                normals)
        got = out.array()
        ref = gd[f"{key}_out"]
        compare_instanced(s, pts, got, which, ref, gd[f"{key}_object"], f"{name} {key} bits {bits}")
        if normals:
            same = (got["index"] == ref["index"]) & (which != R.UINT_MAX)
            assert np.allclose(got["n"][same], ref["n"][same], atol=1e-5)
    assert g.check_errors() == 0


@pytest.mark.parametrize("name", NAMES)
def test_rays_match_reference(name):
    gd = load(name)
    s = scene_of(gd)
    g = gpu_of(s, branching=4, bits=32)
    o, d = gd["ray_o"], gd["ray_d"]
    tmax = np.full(len(o), R.FLT_MAX, np.float32)
    out = F.GPUInteractionList()
    which = g.intersect_rays_instanced(o, d, tmax, out)
    got = out.array()
    rays = R.make_rays(o, d, tmax)
    compare_rays_instanced(s, rays, got, which, gd["ray_out"], gd["ray_hit"], gd["ray_object"], f"{name} rays")
    out2 = F.GPUInteractionList()
    occ_which = g.intersect_rays_instanced(o, d, tmax, out2, True)
    compare_rays_instanced(s, rays, out2.array(), occ_which, None, gd["occ_hit"], None, f"{name} occlusion",
                           occl=True)


def compare_rays_instanced(s, rays, got, which, ref, ref_hit, ref_obj, what, occl=False):
    """The tie-aware ray parity of helpers.compare_rays over the scene's
    world-space primitives (every instance's primitives mapped to world space,
    concatenated): a GPU answer names its instance, a reference answer its
    object, whose instance is taken as the one whose FP64 hit parameter of
    that primitive lies nearest the reference's distance. Distances carry the
    FP32 rounding floor of the transforms."""
    dim = s.DIM
    wp = world_prims(s)
    offs = np.concatenate([[0], np.cumsum([len(p) for p in wp])]).astype(np.int64)
    allp = np.concatenate(wp)
    allp["index"] = np.arange(len(allp))
    g = got.copy()
    hit = which != R.UINT_MAX
    g["index"] = np.where(hit, offs[np.where(hit, which, 0)] + got["index"], R.UINT_MAX).astype(np.uint32)
    r = None
    if ref is not None:
        r = ref.copy()
        rf = rays.view(np.float32).reshape(len(rays), 10).astype(np.float64)
        inst_obj = s.instances.instance_objects
        for q in np.nonzero(np.asarray(ref_hit, bool))[0]:
            cands = np.nonzero(inst_obj == ref_obj[q])[0]
            pos = offs[cands] + int(ref["index"][q])
            t, _, _, _ = ray_prim_f64(dim, _prim_vertices(dim, allp, pos), np.repeat(rf[q:q + 1, 0:3], len(pos), 0),
                                      np.repeat(rf[q:q + 1, 3:6], len(pos), 0))
            r["index"][q] = pos[np.nanargmin(np.abs(t - float(ref["d"][q])))]
    return compare_rays(dim, allp, rays, g, r, ref_hit, occl=occl, floor=True, what=what)


def random_affines(n, rng, spread=6.0):
    out = []
    for _ in range(n):
        a = rng.normal(size=3)
        a /= np.linalg.norm(a)
        ang = rng.uniform(0, 2 * np.pi)
        k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        rot = np.eye(3) * np.cos(ang) + np.sin(ang) * k + (1 - np.cos(ang)) * np.outer(a, a)
        m = np.eye(4)
        m[:3, :3] = rot * rng.uniform(0.2, 0.9)
        m[:3, 3] = rng.uniform(-spread, spread, 3)
        out.append(m.astype(np.float32))
    return out


@pytest.fixture(scope="module")
def many_instances():
    rng = np.random.default_rng(2024)
    v0, f0 = W.torus(96, 48, W.SEED_BASE + 110)
    v1, f1 = W.perturbed_sphere(12, W.SEED_BASE + 111)
    s = F.Scene3D()
    s.set_object_count(3)
    objs = [(v0, f0), (v1, f1), ((v1 * 0.5 + 3.0).astype(np.float32), f1)]
    for k, (v, f) in enumerate(objs):
        s.set_object_vertices(v, k)
        s.set_object_triangles(f, k)
    s.set_object_instance_transforms(random_affines(40, rng), 0)
    s.set_object_instance_transforms(random_affines(25, rng), 1)
    s.build(F.AggregateType.Bvh_SurfaceArea, False)
    pts = W.uniform_points(60000, 3, -7, 7, 112)
    inst, tn, tr, mats, ob = oracle_inputs(s)
    ref, ref_inst = O.instanced_closest_points(3, tn, tr, mats, inst.instance_objects, inst.transformed, ob,
                                               R.make_spheres(pts, R.FLT_MAX), False)
    ref_obj = np.where(ref_inst != R.UINT_MAX,
                       inst.instance_objects[np.minimum(ref_inst, len(inst) - 1)].astype(np.int64), -1)
    return s, pts, ref, ref_obj


@pytest.mark.parametrize("cfg", [dict(bits=32), dict(bits=16, leaf_size=8), dict(bits=8, sort_queries=False)])
def test_many_instances_match_oracle(many_instances, cfg):
    s, pts, ref, ref_obj = many_instances
    g = gpu_of(s, branching=4, **cfg)
    out = F.GPUInteractionList()
    which = g.find_closest_points_instanced(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    compare_instanced(s, pts, out.array(), which, ref, ref_obj, f"66 instances {cfg}")
    assert g.check_errors() == 0


def test_entry_points_agree_and_repeat(many_instances):
    """The regular host and device entry points give the _instanced answers,
    and a second call (sorted and unsorted) repeats them byte for byte."""
    import torch
    s, pts, _, _ = many_instances
    pts = pts[:20000]
    r2 = np.full(len(pts), R.FLT_MAX, np.float32)
    g = gpu_of(s, branching=4, bits=32)
    out = F.GPUInteractionList()
    which = g.find_closest_points_instanced(pts, r2, out)
    first = out.array().tobytes()
    out2 = F.GPUInteractionList()
    assert g.find_closest_points_instanced(pts, r2, out2).tobytes() == which.tobytes()
    assert out2.array().tobytes() == first
    plain = F.GPUInteractionList()
    g.find_closest_points(pts, r2, plain)
    assert plain.array().tobytes() == first
    sph = torch.zeros((len(pts), 4), dtype=torch.float32, device="cuda")
    sph[:, :3] = torch.from_numpy(pts).cuda()
    sph[:, 3] = float(R.FLT_MAX)
    res = g.find_closest_points_tensor(sph)
    torch.cuda.synchronize()
    assert res.raw.cpu().numpy().view(R.INTERACTION).reshape(-1).tobytes() == first


def test_layouts_agree(many_instances):
    """Records of every box precision and leaf size, compared with the float
    layout: the answers are the same primitives; where records differ, the
    message says in which fields."""
    s, pts, _, _ = many_instances
    pts = pts[:20000]
    r2 = np.full(len(pts), R.FLT_MAX, np.float32)
    base = None
    report = []
    for cfg in [dict(bits=32), dict(bits=8), dict(bits=16, leaf_size=6), dict(bits=32, sort_queries=False)]:
        g = gpu_of(s, branching=4, **cfg)
        out = F.GPUInteractionList()
        which = g.find_closest_points_instanced(pts, r2, out)
        rec = out.array()
        if base is None:
            base = (rec, which)
            continue
        diff = rec.tobytes() != base[0].tobytes() or which.tobytes() != base[1].tobytes()
        if diff:
            fields = {f: int(np.count_nonzero((rec[f] != base[0][f]).reshape(len(rec), -1).any(1)))
                      for f in ("p", "n", "uv", "d", "index")}
            fields["instance"] = int(np.count_nonzero(which != base[1]))
            k = int(np.nonzero((which != base[1]) | (rec["d"] != base[0]["d"]))[0][:1].tolist()[0]) \
                if (fields["instance"] or fields["d"]) else -1
            sample = (f" first: query {k}, d {rec['d'][k]!r} vs {base[0]['d'][k]!r}, instance {which[k]} vs "
                      f"{base[1][k]}, index {rec['index'][k]} vs {base[0]['index'][k]}") if k >= 0 else ""
            report.append(f"{cfg}: {fields}{sample}")
    assert not report, "; ".join(report)


def test_single_tree_operations_refuse_instanced_scene():
    gd = load("instanced3d")
    s = scene_of(gd)
    g = gpu_of(s)
    pts = gd["cp_points"][:100]
    with pytest.raises(F.FcpwError):
        g.refit_arrays()
    # objects built without silhouettes: every silhouette result keeps its default record
    sil = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(100, R.FLT_MAX, np.float32), np.zeros(100, np.uint32), sil)
    assert (sil.array()["index"] == R.UINT_MAX).all()
    with pytest.raises(F.FcpwError):
        g.contains(pts)
    # a single-tree transfer replaces the instanced scene
    one = F.Scene3D()
    one.set_object_count(1)
    one.set_object_vertices(gd["obj0_positions"], 0)
    one.set_object_triangles(gd["obj0_indices"], 0)
    one.build(F.AggregateType.Bvh_SurfaceArea, False)
    g.transfer_to_gpu(one)
    out = F.GPUInteractionList()
    g.find_closest_points(pts, np.full(100, R.FLT_MAX, np.float32), out)
    assert (out.array()["index"] != R.UINT_MAX).all()


def _objects_of(s, which):
    inst = s.instances.instance_objects
    return np.where(which != R.UINT_MAX, inst[np.minimum(which, len(inst) - 1)].astype(np.int64), -1)


@pytest.mark.parametrize("name", NAMES + SIL_NAMES)
def test_sphere_sampling_matches_reference(name):
    """Scene::intersect(sphere, randNums) on several objects: the reference's
    stochastic top-level descent, every instance of the chosen leaf sampled
    with the current random number through its transform. The same object
    and primitive are chosen (the selection rescales one random number through
    every choice, so a last-bit difference in an area can flip a choice: at
    most 1 in 1000), and the sample's point and pdf agree."""
    gd = load(name)
    s = scene_of(gd)
    g = gpu_of(s, branching=4, bits=32)
    out = F.GPUInteractionList()
    which = g.intersect_spheres_instanced(gd["ss_c"], gd["ss_r2"], gd["ss_rand"], out)
    got, ref, hit = out.array(), gd["ss_out"], gd["ss_hit"]
    gh = which != R.UINT_MAX
    assert (gh != hit).sum() <= 1
    both = gh & hit
    assert both.sum() >= 20
    same = (got["index"][both] == ref["index"][both]) & (_objects_of(s, which)[both] == gd["ss_object"][both])
    assert same.mean() > 0.999
    assert np.allclose(got["d"][both][same], ref["d"][both][same], rtol=1e-4)
    assert np.allclose(got["p"][both][same], ref["p"][both][same], atol=1e-4)
    plain = F.GPUInteractionList()  # the regular entry point routes to the same kernel
    g.intersect(gd["ss_c"], gd["ss_r2"], gd["ss_rand"], plain)
    assert plain.array().tobytes() == got.tobytes()
    assert g.check_errors() == 0


@pytest.mark.parametrize("name", SIL_NAMES)
def test_silhouettes_match_reference(name):
    """Closest silhouette points on several objects with instance transforms:
    found flags equal, distances within the reference's own classification
    precision (1e-3, tests/aggregate_tests.cpp:610), and the object the same
    unless the two silhouette points are at the same distance."""
    gd = load(name)
    s = scene_of(gd)
    dim = s.DIM
    g = gpu_of(s, branching=4, bits=32)
    pts = gd["sil_points"]
    out = F.GPUInteractionList()
    which = g.find_closest_silhouette_points_instanced(pts, np.full(len(pts), R.FLT_MAX, np.float32),
                                                       gd["sil_flip"], out)
    got, ref = out.array(), gd["sil_out"]
    fg, fr = which != R.UINT_MAX, gd["sil_object"] >= 0
    assert (fg != fr).sum() <= 1
    both = fg & fr
    tol = distance_tolerance(pts[both], ref["p"][both][:, :dim], ref["d"][both])
    dd = np.abs(got["d"][both].astype(np.float64) - ref["d"][both])
    assert np.all(dd <= 1e-3 * ref["d"][both] + tol)
    obj_diff = _objects_of(s, which)[both] != gd["sil_object"][both]
    assert np.all(dd[obj_diff] <= 1e-3 * ref["d"][both][obj_diff] + tol[obj_diff])
    plain = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), gd["sil_flip"], plain)
    assert plain.array().tobytes() == got.tobytes()
    assert g.check_errors() == 0


@pytest.mark.parametrize("name", NAMES + SIL_NAMES)
@pytest.mark.parametrize("device_update", [False, True])
def test_object_refit_matches_reference(name, device_update):
    """After the first object's vertices move, refitting that object (from its
    records, or from device vertex positions) and the top level gives the
    reference's refit top-level boxes bit for bit and its closest points."""
    import torch
    gd = load(name)
    s = scene_of(gd)
    g = gpu_of(s, branching=4, bits=32)
    moved = gd["refit_positions"]
    if device_update:
        g.update_object_vertices_tensor(0, torch.from_numpy(moved).cuda())
        torch.cuda.synchronize()
    else:
        s.update_object_vertices(moved, 0)
        g.refit(s)
    top = g.export_top_nodes()
    assert top.tobytes() == gd["refit_top_nodes"].tobytes()
    pts = gd["cp_points"]
    out = F.GPUInteractionList()
    which = g.find_closest_points_instanced(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    moved_scene = scene_of(dict(gd, obj0_positions=moved))
    compare_instanced(moved_scene, pts, out.array(), which, gd["refit_cp_out"], gd["refit_cp_object"],
                      f"{name} after refit")
    assert g.check_errors() == 0
