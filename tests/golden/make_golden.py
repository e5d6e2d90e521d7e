"""Generates the golden fixtures in this directory from the REFERENCE ITSELF.

Run where the reference headers can be staged (oracle/build.py stages them
from the reference checkout into baseline/_ref):

    python tests/golden/make_golden.py [fixture names]

Each fixture holds a small seeded scene, the reference's flattened BVH
(reference Scene<DIM>::build with vectorize=false, read in the GPU interop
layouts) and the reference CPU query results on seeded queries: closest points
(infinite and finite radius, with normals), rays (first hit and occlusion),
closest silhouette points, sphere sampling and a refit after moving the
vertices; the instanced fixtures hold scenes of several objects with
instance transforms, the reference's top-level tree and its answers with the
object of every result. The reference is compiled from its own headers against the Eigen API
shim in oracle/compat (oracle/build.py).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from fcpw_gb300 import records as R  # noqa: E402
from fcpw_gb300 import workloads as W  # noqa: E402
from oracle.reference import RefMultiScene, RefScene, available  # noqa: E402

SEED = 777


def _queries(dim, n, lo, hi, seed):
    return W.uniform_points(n, dim, lo, hi, seed)


def make(name, dim, verts, idx, aggregate, silhouettes, box, n=1500):
    lo, hi = box
    ref = RefScene(dim, verts, idx, aggregate, silhouettes)
    nodes, prims, sils, info = ref.export()
    out = {"dim": dim, "aggregate": aggregate, "silhouettes": int(silhouettes), "positions": verts, "indices": idx,
           "nodes": nodes, "prims": prims, "n_leaves": info["n_leaves"], "max_depth": info["max_depth"]}
    if sils is not None:
        out["sils"] = sils

    pts = _queries(dim, n, lo, hi, SEED + 1)
    sp = R.make_spheres(pts, R.FLT_MAX)
    res, vis = ref.closest_points(sp, visited=True)
    out.update(cp_points=pts, cp_out=res, cp_visited=vis)

    ext = float(np.linalg.norm(np.asarray(hi, np.float32) - np.asarray(lo, np.float32)))
    r2 = (0.1 * W.rng(SEED + 2).uniform(0, 1, n) * ext).astype(np.float32)  # tests/gpu_tests.cpp:65
    out.update(cpr_points=pts, cpr_r2=r2, cpr_out=ref.closest_points(R.make_spheres(pts, r2), record_normals=True))

    o = _queries(dim, n, lo, hi, SEED + 3)
    d = W.uniform_directions(n, dim, SEED + 4)
    rays = R.make_rays(o, d, R.FLT_MAX)
    ro, rh = ref.intersect_rays(rays)
    oo, oh = ref.intersect_rays(rays, occlusion=True)
    out.update(ray_o=o, ray_d=d, ray_out=ro, ray_hit=rh, occ_hit=oh)

    c = _queries(dim, n, lo, hi, SEED + 5)
    rr = (W.rng(SEED + 6).uniform(0.02, 0.4, n) ** 2).astype(np.float32)
    rn = W.rng(SEED + 7).uniform(0, 1, (n, 3)).astype(np.float32)
    so, sh = ref.sphere_sample(R.make_spheres(c, rr), rn)
    out.update(ss_c=c, ss_r2=rr, ss_rand=rn, ss_out=so, ss_hit=sh)

    # Scene::contains / hasLineOfSight (CPU-only in the reference; batched on the GPU here)
    b = _queries(dim, n, lo, hi, SEED + 12)
    out.update(in_points=pts, in_out=ref.contains(pts), los_a=pts, los_b=b, los_out=ref.line_of_sight(pts, b))

    if silhouettes:
        flip = (W.rng(SEED + 8).uniform(0, 1, n) < 0.5).astype(np.uint32)
        out.update(sil_points=pts, sil_flip=flip,
                   sil_out=ref.silhouettes_query(sp, flip, 0.0, 1e-3))

    moved = (verts + 0.01 * W.rng(SEED + 9).standard_normal(verts.shape)).astype(np.float32)
    ref.update_and_refit(moved)
    rnodes, rprims, rsils, _ = ref.export()
    out.update(refit_positions=moved, refit_nodes=rnodes, refit_prims=rprims,
               refit_cp_out=ref.closest_points(sp))
    if rsils is not None:
        out["refit_sils"] = rsils
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: {len(nodes)} nodes, {len(prims)} primitives, {0 if sils is None else len(sils)} silhouettes")


def affine(dim, rng):
    """Seeded (dim+1)x(dim+1) affine map: a rotation, a uniform scale in
    [0.3, 1.2] and a translation in [-4, 4]^dim."""
    m = np.eye(dim + 1)
    if dim == 3:
        a = rng.normal(size=3)
        a /= np.linalg.norm(a)
        ang = rng.uniform(0, 2 * np.pi)
        k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        rot = np.eye(3) * np.cos(ang) + np.sin(ang) * k + (1 - np.cos(ang)) * np.outer(a, a)
    else:
        ang = rng.uniform(0, 2 * np.pi)
        rot = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
    m[:dim, :dim] = rot * rng.uniform(0.3, 1.2)
    m[:dim, dim] = rng.uniform(-4, 4, dim)
    return m.astype(np.float32)


def make_instanced(name, dim, objects, n_transforms, aggregate, box, seed, n=2000, silhouettes=False):
    """A scene of several objects with instance transforms (Scene::setObjectCount,
    setObjectInstanceTransforms): the reference's top-level tree (leaf
    references as instance numbers: objects in turn, an object without
    transforms one instance, an object's transforms in turn) and its answers
    with the object index of every result: closest points, rays, sphere
    samples, closest silhouette points (scenes built with silhouettes), and,
    after moving the first object's vertices (updateObjectVertices + refit),
    the refit top-level tree and closest points."""
    rng = np.random.default_rng(seed)
    transforms = [[affine(dim, rng) for _ in range(k)] for k in n_transforms]
    ref = RefMultiScene(dim, objects, transforms, aggregate, silhouettes=silhouettes)
    top_nodes, agg_refs = ref.export_top()
    agg_to_inst, inst, nxt = {}, 0, len(objects)
    for k, ts in enumerate(transforms):
        if not ts:
            agg_to_inst[k] = inst
            inst += 1
        for _ in ts:
            agg_to_inst[nxt] = inst
            nxt += 1
            inst += 1
    top_refs = np.array([agg_to_inst[int(a)] for a in agg_refs] if len(top_nodes) else [], np.uint32)
    out = {"dim": dim, "aggregate": aggregate, "n_objects": len(objects), "silhouettes": bool(silhouettes),
           "n_transforms": np.array(n_transforms, np.int32),
           "transforms": np.array([m for ts in transforms for m in ts], np.float32).reshape(-1, dim + 1, dim + 1),
           "top_nodes": top_nodes, "top_refs": top_refs}
    for k, (v, f) in enumerate(objects):
        out[f"obj{k}_positions"] = v
        out[f"obj{k}_indices"] = f
    lo, hi = box
    pts = _queries(dim, n, lo, hi, seed + 1)
    res, obj = ref.closest_points_objects(R.make_spheres(pts, R.FLT_MAX), record_normals=True)
    r2 = (W.rng(seed + 2).uniform(0, 1, n) * 0.5).astype(np.float32)
    res2, obj2 = ref.closest_points_objects(R.make_spheres(pts, r2), record_normals=False)
    o = _queries(dim, n, lo, hi, seed + 3)
    d = W.uniform_directions(n, dim, seed + 4)
    rays = R.make_rays(o, d, R.FLT_MAX)
    ro, rh, robj = ref.intersect_rays_objects(rays)
    _, oh, _ = ref.intersect_rays_objects(rays, occlusion=True)
    out.update(cp_points=pts, cp_out=res, cp_object=obj, cpr_r2=r2, cpr_out=res2, cpr_object=obj2,
               ray_o=o, ray_d=d, ray_out=ro, ray_hit=rh, ray_object=robj, occ_hit=oh)
    # sphere sampling (Scene::intersect(sphere, randNums)): radii that reach a few primitives
    ss_c = _queries(dim, n, lo, hi, seed + 5)
    ss_r2 = (W.rng(seed + 6).uniform(0.05, 1.5, n) ** 2).astype(np.float32)
    ss_rand = W.rng(seed + 7).uniform(0, 1, (n, 3)).astype(np.float32)
    ss_out, ss_hit, ss_obj = ref.sphere_sample_objects(R.make_spheres(ss_c, ss_r2), ss_rand)
    out.update(ss_c=ss_c, ss_r2=ss_r2, ss_rand=ss_rand, ss_out=ss_out, ss_hit=ss_hit, ss_object=ss_obj)
    if silhouettes:
        sil_pts = _queries(dim, n, lo, hi, seed + 8)
        sil_flip = (W.rng(seed + 9).uniform(0, 1, n) < 0.5).astype(np.uint32)
        sil_out, sil_obj = ref.silhouettes_objects(R.make_spheres(sil_pts, R.FLT_MAX), sil_flip)
        out.update(sil_points=sil_pts, sil_flip=sil_flip, sil_out=sil_out, sil_object=sil_obj)
    # refit after moving the first object (shared by all its instances)
    v0 = np.asarray(objects[0][0], np.float32)
    moved = (v0 * np.float32(1.04) + W.rng(seed + 10).normal(0, 0.01, v0.shape)).astype(np.float32)
    ref.update_object_and_refit(0, moved)
    rt_nodes, _ = ref.export_top()
    rres, robj2 = ref.closest_points_objects(R.make_spheres(pts, R.FLT_MAX), record_normals=False)
    out.update(refit_positions=moved, refit_top_nodes=rt_nodes, refit_cp_out=rres, refit_cp_object=robj2)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: {len(objects)} objects, {inst} instances, {len(top_nodes)} top-level nodes")


def main(names=()):
    if not available():
        raise SystemExit("the reference checkout is required to regenerate the golden fixtures")
    want = lambda n: not names or n in names  # noqa: E731
    v, f = W.perturbed_sphere(8, SEED)
    if want("sphere3d_sah"):
        make("sphere3d_sah", 3, v, f, 3, False, (-1.5, 1.5))
    if want("sphere3d_overlap_sah"):
        make("sphere3d_overlap_sah", 3, v, f, 2, False, (-1.5, 1.5))
    vt, ft = W.torus(32, 16, SEED + 10)
    if want("torus3d_snch"):
        make("torus3d_snch", 3, vt, ft, 3, True, (-2.0, 2.0))
    vs, sg = W.star_polylines(9, 32, SEED + 11)
    if want("stars2d_snch"):
        make("stars2d_snch", 2, vs, sg, 3, True, (-3.0, 3.0))
    if want("stars2d_bvh"):
        make("stars2d_bvh", 2, vs, sg, 1, False, (-3.0, 3.0))
    vs2, fs2 = W.torus(16, 8, SEED + 13)
    if want("instanced3d"):
        make_instanced("instanced3d", 3, [(vt, ft), (v, f), (vs2, fs2)], [13, 0, 7], 3, (-5.0, 5.0), SEED + 20)
    if want("instanced3d_single"):
        make_instanced("instanced3d_single", 3, [(vt, ft)], [1], 3, (-5.0, 5.0), SEED + 30)
    if want("multi3d_plain"):
        make_instanced("multi3d_plain", 3, [(vt, ft), (v, f)], [0, 0], 2, (-2.5, 2.5), SEED + 40)
    s0, g0 = W.star_polylines(2, 64, SEED + 14)
    s1, g1 = W.star_polylines(1, 40, SEED + 15)
    if want("instanced2d"):
        make_instanced("instanced2d", 2, [(s0, g0), (s1, g1)], [9, 6], 3, (-5.0, 5.0), SEED + 50)
    if want("instanced3d_sil"):
        make_instanced("instanced3d_sil", 3, [(vt, ft), (v, f)], [6, 0], 3, (-5.0, 5.0), SEED + 60, silhouettes=True)
    if want("instanced2d_sil"):
        make_instanced("instanced2d_sil", 2, [(s0, g0), (s1, g1)], [5, 3], 3, (-5.0, 5.0), SEED + 70,
                       silhouettes=True)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
