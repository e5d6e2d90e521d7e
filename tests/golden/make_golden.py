"""Generates the golden fixtures in this directory from the REFERENCE ITSELF.

Run where the reference checkout exists (default /root/reference, override with
FCPW_REFERENCE_ROOT):

    python tests/golden/make_golden.py

Each fixture holds a small seeded scene, the reference's flattened BVH
(reference Scene<DIM>::build with vectorize=false, read in the GPU interop
layouts) and the reference CPU query results on seeded queries: closest points
(infinite and finite radius, with normals), rays (first hit and occlusion),
closest silhouette points, sphere sampling and a refit after moving the
vertices. The reference is compiled from its own headers against the Eigen API
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
from oracle.reference import RefScene, available  # noqa: E402

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


def main():
    if not available():
        raise SystemExit("the reference checkout is required to regenerate the golden fixtures")
    v, f = W.perturbed_sphere(8, SEED)
    make("sphere3d_sah", 3, v, f, 3, False, (-1.5, 1.5))
    make("sphere3d_overlap_sah", 3, v, f, 2, False, (-1.5, 1.5))
    vt, ft = W.torus(32, 16, SEED + 10)
    make("torus3d_snch", 3, vt, ft, 3, True, (-2.0, 2.0))
    vs, sg = W.star_polylines(9, 32, SEED + 11)
    make("stars2d_snch", 2, vs, sg, 3, True, (-3.0, 3.0))
    make("stars2d_bvh", 2, vs, sg, 1, False, (-3.0, 3.0))


if __name__ == "__main__":
    main()
