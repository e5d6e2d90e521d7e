"""CPU-only checks: the host BVH producer's structural invariants, the oracle's
internal consistency (BVH traversal == Baseline brute force, FP32 vs FP64), and
the C ABI library's exported symbols."""
import re
from pathlib import Path

import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import build_scene, compare_closest, distance_tolerance
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent


def _check_tree(nodes, prims, dim):
    n = len(nodes)
    covered = np.zeros(len(prims), np.int32)
    stack = [(0, 0)]
    seen = 0
    max_depth = 0
    eps = np.float32(np.finfo(np.float32).eps)
    while stack:
        i, depth = stack.pop()
        seen += 1
        max_depth = max(max_depth, depth)
        nd = nodes[i]
        if nd["nPrimitives"] > 0:
            lo, hi = int(nd["offset"]), int(nd["offset"] + nd["nPrimitives"])
            covered[lo:hi] += 1
            pts = [prims["pa"][lo:hi], prims["pb"][lo:hi]] + ([prims["pc"][lo:hi]] if dim == 3 else [])
            allp = np.concatenate(pts)[:, :dim]
            assert np.all(allp - eps >= nd["pMin"][:dim]) and np.all(allp + eps <= nd["pMax"][:dim])
        else:
            l, r = i + 1, i + int(nd["offset"])
            assert r < n
            for c in (l, r):
                assert np.all(nodes[c]["pMin"] >= nd["pMin"]) and np.all(nodes[c]["pMax"] <= nd["pMax"])
            stack += [(r, depth + 1), (l, depth + 1)]
    assert seen == n
    assert np.all(covered == 1)
    return max_depth


@pytest.mark.parametrize("dim", [2, 3])
def test_builder_invariants(dim):
    if dim == 3:
        v, idx = W.perturbed_sphere(16, 101)
    else:
        v, idx = W.star_polylines(9, 40, 102)
    s = build_scene(dim, v, idx)
    nodes, prims, _ = s.cpu_bvh.export()
    depth = _check_tree(nodes, prims, dim)
    assert depth == s.cpu_bvh.info.max_depth
    assert np.all(nodes["nPrimitives"] <= 4)
    # primitives carry their original indices exactly once
    assert np.array_equal(np.sort(prims["index"]), np.arange(len(idx)))
    # leaf-order records hold the caller's geometry
    imap, pv, pidx, _ = s.cpu_bvh.topology()
    assert np.array_equal(pidx, prims["index"])
    assert np.array_equal(pv, idx[prims["index"]])
    assert np.array_equal(prims["pa"][:, :dim], v[pv[:, 0]])


def test_builder_is_deterministic():
    v, f = W.torus(64, 32, 103)
    a = build_scene(3, v, f).cpu_bvh.export()[0]
    b = build_scene(3, v, f).cpu_bvh.export()[0]
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("agg", [F.AggregateType.Bvh_LongestAxisCenter, F.AggregateType.Bvh_OverlapSurfaceArea,
                                 F.AggregateType.Bvh_SurfaceArea, F.AggregateType.Bvh_Volume,
                                 F.AggregateType.Bvh_OverlapVolume])
def test_all_heuristics_build_valid_trees(agg):
    v, f = W.perturbed_sphere(8, 104)
    s = build_scene(3, v, f, aggregate=agg)
    nodes, prims, _ = s.cpu_bvh.export()
    _check_tree(nodes, prims, 3)


def test_builder_rejects_bad_input():
    with pytest.raises(F.FcpwError):
        F.CpuBvh(3, np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.int32), 3, False)
    with pytest.raises(F.FcpwError):
        F.CpuBvh(3, np.zeros((3, 3), np.float32), np.zeros((0, 3), np.int32), 3, False)
    with pytest.raises(F.FcpwError):
        F.CpuBvh(3, np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.int32), 0, False)  # Baseline
    bad = np.zeros((3, 3), np.float32)
    bad[0, 0] = np.nan
    with pytest.raises(F.FcpwError):
        F.CpuBvh(3, bad, np.array([[0, 1, 2]], np.int32), 3, False)


def test_snch_silhouette_references():
    v, f = W.perturbed_sphere(8, 105)
    s = build_scene(3, v, f, silhouettes=True)
    nodes, prims, sils = s.cpu_bvh.export()
    assert nodes.dtype == R.SNCH_NODE and len(sils) > 0
    # every leaf lists each edge of its triangles once; edges of a closed mesh have two faces
    leaves = nodes[nodes["nPrimitives"] > 0]
    assert leaves["nSilhouettes"].sum() == len(sils)
    assert np.all(sils["hasOneAdjacentFace"] == 0)
    assert np.allclose(np.linalg.norm(sils["n0"], axis=1), 1, atol=1e-5)
    # cones bound every silhouette face normal below them (checked at the leaves)
    for nd in leaves[:200]:
        if nd["halfAngle"] >= np.pi / 2:
            continue
        e = sils[nd["silhouetteOffset"]: nd["silhouetteOffset"] + nd["nSilhouettes"]]
        for n in (e["n0"], e["n1"]):
            ang = np.arccos(np.clip(n @ nd["axis"], -1, 1))
            assert np.all(ang <= nd["halfAngle"] + 1e-5)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_bvh_equals_brute_force(dim):
    if dim == 3:
        v, idx = W.perturbed_sphere(16, 106)
        pts = W.uniform_points(3000, 3, -1.5, 1.5, 107)
    else:
        v, idx = W.star_polylines(16, 64, 108)
        pts = W.uniform_points(3000, 2, -3, 3, 109)
    s = build_scene(dim, v, idx)
    nodes, prims, _ = s.cpu_bvh.export()
    sp = R.make_spheres(pts, R.FLT_MAX)
    a = O.closest_points_bvh(dim, nodes, prims, sp)
    b = O.closest_points_brute(dim, prims, sp)
    # both are exact FP32 minima over the same primitive tests: identical distances
    assert np.array_equal(a["d"], b["d"])
    compare_closest(dim, prims, pts, a, b, "oracle bvh vs brute")
    d64, _ = O.closest_points_brute_f64(dim, prims, sp)
    assert np.all(np.abs(a["d"] - d64) <= distance_tolerance(pts, a["p"][:, :dim], d64))


def test_oracle_rays_agree_with_fp64():
    v, f = W.torus(64, 32, 110)
    s = build_scene(3, v, f)
    nodes, prims, _ = s.cpu_bvh.export()
    n = 3000
    rays = R.make_rays(W.uniform_points(n, 3, -2, 2, 111), W.uniform_directions(n, 3, 112), R.FLT_MAX)
    out, hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    t64, _ = O.intersect_rays_brute_f64(3, prims, rays)
    assert (np.isfinite(t64) != hit).sum() <= 2
    both = hit & np.isfinite(t64)
    assert np.all(np.abs(out["d"][both] - t64[both]) <= 1e-5 * np.maximum(t64[both], 1))


def test_oracle_refit_is_identity_without_motion():
    v, f = W.perturbed_sphere(8, 113)
    s = build_scene(3, v, f)
    nodes, prims, _ = s.cpu_bvh.export()
    again = O.refit(3, nodes, prims)
    assert again.tobytes() == nodes.tobytes()


def test_record_layouts_match():
    assert O.record_sizes() == [32, 60, 40, 28, 44, 56, 16, 40, 40]


def test_c_abi_exports_every_declared_symbol():
    import ctypes
    header = (ROOT / "include" / "fcpw_gb300.h").read_text()
    declared = sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(fcpwgb_[a-z0-9_]+)\s*\(", header, re.M)))
    assert len(declared) >= 20
    lib = ctypes.CDLL(str(F.library_path()))
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, f"symbols declared but not exported: {missing}"
    from fcpw_gb300._lib import SIGNATURES
    assert set(SIGNATURES) == set(declared)


def test_library_reports_no_device_without_gpu():
    from fcpw_gb300._lib import lib
    assert lib().fcpwgb_device_count() >= 0
    assert b"sm_103a" in lib().fcpwgb_version()
