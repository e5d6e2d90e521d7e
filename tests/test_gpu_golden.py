"""GPU parity against the golden fixtures made by the reference itself: the
reference's own flattened tree is uploaded through the C ABI (no host
producer involved) and the CUDA kernels' answers are compared with the
reference CPU answers stored in the fixture."""
from pathlib import Path

import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from helpers import compare_closest, compare_rays, distance_tolerance

pytestmark = pytest.mark.gpu

# single-tree fixtures (the instanced ones are covered by test_*_instanced.py)
GOLDEN = sorted(p for p in (Path(__file__).resolve().parent / "golden").glob("*.npz")
                if not p.name.startswith(("instanced", "multi")))


def bvh_type(fx):
    dim, sil = int(fx["dim"]), bool(fx["silhouettes"])
    if dim == 3:
        return R.TRIANGLE_SNCH if sil else R.TRIANGLE_BVH
    return R.LINE_SEGMENT_SNCH if sil else R.LINE_SEGMENT_BVH


@pytest.fixture(params=GOLDEN, ids=[p.stem for p in GOLDEN])
def loaded(request):
    fx = dict(np.load(request.param))
    dim = int(fx["dim"])
    g = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    g.transfer_arrays(bvh_type(fx), fx["nodes"], fx["prims"], fx.get("sils"))
    return fx, g, dim


def test_closest_points_match_reference(loaded):
    fx, g, dim = loaded
    pts = fx["cp_points"]
    out = F.GPUInteractionList()
    g.find_closest_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    compare_closest(dim, fx["prims"], pts, out.array(), fx["cp_out"], "closest point vs reference")
    out2 = F.GPUInteractionList()
    g.find_closest_points(fx["cpr_points"], fx["cpr_r2"], out2, True)
    got, ref = out2.array(), fx["cpr_out"]
    compare_closest(dim, fx["prims"], fx["cpr_points"], got, ref, "finite radius vs reference")
    same = (got["index"] == ref["index"]) & (ref["index"] != R.UINT_MAX)
    assert np.allclose(got["n"][same], ref["n"][same], atol=1e-6)


def test_rays_match_reference(loaded):
    fx, g, dim = loaded
    o, d = fx["ray_o"], fx["ray_d"]
    tmax = np.full(len(o), R.FLT_MAX, np.float32)
    rays = R.make_rays(o, d, tmax)
    out = F.GPUInteractionList()
    g.intersect(o, d, tmax, out)
    got = out.array()
    st = compare_rays(dim, fx["prims"], rays, got, fx["ray_out"], fx["ray_hit"], what="rays vs reference")
    # the reference's own arithmetic: where the primitive agrees, the record is the reference's bit for bit
    same = (got["index"] == fx["ray_out"]["index"]) & fx["ray_hit"]
    for k in ("d", "p", "n", "uv"):
        assert np.array_equal(got[k][same], fx["ray_out"][k][same]), k
    assert st["flips"] == 0
    occ = F.GPUInteractionList()
    g.intersect(o, d, tmax, occ, True)
    compare_rays(dim, fx["prims"], rays, occ.array(), None, fx["occ_hit"], occl=True, what="occlusion vs reference")


def test_sphere_sampling_matches_reference(loaded):
    fx, g, dim = loaded
    out = F.GPUInteractionList()
    g.intersect(fx["ss_c"][:, :dim], fx["ss_r2"], fx["ss_rand"], out)
    got, ref, hit = out.array(), fx["ss_out"], fx["ss_hit"]
    gh = got["index"] != R.UINT_MAX
    assert (gh != hit).sum() <= 1
    both = gh & hit
    same = got["index"][both] == ref["index"][both]
    assert same.mean() > 0.999
    assert np.allclose(got["d"][both][same], ref["d"][both][same], rtol=1e-4)


def test_silhouettes_match_reference(loaded):
    fx, g, dim = loaded
    if "sil_out" not in fx:
        pytest.skip("fixture without silhouettes")
    pts = fx["sil_points"]
    out = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), fx["sil_flip"], out)
    got, ref = out.array(), fx["sil_out"]
    fg, fr = got["index"] != R.UINT_MAX, ref["index"] != R.UINT_MAX
    assert (fg != fr).sum() <= 1
    both = fg & fr
    tol = distance_tolerance(pts[both], ref["p"][both][:, :dim], ref["d"][both])
    assert np.all(np.abs(got["d"][both] - ref["d"][both]) <= 1e-3 * ref["d"][both] + tol)


def test_refit_boxes_bit_exact_with_reference(loaded):
    fx, g, dim = loaded
    g.refit_arrays(fx["refit_prims"], fx.get("refit_sils"))
    nodes = g.export_nodes()
    ref = fx["refit_nodes"]
    assert np.array_equal(nodes["pMin"], ref["pMin"]) and np.array_equal(nodes["pMax"], ref["pMax"])
    pts = fx["cp_points"]
    out = F.GPUInteractionList()
    g.find_closest_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    compare_closest(dim, fx["refit_prims"], pts, out.array(), fx["refit_cp_out"], "closest point after refit")


def test_contains_and_line_of_sight_equal_reference(loaded):
    """Scene::contains / hasLineOfSight as GPU batches, computed with the
    reference CPU arithmetic: equal to the reference's answers."""
    fx, g, dim = loaded
    assert np.array_equal(g.contains(fx["in_points"]), fx["in_out"])
    assert np.array_equal(g.has_line_of_sight(fx["los_a"], fx["los_b"]), fx["los_out"])
    assert g.check_errors() == 0
