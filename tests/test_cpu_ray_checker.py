"""The ray parity check of helpers.compare_rays on the CPU: it accepts two
correct evaluations (the oracle's FP32 restatement of the reference against
an FP64 brute force, on random rays and on rays aimed at edges and vertices,
where grazing hits and equidistant ties are common), and it rejects mistakes
planted in the oracle's answers: a clear hit dropped, a clear hit given
another primitive's index, a distance off by 2e-6 relative, a clear occlusion
dropped."""
import numpy as np
import pytest

from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import build_scene, compare_rays, edge_aimed_rays, leaf_positions, ray_prim_f64, _prim_vertices
from oracle import oracle as O


@pytest.fixture(scope="module")
def case():
    v, f = W.torus(48, 24, W.SEED_BASE + 70)
    s = build_scene(3, v, f)
    nodes, prims, _ = s.cpu_bvh.export()
    n = 12000
    o = W.uniform_points(n, 3, -2.0, 2.0, 71)
    d = W.uniform_directions(n, 3, 72)
    m = n // 2  # half the rays aimed at edge midpoints and vertices
    d[:m] = edge_aimed_rays(v, f, o[:m], 73)
    rays = R.make_rays(o, d, np.full(n, R.FLT_MAX, np.float32))
    ref, hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    return prims, nodes, rays, ref, hit


def test_accepts_the_oracle_itself(case):
    prims, _, rays, ref, hit = case
    st = compare_rays(3, prims, rays, ref.copy(), ref, hit)
    assert st["flips"] == 0 and st["ties"] == 0 and st["grazed"] == 0


def test_accepts_fp64_brute_force(case):
    """FP64 disagrees with FP32 on grazing rays and ties; all of them must pass."""
    prims, _, rays, ref, hit = case
    t64, i64 = O.intersect_rays_brute_f64(3, prims, rays)
    got = R.default_interactions(len(rays))
    got["index"] = i64
    same = i64 == ref["index"]
    got["d"] = np.where(same, ref["d"], np.where(i64 != R.UINT_MAX, t64, R.FLT_MAX)).astype(np.float32)
    st = compare_rays(3, prims, rays, got, ref, hit)
    assert st["ties"] + st["grazed"] + st["flips"] > 100  # the edge-aimed rays do exercise the rules


def _clear_hits(prims, rays, ref, hit):
    """Rays whose reference hit is well inside its triangle (no tie, no graze)."""
    lp = leaf_positions(prims)
    rf = rays.view(np.float32).reshape(len(rays), 10).astype(np.float64)
    k = np.nonzero(hit)[0]
    _, m, _, band = ray_prim_f64(3, _prim_vertices(3, prims, lp[ref["index"][k].astype(np.int64)]), rf[k, :3],
                                 rf[k, 3:6])
    return k[m > 100 * band]


def test_rejects_a_dropped_hit(case):
    prims, _, rays, ref, hit = case
    got = ref.copy()
    q = _clear_hits(prims, rays, ref, hit)[0]
    got["index"][q] = R.UINT_MAX
    got["d"][q] = R.FLT_MAX
    with pytest.raises(AssertionError, match="not grazing"):
        compare_rays(3, prims, rays, got, ref, hit)


def test_rejects_a_wrong_index(case):
    prims, _, rays, ref, hit = case
    got = ref.copy()
    q = _clear_hits(prims, rays, ref, hit)[:5]
    got["index"][q] = (got["index"][q] + len(prims) // 2) % len(prims)
    with pytest.raises(AssertionError, match="neither ties nor grazing"):
        compare_rays(3, prims, rays, got, ref, hit)


def test_rejects_a_distance_off_by_2e6(case):
    prims, _, rays, ref, hit = case
    got = ref.copy()
    q = _clear_hits(prims, rays, ref, hit)[0]
    got["d"][q] = np.float32(ref["d"][q] * (1 + 2e-6))
    with pytest.raises(AssertionError, match="1e-6 relative"):
        compare_rays(3, prims, rays, got, ref, hit)


def test_rejects_a_dropped_occlusion(case):
    prims, nodes, rays, ref, hit = case
    occ, ohit = O.intersect_rays_bvh(3, nodes, prims, rays, occlusion=True)
    assert np.array_equal(ohit, hit)
    got = ref.copy()  # an occlusion answer that names the primitive it hit, as the GPU's do
    compare_rays(3, prims, rays, got, None, ohit, occl=True)
    q = _clear_hits(prims, rays, ref, hit)[0]
    got["index"][q] = R.UINT_MAX
    with pytest.raises(AssertionError, match="clear FP64 hit"):
        compare_rays(3, prims, rays, got, None, ohit, occl=True)
