"""The sequential model of the device linear-BVH build (oracle.lbvh_build):
a valid tree in the interop layout whose queries agree with brute force. The
GPU tests hold the device build to this model byte for byte."""
import numpy as np
import pytest

from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import compare_closest
from oracle import oracle as O


def check_tree(dim, pos, idx, nodes, prims, pv, max_leaf):
    n = len(idx)
    assert len(nodes) >= 1 and len(nodes) <= 2 * n - 1
    # primitives: a permutation of the input, vertices copied
    assert sorted(prims["index"].tolist()) == list(range(n))
    assert np.array_equal(pv, idx[prims["index"]])
    corners = ("pa", "pb", "pc")[:dim]
    for j, c in enumerate(corners):
        assert np.array_equal(prims[c][:, :dim], pos[pv[:, j]])
    # pre-order: every primitive in exactly one leaf, leaves <= max_leaf, boxes nest
    covered = np.zeros(n, np.int32)
    stack = [(0, None)]
    seen = 0
    while stack:
        i, parent = stack.pop()
        seen += 1
        nd = nodes[i]
        if parent is not None:
            pn = nodes[parent]
            assert np.all(pn["pMin"] <= nd["pMin"]) and np.all(pn["pMax"] >= nd["pMax"])
        if nd["nPrimitives"] > 0:
            k0, k1 = int(nd["offset"]), int(nd["offset"] + nd["nPrimitives"])
            assert nd["nPrimitives"] <= max_leaf
            covered[k0:k1] += 1
            for c in corners:
                v = prims[c][k0:k1, :dim]
                assert np.all(nd["pMin"][:dim] <= v) and np.all(nd["pMax"][:dim] >= v)
        else:
            stack.append((i + int(nd["offset"]), i))
            stack.append((i + 1, i))
    assert seen == len(nodes)
    assert np.all(covered == 1)


@pytest.mark.parametrize("max_leaf", [1, 4, 15])
def test_model_tree_is_valid_3d(max_leaf):
    v, f = W.torus(48, 24, W.SEED_BASE + 90)
    nodes, prims, pv = O.lbvh_build(3, v, f, max_leaf)
    check_tree(3, v, f, nodes, prims, pv, max_leaf)


def test_model_tree_is_valid_2d():
    v, f = W.star_polylines(8, 48, W.SEED_BASE + 91)
    nodes, prims, pv = O.lbvh_build(2, v, f, 4)
    check_tree(2, v, f, nodes, prims, pv, 4)


def test_model_degenerate_inputs():
    # one primitive; fewer primitives than a leaf holds; every centroid equal
    v, f = W.torus(8, 4, W.SEED_BASE + 92)
    for n in (1, 2, 3, 4):
        nodes, prims, pv = O.lbvh_build(3, v, f[:n], 4)
        assert len(nodes) == 1 and nodes[0]["nPrimitives"] == n
        check_tree(3, v, f[:n], nodes, prims, pv, 4)
    same = np.repeat(f[:1], 300, axis=0)
    nodes, prims, pv = O.lbvh_build(3, v, same, 2)
    check_tree(3, v, same, nodes, prims, pv, 2)
    # equal codes order by primitive index: leaves list primitives in input order
    assert np.array_equal(prims["index"], np.arange(300))


def test_model_queries_match_brute_force():
    v, f = W.torus(64, 32, W.SEED_BASE + 93)
    nodes, prims, _ = O.lbvh_build(3, v, f, 4)
    pts = W.uniform_points(4000, 3, -2, 2, 94)
    sph = R.make_spheres(pts, R.FLT_MAX)
    got = O.closest_points_bvh(3, nodes, prims, sph)
    ref = O.closest_points_brute(3, prims, sph)
    compare_closest(3, prims, pts, got, ref, "model tree vs brute force")
