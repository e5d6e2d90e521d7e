"""CPU checks of the wide / quantised tree the GPU fast path traverses: every
binary leaf is reachable exactly once, and every dequantised child box (as the
kernel computes it, fmaf(q, 2^e, origin) rounded once to float32) contains
the float box of the binary node behind the slot, so pruning is never wrong."""
from fractions import Fraction

import numpy as np
import pytest

from fcpw_gb300 import wide_format as WF
from fcpw_gb300 import workloads as W
from helpers import build_scene

EMPTY = 255


def f32_round(x: Fraction) -> np.float32:
    """Correct rounding of an exact rational to float32 (ties to even)."""
    f = np.float32(float(x))
    cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
    best = min(cands, key=lambda c: (abs(Fraction(float(c)) - x), int(np.float32(c).view(np.uint32)) & 1))
    return np.float32(best)


def dequant(q: int, e: int, o: np.float32) -> np.float32:
    return f32_round(Fraction(q) * Fraction(2) ** e + Fraction(float(o)))


@pytest.fixture(scope="module")
def scenes():
    v, f = W.perturbed_sphere(16, 301)
    vt, ft = W.torus(48, 24, 302)
    v2, s2 = W.star_polylines(9, 48, 303)
    return {3: [build_scene(3, v, f), build_scene(3, vt, ft, silhouettes=True)], 2: [build_scene(2, v2, s2)]}


@pytest.mark.parametrize("branching", [2, 4, 8])
@pytest.mark.parametrize("bits", [32, 16, 8])
def test_wide_tree_covers_leaves_and_contains_children(scenes, branching, bits):
    for dim, lst in scenes.items():
        for s in lst:
            nodes, prims, _ = s.cpu_bvh.export()
            raw, cb = s.cpu_bvh.export_wide(branching, bits)
            d = WF.decode(raw, branching, bits)
            # leaf coverage: the leaf slots list exactly the binary leaves
            leaf_slots = (d["cnt"] != 0) & (d["cnt"] != EMPTY)
            got = sorted(zip(d["refs"][leaf_slots].tolist(), d["cnt"][leaf_slots].tolist()))
            bl = nodes[nodes["nPrimitives"] > 0]
            want = sorted(zip(bl["offset"].tolist(), bl["nPrimitives"].tolist()))
            assert got == want
            # inner slots reference every wide node except the root exactly once
            inner = d["refs"][d["cnt"] == 0]
            assert sorted(inner.tolist()) == list(range(1, len(raw)))
            # child boxes
            valid = cb >= 0
            assert np.array_equal(valid, d["cnt"] != EMPTY)
            lo = np.stack([nodes["pMin"][cb.clip(0)][..., a] for a in range(3)], 1)  # (n, 3, W)
            hi = np.stack([nodes["pMax"][cb.clip(0)][..., a] for a in range(3)], 1)
            if bits == 32:
                assert np.array_equal(np.where(valid[:, None, :], d["bounds"][:, :3], 0), np.where(valid[:, None, :], lo, 0))
                assert np.array_equal(np.where(valid[:, None, :], d["bounds"][:, 3:], 0), np.where(valid[:, None, :], hi, 0))
                continue
            # exact check on a sample of nodes (the quantiser checks every node with fmaf itself)
            rng = np.random.default_rng(0)
            for i in rng.choice(len(raw), size=min(len(raw), 40), replace=False):
                for c in range(branching):
                    if not valid[i, c]:
                        continue
                    for a in range(3):
                        e, o = int(d["exponent"][i, a]), d["origin"][i, a]
                        assert dequant(int(d["q"][i, a, c]), e, o) <= lo[i, a, c]
                        assert dequant(int(d["q"][i, 3 + a, c]), e, o) >= hi[i, a, c]


def test_quantised_boxes_stay_tight(scenes):
    """8-bit boxes grow each child extent by at most about 2/255 of the parent extent."""
    s = scenes[3][0]
    nodes, _, _ = s.cpu_bvh.export()
    raw, cb = s.cpu_bvh.export_wide(4, 8)
    d = WF.decode(raw, 4, 8)
    i = 0
    valid = cb[i] >= 0
    ext = max(float(nodes["pMax"][cb[i][valid]].max() - nodes["pMin"][cb[i][valid]].min()), 1e-6)
    for c in np.nonzero(valid)[0]:
        for a in range(3):
            e, o = int(d["exponent"][i, a]), float(d["origin"][i, a])
            qlo = o + d["q"][i, a, c] * 2.0 ** e
            qhi = o + d["q"][i, 3 + a, c] * 2.0 ** e
            assert qhi - qlo <= (nodes["pMax"][cb[i, c], a] - nodes["pMin"][cb[i, c], a]) + 4 * ext / 255 + 1e-6


@pytest.mark.parametrize("leaf_size", [6, 8, 12])
@pytest.mark.parametrize("branching", [4, 8])
def test_merged_leaves_cover_every_primitive_once(scenes, branching, leaf_size):
    """leaf_size > 0 merges binary subtrees of at most leaf_size primitives into
    one wide leaf: the leaf slots still cover every primitive exactly once, no
    leaf is larger than allowed, and each merged slot's box is the box of the
    binary subtree it replaces (its child_binary entry)."""
    for dim, lst in scenes.items():
        for s in lst:
            nodes, prims, _ = s.cpu_bvh.export()
            raw, cb = s.cpu_bvh.export_wide(branching, 32, leaf_size)
            d = WF.decode(raw, branching, 32)
            leaf_slots = (d["cnt"] != 0) & (d["cnt"] != EMPTY)
            refs, cnts = d["refs"][leaf_slots], d["cnt"][leaf_slots]
            assert cnts.max() <= max(leaf_size, int(nodes["nPrimitives"].max()))
            covered = np.zeros(len(prims), np.int32)
            for r, c in zip(refs.tolist(), cnts.tolist()):
                covered[r:r + c] += 1
            assert np.all(covered == 1)
            raw0, _ = s.cpu_bvh.export_wide(branching, 32, 0)
            assert len(raw) <= len(raw0)  # merging never adds records
            valid = cb >= 0
            lo = np.stack([nodes["pMin"][cb.clip(0)][..., a] for a in range(3)], 1)
            assert np.array_equal(np.where(valid[:, None, :], d["bounds"][:, :3], 0),
                                  np.where(valid[:, None, :], lo, 0))
