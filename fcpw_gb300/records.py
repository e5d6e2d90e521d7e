"""numpy dtypes of the interop records (byte-identical to include/fcpw_gb300.h and
to the reference's include/fcpw/gpu/bvh_interop_structures.h)."""
import numpy as np

f3 = ("<f4", (3,))

SPHERE = np.dtype([("c", *f3), ("r2", "<f4")])
RAY = np.dtype([("o", *f3), ("d", *f3), ("dInv", *f3), ("tMax", "<f4")])
INTERACTION = np.dtype([("p", *f3), ("n", *f3), ("uv", "<f4", (2,)), ("d", "<f4"), ("index", "<u4")])
BVH_NODE = np.dtype([("pMin", *f3), ("pMax", *f3), ("nPrimitives", "<u4"), ("offset", "<u4")])
SNCH_NODE = np.dtype([("pMin", *f3), ("pMax", *f3), ("axis", *f3), ("halfAngle", "<f4"), ("radius", "<f4"),
                      ("nPrimitives", "<u4"), ("offset", "<u4"), ("nSilhouettes", "<u4"),
                      ("silhouetteOffset", "<u4")])
TRIANGLE = np.dtype([("pa", *f3), ("pb", *f3), ("pc", *f3), ("index", "<u4")])
LINE_SEGMENT = np.dtype([("pa", *f3), ("pb", *f3), ("index", "<u4")])
VERTEX = np.dtype([("p", *f3), ("n0", *f3), ("n1", *f3), ("index", "<u4"), ("hasOneAdjacentFace", "<u4")])
EDGE = np.dtype([("pa", *f3), ("pb", *f3), ("n0", *f3), ("n1", *f3), ("index", "<u4"),
                 ("hasOneAdjacentFace", "<u4")])

assert SPHERE.itemsize == 16 and RAY.itemsize == 40 and INTERACTION.itemsize == 40
assert BVH_NODE.itemsize == 32 and SNCH_NODE.itemsize == 60
assert TRIANGLE.itemsize == 40 and LINE_SEGMENT.itemsize == 28
assert VERTEX.itemsize == 44 and EDGE.itemsize == 56

UINT_MAX = 0xFFFFFFFF
FLT_MAX = np.float32(3.402823466e38)

# FCPW_BVH_TYPE numbering
LINE_SEGMENT_BVH, TRIANGLE_BVH, LINE_SEGMENT_SNCH, TRIANGLE_SNCH = 1, 2, 3, 4


def default_interactions(n: int) -> np.ndarray:
    out = np.zeros(n, INTERACTION)
    out["d"] = FLT_MAX
    out["index"] = UINT_MAX
    return out


def make_spheres(centers, r2) -> np.ndarray:
    centers = np.asarray(centers, np.float32)
    n = centers.shape[0]
    s = np.zeros(n, SPHERE)
    s["c"][:, : centers.shape[1]] = centers
    s["r2"] = np.broadcast_to(np.asarray(r2, np.float32), (n,))
    return s


def make_rays(origins, directions, t_max) -> np.ndarray:
    origins = np.asarray(origins, np.float32)
    directions = np.asarray(directions, np.float32)
    n = origins.shape[0]
    r = np.zeros(n, RAY)
    r["o"][:, : origins.shape[1]] = origins
    r["d"][:, : directions.shape[1]] = directions
    with np.errstate(divide="ignore"):
        r["dInv"] = np.float32(1.0) / r["d"]
    r["tMax"] = np.broadcast_to(np.asarray(t_max, np.float32), (n,))
    return r
