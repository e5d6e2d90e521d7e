"""Scenes of several objects and instances, on the CPU: the host build of the
instanced structure (one tree per object, instance transforms and inverses,
the top-level tree) equals the reference's (tests/golden/instanced*.npz,
generated from the reference's own Scene with setObjectInstanceTransforms),
and the oracle's instanced traversals reproduce the reference's answers bit
for bit on it."""
from pathlib import Path

import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ["instanced3d", "instanced3d_single", "multi3d_plain", "instanced2d"]
SIL_NAMES = ["instanced3d_sil", "instanced2d_sil"]


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def scene_of(g):
    """The fixture's scene built through the Python drop-in, instances in the reference's order."""
    dim = int(g["dim"])
    s = F.Scene3D() if dim == 3 else F.Scene2D()
    k = int(g["n_objects"])
    s.set_object_count(k)
    t = 0
    for i in range(k):
        s.set_object_vertices(g[f"obj{i}_positions"], i)
        if dim == 3:
            s.set_object_triangles(g[f"obj{i}_indices"], i)
        else:
            s.set_object_line_segments(g[f"obj{i}_indices"], i)
        n = int(g["n_transforms"][i])
        if n:
            s.set_object_instance_transforms(list(g["transforms"][t:t + n]), i)
            t += n
    if bool(g.get("silhouettes", False)):
        s.compute_silhouettes()
    s.build(int(g["aggregate"]), False)
    return s


def oracle_inputs(s):
    inst = s.instances
    top_nodes, top_refs, mats = inst.export()
    objs = [o.export()[:2] for o in inst.objects]
    return inst, top_nodes, top_refs, mats, objs


@pytest.mark.parametrize("name", NAMES + SIL_NAMES)
def test_top_level_tree_equals_reference(name):
    g = load(name)
    s = scene_of(g)
    inst, top_nodes, top_refs, mats, _ = oracle_inputs(s)
    assert len(inst) == int(sum(max(int(n), 1) for n in g["n_transforms"]))
    assert top_nodes.tobytes() == g["top_nodes"].tobytes()
    assert np.array_equal(top_refs, g["top_refs"])
    # transforms are stored as given; inverses are inverses
    dim = int(g["dim"])
    flagged = np.nonzero(inst.transformed)[0]
    for j, i in enumerate(flagged):
        t = mats[i, :12].reshape(3, 4)
        ti = mats[i, 12:].reshape(3, 4)
        full = np.eye(dim + 1)
        full[:dim, :dim + 1] = np.concatenate([t[:dim, :dim], t[:dim, 3:4]], axis=1)
        inv = np.eye(dim + 1)
        inv[:dim, :dim + 1] = np.concatenate([ti[:dim, :dim], ti[:dim, 3:4]], axis=1)
        assert np.allclose(full @ inv, np.eye(dim + 1), atol=1e-5)
        assert np.array_equal(full[:dim].astype(np.float32), g["transforms"][j][:dim])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_equals_reference_answers(name):
    g = load(name)
    dim = int(g["dim"])
    s = scene_of(g)
    inst, top_nodes, top_refs, mats, objs = oracle_inputs(s)
    pts = g["cp_points"]
    for r2, key, normals in ((R.FLT_MAX, "cp", True), (g["cpr_r2"], "cpr", False)):
        out, which = O.instanced_closest_points(dim, top_nodes, top_refs, mats, inst.instance_objects,
                                                inst.transformed, objs, R.make_spheres(pts, r2), normals)
        assert out.tobytes() == g[f"{key}_out"].tobytes()
        found = which != R.UINT_MAX
        obj = np.where(found, inst.instance_objects[np.minimum(which, len(inst) - 1)].astype(np.int64), -1)
        assert np.array_equal(obj, g[f"{key}_object"])
    rays = R.make_rays(g["ray_o"], g["ray_d"], R.FLT_MAX)
    out, hit, which = O.instanced_rays(dim, top_nodes, top_refs, mats, inst.instance_objects, inst.transformed,
                                       objs, rays)
    assert np.array_equal(hit, g["ray_hit"]) and out.tobytes() == g["ray_out"].tobytes()
    obj = np.where(hit, inst.instance_objects[np.minimum(which, len(inst) - 1)].astype(np.int64), -1)
    assert np.array_equal(obj, g["ray_object"])
    _, occ, _ = O.instanced_rays(dim, top_nodes, top_refs, mats, inst.instance_objects, inst.transformed, objs,
                                 rays, occlusion=True)
    assert np.array_equal(occ, g["occ_hit"])


def test_instance_input_is_checked():
    g = load("instanced3d")
    s = F.Scene3D()
    s.set_object_count(1)
    s.set_object_vertices(g["obj0_positions"], 0)
    s.set_object_triangles(g["obj0_indices"], 0)
    with pytest.raises(ValueError):
        s.set_object_instance_transforms([np.eye(3)], 0)          # not (DIM+1) x (DIM+1)
    s.set_object_instance_transforms([np.zeros((4, 4), np.float32)], 0)
    with pytest.raises(F.FcpwError):
        s.build(F.AggregateType.Bvh_SurfaceArea, False)           # singular transform
    s.set_object_count(1)
    s.set_object_vertices(g["obj0_positions"], 0)
    s.set_object_triangles(g["obj0_indices"], 0)
    bad = np.eye(4, dtype=np.float32)
    bad[0, 3] = np.nan
    s.set_object_instance_transforms([bad], 0)
    with pytest.raises(F.FcpwError):
        s.build(F.AggregateType.Bvh_SurfaceArea, False)           # non-finite transform
    s2 = scene_of(g)
    with pytest.raises(RuntimeError):
        s2.cpu_bvh                                                 # one tree per object instead
