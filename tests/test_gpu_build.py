"""GPU BVH construction (fcpwgb_gpu_scene_build): the device-built tree equals
the sequential model of the build byte for byte (and so does its refit),
queries on it agree with the oracle's traversal of that tree (the parity
tolerances of helpers.py) and with FP64 brute force on every fast path, and
bad input is refused before any vertex is read."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import compare_closest, compare_rays, relative_error
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _run(g, pts, r2=None):
    out = F.GPUInteractionList()
    r2 = np.full(len(pts), R.FLT_MAX, np.float32) if r2 is None else r2
    g.find_closest_points(pts, r2, out)
    return out.array()


def _scene(dim):
    return F.GPUScene3D() if dim == 3 else F.GPUScene2D()


@pytest.mark.parametrize("dim,max_leaf", [(3, 4), (3, 1), (3, 15), (2, 4)])
def test_device_tree_equals_model(dim, max_leaf):
    if dim == 3:
        v, f = W.torus(192, 96, W.SEED_BASE + 95)
    else:
        v, f = W.star_polylines(24, 96, W.SEED_BASE + 96)
    nodes, prims, pv = O.lbvh_build(dim, v, f, max_leaf)
    g = _scene(dim)
    g.build_on_gpu(v, f, max_leaf)
    info = g.info()
    assert info["n_nodes"] == len(nodes) and info["n_primitives"] == len(f)
    assert g.export_nodes().tobytes() == nodes.tobytes()
    # the reference-order binary traversal of the same tree agrees with the oracle's
    lo, hi = (-2.0, 2.0) if dim == 3 else (-3.0, 3.0)
    pts = W.uniform_points(20000, dim, lo, hi, 97)
    g.set_traversal(0)
    got = _run(g, pts)
    ref = O.closest_points_bvh(dim, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    compare_closest(dim, prims, pts, got, ref, f"device-built tree, leaf {max_leaf}")
    assert g.check_errors() == 0


def test_host_and_device_entries_agree_and_repeat():
    import torch
    v, f = W.torus(128, 64, W.SEED_BASE + 98)
    a, b, c = F.GPUScene3D(), F.GPUScene3D(), F.GPUScene3D()
    a.build_on_gpu(v, f)
    b.build_on_gpu(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda())
    c.build_on_gpu(v, f)
    na = a.export_nodes().tobytes()
    assert na == b.export_nodes().tobytes() == c.export_nodes().tobytes()


@pytest.mark.parametrize("cfg", [dict(branching=4, bits=32, packet=True), dict(branching=4, bits=8, leaf_size=8),
                                 dict(branching=8, bits=16), dict(branching=2, bits=32, persistent=False)])
def test_fast_paths_on_device_tree(cfg):
    v, f = W.torus(256, 128, W.SEED_BASE + 99)
    g = F.GPUScene3D()
    g.build_on_gpu(v, f)
    pts = W.uniform_points(60000, 3, -2, 2, 100)
    g.set_traversal(**cfg)
    got = _run(g, pts)
    nodes, prims, _ = O.lbvh_build(3, v, f, 4)
    ref = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
    compare_closest(3, prims, pts, got, ref, f"device-built tree {cfg}")
    d64, _ = O.closest_points_brute_f64(3, prims, R.make_spheres(pts, R.FLT_MAX))
    assert relative_error(got["d"], d64).max() <= 1e-6
    assert g.check_errors() == 0


def test_same_distances_as_the_host_sah_tree():
    from helpers import build_scene
    v, f = W.torus(128, 64, W.SEED_BASE + 101)
    s = build_scene(3, v, f)
    host, dev = F.GPUScene3D(), F.GPUScene3D()
    host.transfer_to_gpu(s)
    dev.build_on_gpu(v, f)
    pts = W.uniform_points(30000, 3, -2, 2, 102)
    a, b = _run(host, pts), _run(dev, pts)
    _, prims, _ = s.cpu_bvh.export()
    compare_closest(3, prims, pts, b, a, "device-built vs host SAH tree")


def test_rays_and_refit_on_device_tree():
    import torch
    v, f = W.torus(96, 48, W.SEED_BASE + 103)
    g = F.GPUScene3D()
    g.build_on_gpu(v, f)
    rng = np.random.default_rng(104)
    o = rng.uniform(-2, 2, (5000, 3)).astype(np.float32)
    d = W.uniform_directions(5000, 3, 105)
    out = F.GPUInteractionList()
    g.intersect(o, d, np.full(5000, R.FLT_MAX, np.float32), out, False)
    nodes, prims, _ = O.lbvh_build(3, v, f, 4)
    rays = R.make_rays(o, d, np.full(5000, R.FLT_MAX, np.float32))
    ref, hit = O.intersect_rays_bvh(3, nodes, prims, rays)
    compare_rays(3, prims, rays, out.array(), ref, hit)
    # moved vertices: the device refit of the built tree equals the oracle's
    # refit of the model tree over the moved primitives, and so do the queries
    moved = (v * 1.05).astype(np.float32)
    g.update_vertices_tensor(torch.from_numpy(moved).cuda())
    _, _, pv = O.lbvh_build(3, v, f, 4)
    pm = prims.copy()
    pm["pa"], pm["pb"], pm["pc"] = moved[pv[:, 0]], moved[pv[:, 1]], moved[pv[:, 2]]
    nm = O.refit(3, nodes, pm)
    assert g.export_nodes().tobytes() == nm.tobytes()
    pts = W.uniform_points(8000, 3, -2, 2, 106)
    ref = O.closest_points_bvh(3, nm, pm, R.make_spheres(pts, R.FLT_MAX))
    compare_closest(3, pm, pts, _run(g, pts), ref, "refit device-built tree")


def test_small_and_degenerate_inputs():
    v, f = W.torus(8, 4, W.SEED_BASE + 107)
    pts = W.uniform_points(512, 3, -2, 2, 108)
    for sub in (f[:1], f[:2], f[:4], f[:5], np.repeat(f[:1], 700, axis=0)):
        nodes, prims, _ = O.lbvh_build(3, v, sub, 4)
        g = F.GPUScene3D()
        g.build_on_gpu(v, sub)
        assert g.export_nodes().tobytes() == nodes.tobytes()
        g.set_traversal(0)
        ref = O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts, R.FLT_MAX))
        compare_closest(3, prims, pts, _run(g, pts), ref, f"{len(sub)} primitives")


def test_bad_input_is_refused():
    import torch
    v, f = W.torus(8, 4, W.SEED_BASE + 109)
    bad = f.copy()
    bad[3, 1] = len(v)
    g = F.GPUScene3D()
    with pytest.raises(F.FcpwError):
        g.build_on_gpu(v, bad)
    with pytest.raises(F.FcpwError):
        g.build_on_gpu(torch.from_numpy(v).cuda(), torch.from_numpy(bad).cuda())
    neg = f.copy()
    neg[0, 0] = -1
    with pytest.raises(F.FcpwError):
        g.build_on_gpu(torch.from_numpy(v).cuda(), torch.from_numpy(neg).cuda())
    with pytest.raises(F.FcpwError):
        g.build_on_gpu(v, f, max_leaf_size=16)
    # the scene stays usable after a refused build
    g.build_on_gpu(v, f)
    assert g.info()["n_primitives"] == len(f)


# ------------------------------------------------------------- the reference's SAH tree on the device
@pytest.mark.parametrize("dim,aggregate,size", [(3, 3, "large"), (3, 3, "small"), (3, 2, "large"), (3, 5, "large"),
                                                (3, 1, "large"), (3, 4, "large"), (2, 3, "large")])
def test_device_sah_tree_equals_host_build(dim, aggregate, size):
    """fcpwgb_gpu_scene_build_sah builds the host builder's tree (which is the
    reference's, tests/test_golden_cpu.py) byte for byte: nodes and the
    primitive order, for every heuristic, with large nodes split level by
    level on the whole GPU and small subtrees by one thread each."""
    from helpers import build_scene
    if dim == 3:
        v, f = (W.torus(192, 96, W.SEED_BASE + 120) if size == "large" else W.torus(12, 8, W.SEED_BASE + 121))
    else:
        v, f = W.star_polylines(48, 128, W.SEED_BASE + 122)
    s = build_scene(dim, v, f, aggregate=aggregate)
    nodes, prims, _ = s.cpu_bvh.export()
    g = _scene(dim)
    g.build_on_gpu(v, f, method="sah", aggregate_type=aggregate)
    got = g.export_nodes()
    assert len(got) == len(nodes)
    diff = np.nonzero((got.view(np.uint8).reshape(len(got), -1) != nodes.view(np.uint8).reshape(len(nodes), -1))
                      .any(1))[0]
    assert len(diff) == 0, f"{len(diff)} nodes differ, first {diff[:3]}: {got[diff[:1]]} vs {nodes[diff[:1]]}"
    lo, hi = (-2.0, 2.0) if dim == 3 else (-3.0, 3.0)
    pts = W.uniform_points(20000, dim, lo, hi, 123)
    g.set_traversal(0)
    host = _scene(dim)
    host.transfer_to_gpu(s)
    host.set_traversal(0)
    assert _run(g, pts).tobytes() == _run(host, pts).tobytes()


def test_device_sah_tree_edge_cases():
    from helpers import build_scene
    v, f = W.torus(8, 4, W.SEED_BASE + 124)
    for sub in (f[:1], f[:5], np.repeat(f[:2], 900, axis=0), np.concatenate([f] * 20)):
        s = build_scene(3, v, sub)
        nodes, _, _ = s.cpu_bvh.export()
        g = F.GPUScene3D()
        g.build_on_gpu(v, sub, method="sah")
        assert g.export_nodes().tobytes() == nodes.tobytes(), f"{len(sub)} primitives"
    with pytest.raises(F.FcpwError):
        g.build_on_gpu(v, f, method="sah", aggregate_type=0)       # Baseline has no tree
