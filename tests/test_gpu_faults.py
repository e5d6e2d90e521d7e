"""Failures injected on the host (no GPU fault, trap or hang): queries that
are not finite or have empty radii, an allocation that fails, mismatched
array sizes, and queries before a transfer. Each returns a defined result or
a status, and the scene stays usable."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from fcpw_gb300._lib import check, lib
from helpers import build_scene

pytestmark = pytest.mark.gpu

CONFIGS = [dict(branching=0), dict(branching=4, bits=8, persistent=False), dict(branching=4, bits=32, packet=True),
           dict(branching=4, bits=16, persistent=True), dict(branching=4, bits=32, packet=True, sort_queries=False)]


def bad_rows(dim, n, rng):
    """n clean queries plus a block of bad ones: NaN and infinite centres,
    NaN and negative squared radii, and an empty radius of 0."""
    pts = W.uniform_points(n, dim, -2, 2, int(rng.integers(1 << 30)))
    r2 = np.full(n, R.FLT_MAX, np.float32)
    bad = pts[:10].copy()
    bad_r2 = np.full(10, R.FLT_MAX, np.float32)
    bad[0, 0] = np.nan
    bad[1, 1] = np.inf
    bad[2, 0] = -np.inf
    bad[3] = np.nan
    bad_r2[4] = np.nan
    bad_r2[5] = -1.0
    bad[6, dim - 1] = np.nan
    bad_r2[7] = -np.inf
    bad[8, 0] = np.inf
    bad_r2[8] = 1.0
    bad_r2[9] = 0.0
    idx = np.sort(rng.choice(n + 10, 10, replace=False))
    mask = np.zeros(n + 10, bool)
    mask[idx] = True
    allp = np.empty((n + 10, dim), np.float32)
    allr = np.empty(n + 10, np.float32)
    allp[mask], allr[mask] = bad, bad_r2
    allp[~mask], allr[~mask] = pts, r2
    return allp, allr, mask


@pytest.fixture(scope="module", params=[3, 2], ids=["3d", "2d"])
def scene(request):
    dim = request.param
    if dim == 3:
        v, idx = W.torus(64, 32, W.SEED_BASE + 2)
    else:
        v, idx = W.star_polylines(32, 64, W.SEED_BASE + 3)
    s = build_scene(dim, v, idx, silhouettes=True)
    g = F.GPUScene3D() if dim == 3 else F.GPUScene2D()
    g.transfer_to_gpu(s)
    return dim, s, g


@pytest.mark.parametrize("cfg", CONFIGS)
def test_non_finite_and_empty_queries_give_default_records(scene, cfg):
    dim, s, g = scene
    rng = np.random.default_rng(81)
    pts, r2, mask = bad_rows(dim, 20000, rng)
    g.set_traversal(**cfg)
    out = F.GPUInteractionList()
    g.find_closest_points(pts, r2, out)
    got = out.array()
    clean = F.GPUInteractionList()
    g.find_closest_points(pts[~mask], r2[~mask], clean)
    g.set_traversal(0)
    assert g.check_errors() == 0
    assert np.all(got["index"][mask] == R.UINT_MAX)
    assert np.all(got["d"][mask] == R.FLT_MAX)
    # the other queries of the batch are not affected (a bad query is not
    # even a tie partner: records are byte-identical)
    assert got[~mask].tobytes() == clean.array().tobytes()


@pytest.mark.parametrize("cfg", [dict(branching=0), dict(branching=4, bits=32)])
def test_non_finite_silhouette_and_ray_queries(scene, cfg):
    dim, s, g = scene
    rng = np.random.default_rng(82)
    pts, r2, mask = bad_rows(dim, 8000, rng)
    flip = np.zeros(len(pts), np.uint32)
    g.set_traversal(**cfg)
    out = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, r2, flip, out)
    got = out.array()
    assert np.all(got["index"][mask] == R.UINT_MAX)
    clean = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts[~mask], r2[~mask], flip[~mask], clean)
    assert got[~mask].tobytes() == clean.array().tobytes()
    # rays with non-finite origins or directions miss
    d = rng.normal(size=(len(pts), dim)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[mask] = np.nan
    rays = F.GPUInteractionList()
    g.intersect(pts, d, np.full(len(pts), R.FLT_MAX, np.float32), rays)
    assert np.all(rays.array()["index"][mask] == R.UINT_MAX)
    g.set_traversal(0)
    assert g.check_errors() == 0


def test_injected_allocation_failures_are_reported_and_recoverable():
    """The failure walks through every device allocation of a transfer and a
    first fast-path query (wide tree, sort scratch, refinement scratch): each
    reports FCPWGB_ERR_OUT_OF_MEMORY, and afterwards the same scene object
    transfers and answers exactly as one that never failed."""
    v, f = W.perturbed_sphere(16, W.SEED_BASE + 83)
    s = build_scene(3, v, f)
    pts = W.uniform_points(50000, 3, -1.5, 1.5, 84)
    r2 = np.full(len(pts), R.FLT_MAX, np.float32)
    g0 = F.GPUScene3D()
    g0.transfer_to_gpu(s)
    g0.set_traversal(4, 32, packet=True)
    ref = F.GPUInteractionList()
    g0.find_closest_points(pts, r2, ref)
    failures = 0
    try:
        for skip in range(64):
            g = F.GPUScene3D()
            check(lib().fcpwgb_debug_fail_allocations(skip, 1))
            try:
                g.transfer_to_gpu(s)
                g.set_traversal(4, 32, packet=True)
                g.find_closest_points(pts, r2, F.GPUInteractionList())
                failed = False
            except F.FcpwError as e:
                assert e.code == 5, e  # FCPWGB_ERR_OUT_OF_MEMORY
                failed = True
            check(lib().fcpwgb_debug_fail_allocations(0, 0))
            g.transfer_to_gpu(s)
            g.set_traversal(4, 32, packet=True)
            got = F.GPUInteractionList()
            g.find_closest_points(pts, r2, got)
            assert got.array().tobytes() == ref.array().tobytes(), skip
            assert g.check_errors() == 0
            if not failed:
                break
            failures += 1
    finally:
        check(lib().fcpwgb_debug_fail_allocations(0, 0))
    assert failures >= 5  # transfer buffers, wide tree, sort and refinement scratch
    with pytest.raises(F.FcpwError):
        check(lib().fcpwgb_debug_fail_allocations(-1, 1))


def test_mismatched_sizes_and_missing_transfer_raise():
    v, f = W.perturbed_sphere(8, W.SEED_BASE + 85)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    pts = W.uniform_points(100, 3, -1, 1, 86)
    with pytest.raises(F.FcpwError):
        g.find_closest_points(pts, np.full(100, R.FLT_MAX, np.float32), F.GPUInteractionList())
    g.transfer_to_gpu(s)
    with pytest.raises(ValueError):
        g.find_closest_points(pts, np.full(99, R.FLT_MAX, np.float32), F.GPUInteractionList())
    with pytest.raises(ValueError):
        g.intersect(pts, pts[:50], np.full(100, R.FLT_MAX, np.float32), F.GPUInteractionList())


def test_injected_allocation_failures_in_a_batch():
    """The same walk for a batch of meshes: the forest, the layout and sort
    scratch, the refinement scratch and the captured graph; each failure
    reports FCPWGB_ERR_OUT_OF_MEMORY and the same batch object then answers
    byte-identically to one that never failed."""
    meshes = [W.perturbed_sphere(8, W.SEED_BASE + 87), W.torus(32, 16, W.SEED_BASE + 88)]
    scenes = [build_scene(3, v, f) for v, f in meshes]
    pts = np.concatenate([W.uniform_points(6000, 3, -1.2, 1.2, 89), W.uniform_points(9000, 3, -1.5, 1.5, 90)])
    offsets = np.array([0, 6000, 15000], np.uint32)
    r2 = np.full(len(pts), R.FLT_MAX, np.float32)
    b0 = F.GPUSceneBatch3D()
    b0.set_scenes(scenes)
    b0.set_traversal(4, 32, packet=True)
    ref = F.GPUInteractionList()
    b0.find_closest_points(pts, r2, offsets, ref)
    failures = 0
    try:
        for skip in range(64):
            b = F.GPUSceneBatch3D()
            check(lib().fcpwgb_debug_fail_allocations(skip, 1))
            try:
                b.set_scenes(scenes)
                b.set_traversal(4, 32, packet=True)
                b.find_closest_points(pts, r2, offsets, F.GPUInteractionList())
                failed = False
            except F.FcpwError as e:
                assert e.code == 5, e
                failed = True
            check(lib().fcpwgb_debug_fail_allocations(0, 0))
            b.set_scenes(scenes)
            b.set_traversal(4, 32, packet=True)
            got = F.GPUInteractionList()
            b.find_closest_points(pts, r2, offsets, got)
            assert got.array().tobytes() == ref.array().tobytes(), skip
            if not failed:
                break
            failures += 1
    finally:
        check(lib().fcpwgb_debug_fail_allocations(0, 0))
    assert failures >= 4
