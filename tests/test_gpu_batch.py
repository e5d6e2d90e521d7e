"""GPU parity of batched scenes (one persistent launch over a forest of wide
trees, replayed from a CUDA graph) against the oracle run on every scene on
its own: uneven scene sizes and query counts, empty query sets, every
branching factor and box precision, graph replay and the host-array path."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from fcpw_gb300._lib import FcpwError
from helpers import build_scene, compare_closest
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _meshes3():
    out = []
    for k, (kind, size) in enumerate([("sphere", 6), ("torus", 48), ("sphere", 20), ("torus", 24), ("sphere", 3),
                                      ("torus", 96)]):
        if kind == "sphere":
            v, f = W.perturbed_sphere(size, W.SEED_BASE + 60 + k)
        else:
            v, f = W.torus(size, size // 2, W.SEED_BASE + 60 + k)
        v = v * (0.5 + 0.3 * k) + np.float32(k)  # scenes of different scale and place
        out.append((v.astype(np.float32), f))
    return out


@pytest.fixture(scope="module")
def batch3():
    meshes = _meshes3()
    scenes = [build_scene(3, v, f) for v, f in meshes]
    counts = [5000, 0, 20000, 137, 1, 9000]
    pts, refs, prims = [], [], []
    for k, ((v, f), s, nq) in enumerate(zip(meshes, scenes, counts)):
        lo, hi = v.min(0), v.max(0)
        c, h = (lo + hi) / 2, (hi - lo).max() * 0.9
        p = W.uniform_points(nq, 3, -1.0, 1.0, 70 + k) * h + c if nq else np.zeros((0, 3), np.float32)
        p = p.astype(np.float32)
        nodes, pr, _ = s.cpu_bvh.export()
        refs.append(O.closest_points_bvh(3, nodes, pr, R.make_spheres(p, R.FLT_MAX)) if nq else None)
        pts.append(p)
        prims.append(pr)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    b = F.GPUSceneBatch3D()
    b.set_scenes(scenes)
    return b, scenes, pts, refs, prims, offsets


def _check(b, pts, refs, prims, offsets, got, what):
    for k in range(len(pts)):
        if len(pts[k]) == 0:
            continue
        g = got[offsets[k]:offsets[k + 1]]
        compare_closest(b.DIM, prims[k], pts[k], g, refs[k], f"{what} scene {k}")


def _tensor_run(b, pts, offsets, **kw):
    import torch
    allp = np.concatenate(pts)
    sph = torch.from_numpy(R.make_spheres(allp, R.FLT_MAX).view(np.float32).reshape(-1, 4).copy()).cuda()
    res = b.find_closest_points_tensor(sph, offsets, **kw)
    torch.cuda.synchronize()
    return res.raw.cpu().numpy().view(R.INTERACTION).reshape(-1), sph


@pytest.mark.parametrize("branching", [2, 4, 8])
@pytest.mark.parametrize("bits", [32, 16, 8])
@pytest.mark.parametrize("schedule", ["thread", "persistent", "packet", "packetq", "coop4"])
def test_batch_matches_per_scene_oracle(batch3, branching, bits, schedule):
    """Warps straddling scene boundaries (137 and 1 queries) exercise the
    per-root passes of the packet kernel and the root change of the seeds."""
    b, scenes, pts, refs, prims, offsets = batch3
    b.set_traversal(branching, bits, persistent=schedule in ("persistent", "packetq"), precise=True,
                    packet=schedule in ("packet", "packetq"), threads_per_query=4 if schedule == "coop4" else 1)
    got, _ = _tensor_run(b, pts, offsets)
    _check(b, pts, refs, prims, offsets, got, f"batch {branching}/{bits}/{schedule}")
    assert b.check_errors() == 0


def test_batch_graph_replay_and_host_path_agree(batch3):
    b, scenes, pts, refs, prims, offsets = batch3
    b.set_traversal(4, 8, persistent=False)
    b.use_graph(True)
    first, sph = _tensor_run(b, pts, offsets)
    import torch
    res = b.find_closest_points_tensor(sph, offsets)  # replays the captured graph
    torch.cuda.synchronize()
    second = res.raw.cpu().numpy().view(R.INTERACTION).reshape(-1)
    assert first.tobytes() == second.tobytes()
    b.use_graph(False)
    third, _ = _tensor_run(b, pts, offsets)
    assert first.tobytes() == third.tobytes()
    b.use_graph(True)
    out = F.GPUInteractionList()
    b.find_closest_points(np.concatenate(pts), np.full(int(offsets[-1]), R.FLT_MAX, np.float32), offsets, out)
    assert out.array().tobytes() == first.tobytes()
    info = b.info()
    assert info["scenes"] == len(scenes) and info["sort_cells"] > 0


def test_batch_rejects_bad_offsets(batch3):
    import torch
    b, scenes, pts, refs, prims, offsets = batch3
    sph = torch.zeros((int(offsets[-1]), 4), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        b.find_closest_points_tensor(sph, offsets[:-1])
    bad = offsets.copy()
    bad[2], bad[3] = bad[3], bad[2]
    if bad[2] != bad[3]:
        with pytest.raises(FcpwError):
            b.find_closest_points_tensor(sph, bad)


def test_batch_2d_segments():
    scenes, pts, refs, prims = [], [], [], []
    counts = [3000, 50, 7000]
    for k, nq in enumerate(counts):
        v, sg = W.star_polylines(4 + 6 * k, 64 + 32 * k, W.SEED_BASE + 80 + k)
        s = build_scene(2, v, sg)
        p = W.uniform_points(nq, 2, -3, 3, 90 + k).astype(np.float32)
        nodes, pr, _ = s.cpu_bvh.export()
        refs.append(O.closest_points_bvh(2, nodes, pr, R.make_spheres(p, R.FLT_MAX)))
        scenes.append(s)
        pts.append(p)
        prims.append(pr)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    b = F.GPUSceneBatch2D()
    b.set_scenes(scenes)
    for cfg in [(4, 8, False, True, False), (8, 16, True, True, False), (2, 32, False, True, False),
                (4, 8, False, True, True)]:
        b.set_traversal(*cfg)
        out = F.GPUInteractionList()
        b.find_closest_points(np.concatenate(pts), np.full(int(offsets[-1]), R.FLT_MAX, np.float32), offsets, out)
        _check(b, pts, refs, prims, offsets, out.array(), f"2D batch {cfg}")
        assert np.all(out.array()["p"][:, 2] == 0)
