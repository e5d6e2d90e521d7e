"""fcpwgb_gpu_scene_update_vertices_device_static (refit counters in a static
device array, no allocation) against fcpwgb_gpu_scene_update_vertices_device
(counters owned by the scene), called through the C ABI. Two calls in a row
on the same scene check that the shared array, which keeps the previous call's
arrival counts, is cleared before each refit: before each call the array is
filled with non-zero words, and free device memory is compared around the
call. The refit unions child boxes
with exact min/max and merges cones in a fixed child order, so the two entry
points must agree bit for bit: the tolerance here is exact equality of the
exported nodes and of the closest point records that use them.

Collected last so that it also runs after every other GPU test in a session."""
import ctypes as C

import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from fcpw_gb300._lib import FcpwError, check, lib
from helpers import build_scene

pytestmark = pytest.mark.gpu

MAX_NODES = 1 << 20


def _moved(v, seed, amp):
    return (v + amp * W.rng(seed).standard_normal(v.shape)).astype(np.float32)


def _update(entry, g, positions, stream):
    return getattr(lib(), entry)(g.handle, C.c_void_p(positions.data_ptr()), positions.shape[0], C.c_void_p(stream))


def _closest(g, pts):
    out = F.GPUInteractionList()
    g.find_closest_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    return out.array()


def _silhouettes(g, pts):
    out = F.GPUInteractionList()
    g.find_closest_silhouette_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), np.zeros(len(pts), np.uint32),
                                     out)
    return out.array()


@pytest.mark.parametrize("dim", [3, 2])
def test_static_scratch_refit_matches_scene_scratch_refit(dim):
    import torch
    if dim == 3:
        v, idx = W.perturbed_sphere(24, W.SEED_BASE + 40)
        s = build_scene(3, v, idx)
        a, b = F.GPUScene3D(), F.GPUScene3D()
        amp, lo, hi = 0.02, -1.5, 1.5
    else:
        v, idx = W.star_polylines(32, 96, W.SEED_BASE + 41)
        s = build_scene(2, v, idx, silhouettes=True)
        a, b = F.GPUScene2D(), F.GPUScene2D()
        amp, lo, hi = 0.002, -3.0, 3.0
    a.transfer_to_gpu(s)
    b.transfer_to_gpu(s)
    assert s.cpu_bvh.info.n_nodes <= MAX_NODES
    pts = W.uniform_points(20000, dim, lo, hi, 42)
    stream = torch.cuda.current_stream().cuda_stream
    n_nodes = s.cpu_bvh.info.n_nodes
    for call, seed in enumerate((43, 44)):
        pos = torch.from_numpy(_moved(v, seed, amp)).cuda()
        check(_update("fcpwgb_gpu_scene_update_vertices_device", a, pos, stream))
        # every arrival counter the refit reads starts non-zero unless the call clears it: a refit
        # that skipped the clear would merge nodes before their children are ready
        check(lib().fcpwgb_debug_fill_static_scratch(b.handle, 0x5A5A5A5A if call else 1, n_nodes))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        check(_update("fcpwgb_gpu_scene_update_vertices_device_static", b, pos, stream))
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free refit changed free device memory"
        na, nb = a.export_nodes(), b.export_nodes()
        assert na.tobytes() == nb.tobytes(), f"call {call}: refit nodes differ"
        ra, rb = _closest(a, pts), _closest(b, pts)
        assert np.array_equal(ra["index"], rb["index"]) and np.array_equal(ra["d"], rb["d"]), f"call {call}"
        if dim == 2:
            sa, sb = _silhouettes(a, pts), _silhouettes(b, pts)
            assert np.array_equal(sa["index"], sb["index"]) and np.array_equal(sa["d"], sb["d"]), f"call {call}"
        assert a.check_errors() == 0 and b.check_errors() == 0


def test_static_scratch_refit_rejects_trees_beyond_the_maximum():
    import torch
    v, f = W.torus(1024, 1024, W.SEED_BASE + 45)
    s = build_scene(3, v, f)
    assert s.cpu_bvh.info.n_nodes > MAX_NODES
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    pos = torch.from_numpy(v).cuda()
    rc = _update("fcpwgb_gpu_scene_update_vertices_device_static", g, pos, torch.cuda.current_stream().cuda_stream)
    assert rc == 1  # FCPWGB_ERR_INVALID_ARGUMENT
    msg = lib().fcpwgb_last_error().decode()
    assert "static refit scratch holds at most 1048576" in msg, msg
    with pytest.raises(FcpwError):
        check(rc)


def test_static_scratch_refit_status_codes_equal_the_scene_scratch_entry():
    """Both entry points answer an unsupported scene with the same status."""
    import torch
    v, f = W.perturbed_sphere(8, W.SEED_BASE + 46)
    s = F.Scene3D()
    s.set_object_count(1)
    s.set_object_vertices(v, 0)
    s.set_object_triangles(f, 0)
    s.set_object_instance_transforms([np.eye(4, dtype=np.float32)] * 2, 0)
    s.build(F.AggregateType.Bvh_SurfaceArea, False)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    pos = torch.from_numpy(v).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    rc_scene = _update("fcpwgb_gpu_scene_update_vertices_device", g, pos, stream)
    rc_static = _update("fcpwgb_gpu_scene_update_vertices_device_static", g, pos, stream)
    assert rc_scene == rc_static != 0
    fresh = F.GPUScene3D()
    assert (_update("fcpwgb_gpu_scene_update_vertices_device", fresh, pos, stream)
            == _update("fcpwgb_gpu_scene_update_vertices_device_static", fresh, pos, stream) != 0)
