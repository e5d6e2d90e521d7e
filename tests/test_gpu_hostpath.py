"""The host-array entry point fcpwgb_find_closest_points: in precise mode on
triangles with sorted queries and a page-locked output array, the
refinement pass writes the records straight into that array in the caller's
order; otherwise the records are copied back from a device buffer. Both give
the records of the device-array entry point, byte for byte, and leave the
device error word clear."""
import ctypes as C

import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from fcpw_gb300._lib import check, lib
from helpers import build_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg", [dict(branching=4, bits=32, packet=True, persistent=True),
                                 dict(branching=8, bits=16, packet=False, persistent=True),
                                 dict(branching=4, bits=32, packet=True, sort_queries=False),
                                 dict(branching=4, bits=32, packet=True, precise=False),
                                 dict(branching=0)],
                         ids=["packetq", "w8q16-persistent", "unsorted", "fp32", "binary"])
@pytest.mark.parametrize("record_normals", [0, 1])
def test_host_array_records_equal_device_records(cfg, record_normals):
    import torch
    v, f = W.torus(128, 64, W.SEED_BASE + 2)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    g.set_traversal(**cfg)
    n = 50_000
    pts = W.uniform_points(n, 3, -2.0, 2.0, 88)
    r2 = np.where(W.rng(89).uniform(0, 1, n) < 0.2, 0.05, R.FLT_MAX).astype(np.float32)
    sph = R.make_spheres(pts, r2)
    d_sph = torch.from_numpy(sph.view(np.float32).reshape(n, 4).copy()).cuda()
    d_out = torch.empty((n, 10), dtype=torch.float32, device="cuda")
    check(lib().fcpwgb_find_closest_points_device(g.handle, d_sph.data_ptr(), d_out.data_ptr(), n, record_normals,
                                                  None))
    torch.cuda.synchronize()
    want = d_out.cpu().numpy()
    h_sph = torch.from_numpy(sph.view(np.float32).reshape(n, 4).copy()).pin_memory()
    pinned = torch.full((n, 10), -7.0, dtype=torch.float32).pin_memory()
    check(lib().fcpwgb_find_closest_points(g.handle, h_sph.data_ptr(), pinned.data_ptr(), n, record_normals))
    pageable = np.full((n, 10), -7.0, np.float32)
    check(lib().fcpwgb_find_closest_points(g.handle, h_sph.data_ptr(), pageable.ctypes.data, n, record_normals))
    assert np.array_equal(pinned.numpy().view(np.uint32), want.view(np.uint32))
    assert np.array_equal(pageable.view(np.uint32), want.view(np.uint32))
    assert g.check_errors() == 0


def test_misaligned_arrays():
    """Device arrays off the boundary the kernels read them on are refused
    before anything is launched (the scene stays usable); a page-locked
    output array off a 16 B boundary takes the copy path and gets the same
    records."""
    import torch
    from fcpw_gb300._lib import FcpwError
    v, f = W.torus(64, 32, W.SEED_BASE + 2)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    g.set_traversal(4, 32, packet=True, persistent=True)
    n = 20_000
    sph = R.make_spheres(W.uniform_points(n, 3, -2.0, 2.0, 90), R.FLT_MAX)
    flat = sph.view(np.float32).reshape(n, 4)
    d_out = torch.empty((n, 10), dtype=torch.float32, device="cuda")
    shifted = torch.empty(4 * n + 2, dtype=torch.float32, device="cuda")  # spheres 8 B off their 16 B boundary
    shifted[2:] = torch.from_numpy(flat.reshape(-1).copy()).cuda()
    with pytest.raises(FcpwError):
        check(lib().fcpwgb_find_closest_points_device(g.handle, shifted.data_ptr() + 8, d_out.data_ptr(), n, 0, None))
    odd_out = torch.empty(10 * n + 1, dtype=torch.float32, device="cuda")  # records 4 B off their 8 B boundary
    d_sph = torch.from_numpy(flat.copy()).cuda()
    with pytest.raises(FcpwError):
        check(lib().fcpwgb_find_closest_points_device(g.handle, d_sph.data_ptr(), odd_out.data_ptr() + 4, n, 0, None))
    check(lib().fcpwgb_find_closest_points_device(g.handle, d_sph.data_ptr(), d_out.data_ptr(), n, 0, None))
    torch.cuda.synchronize()
    want = d_out.cpu().numpy()
    h_sph = torch.from_numpy(flat.copy()).pin_memory()
    pinned = torch.full((n + 1, 10), -7.0, dtype=torch.float32).pin_memory()  # record 1 starts 40 B in: 8 B off 16
    check(lib().fcpwgb_find_closest_points(g.handle, h_sph.data_ptr(), pinned.data_ptr() + 40, n, 0))
    got = pinned.numpy()[1:]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.all(pinned.numpy()[0] == -7.0)
    assert g.check_errors() == 0
