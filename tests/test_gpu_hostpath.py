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
