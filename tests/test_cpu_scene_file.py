"""Scene files (no GPU needed to write or inspect them): header counts,
checksum protection against corruption and truncation."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import workloads as W
from helpers import build_scene


@pytest.mark.parametrize("dim,silhouettes", [(3, False), (3, True), (2, True)])
def test_scene_file_header_and_checksum(tmp_path, dim, silhouettes):
    if dim == 3:
        v, f = W.torus(24, 12, W.SEED_BASE + 70)
    else:
        v, f = W.star_polylines(4, 32, W.SEED_BASE + 71)
    s = build_scene(dim, v, f, silhouettes=silhouettes)
    path = tmp_path / "scene.fcpwgb"
    s.cpu_bvh.save(path, wide=[(4, 32), (8, 8, 6)])
    info = F.scene_file_info(path)
    bi = s.cpu_bvh.info
    assert (info["dim"], info["n_nodes"], info["n_primitives"], info["n_vertices"], info["n_wide"]) == \
        (dim, bi.n_nodes, bi.n_primitives, bi.n_vertices, 2)
    assert info["n_silhouettes"] == (bi.n_silhouettes if silhouettes else 0)
    data = bytearray(path.read_bytes())
    assert len(data) % 8 == 0
    # one flipped byte anywhere is caught by the checksum
    bad = tmp_path / "bad.fcpwgb"
    data[len(data) // 2] ^= 0x40
    bad.write_bytes(bytes(data))
    with pytest.raises(F.FcpwError, match="checksum"):
        F.scene_file_info(bad)
    trunc = tmp_path / "trunc.fcpwgb"
    trunc.write_bytes(path.read_bytes()[:-100])
    with pytest.raises(F.FcpwError):
        F.scene_file_info(trunc)
    with pytest.raises(F.FcpwError):
        F.scene_file_info(tmp_path / "missing.fcpwgb")
