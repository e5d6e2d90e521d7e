"""The C++ drop-in (include/fcpw_gb300_gpu.hpp) compiles against the
reference's own headers unmodified (via the Eigen API shim), links against
the library, and turns failures into exceptions. Runs where the reference
headers are staged (oracle/build.py copies them into baseline/_ref from the
reference checkout)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _reference_include():
    from oracle.build import reference_include
    return reference_include()

PROGRAM = r"""
#include <fcpw_gb300_gpu.hpp>
#include <cstdio>
int main() {
    fcpw::Scene<3> scene;
    std::vector<fcpw::Vector3> v = {fcpw::Vector3(0, 0, 0), fcpw::Vector3(1, 0, 0), fcpw::Vector3(0, 1, 0),
                                    fcpw::Vector3(0, 0, 1)};
    std::vector<fcpw::Vector3i> t = {fcpw::Vector3i(0, 1, 2), fcpw::Vector3i(0, 1, 3), fcpw::Vector3i(0, 2, 3),
                                     fcpw::Vector3i(1, 2, 3)};
    scene.setObjectCount(1);
    scene.setObjectVertices(v, 0);
    scene.setObjectTriangles(t, 0);
    scene.build(fcpw::AggregateType::Bvh_SurfaceArea, false);
    try {
        fcpw::GPUScene<3> gpu("unused");
        gpu.transferToGPU(scene);
        std::vector<fcpw::GPUBoundingSphere> s = {fcpw::GPUBoundingSphere(fcpw::float3{0.2f, 0.2f, 2.0f}, 1e30f)};
        std::vector<fcpw::GPUInteraction> out;
        gpu.findClosestPoints(s, out);
        std::printf("ran d=%f index=%u\n", out[0].d, out[0].index);
    } catch (const std::runtime_error &e) {
        std::printf("exception: %s\n", e.what());
    }
    return 0;
}
"""


def test_cpp_dropin_compiles_links_and_reports_errors(tmp_path):
    from fcpw_gb300 import library_path
    REF = _reference_include()
    if REF is None:
        pytest.skip("the reference headers are not staged on this machine (oracle/build.py)")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    lib = library_path()
    cmd = [cxx, "-std=c++17", "-O1", "-I", str(ROOT / "oracle" / "compat"), "-I", str(REF), "-I", str(ROOT / "include"),
           str(src), "-o", str(exe), "-L", str(lib.parent), "-lfcpw_gb300", f"-Wl,-rpath,{lib.parent}", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0
    out = run.stdout
    assert out.startswith("ran d=") or "exception: fcpw_gb300:" in out, out
