"""Build recipe of the oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/_build/liboracle.so``: the plain-C restatement in fcpw_oracle.c,
  compiled with gcc on any host (x86 here, Arm on the GPU machine).
* ``oracle/_ref/libfcpw_ref.so``: the reference's own CPU headers
  (include/fcpw under the reference checkout, default /root/reference) compiled
  unmodified against the Eigen API shim in oracle/compat, with the driver
  ref_driver.cpp. Only built where the reference checkout exists.

Both are compiled without floating-point contraction, so their float results do
not depend on the host ISA.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_LIB = BUILD / "liboracle.so"
REF_LIB = REF_OUT / "libfcpw_ref.so"
REFERENCE_ROOT = Path(os.environ.get("FCPW_REFERENCE_ROOT", "/root/reference"))


def _cc() -> str:
    return os.environ.get("CC") or shutil.which("gcc") or "cc"


def _cxx() -> str:
    return os.environ.get("CXX") or shutil.which("g++") or "c++"


def build_oracle(force: bool = False) -> Path:
    src = HERE / "fcpw_oracle.c"
    BUILD.mkdir(parents=True, exist_ok=True)
    if not force and ORACLE_LIB.exists() and ORACLE_LIB.stat().st_mtime >= src.stat().st_mtime:
        return ORACLE_LIB
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cmd = [_cc(), "-std=c99", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", str(src), "-o", str(tmp),
           "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference(force: bool = False) -> Path | None:
    """Compiles the reference CPU path where its sources are present; None otherwise."""
    inc = REFERENCE_ROOT / "include"
    if not (inc / "fcpw" / "fcpw.h").exists():
        return None
    src = HERE / "ref_driver.cpp"
    deps = [src] + list((HERE / "compat" / "Eigen").glob("*"))
    REF_OUT.mkdir(parents=True, exist_ok=True)
    newest = max(p.stat().st_mtime for p in deps)
    if not force and REF_LIB.exists() and REF_LIB.stat().st_mtime >= newest:
        return REF_LIB
    tmp = REF_LIB.with_suffix(".so.tmp")
    cmd = [_cxx(), "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           "-I", str(HERE / "compat"), "-I", str(inc), str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stderr[-6000:]}")
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
