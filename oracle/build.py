"""Build recipe of the oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/_build/liboracle.so``: the plain-C restatement in fcpw_oracle.c,
  compiled with gcc on any host (x86 here, Arm on the GPU machine).
* ``baseline/_ref/``: an unmodified copy of the reference's CPU headers
  (``include/fcpw``) and of its vendored Enoki headers
  (``deps/enoki/include/enoki``), staged from the reference checkout where one
  exists. The reference root is ``$FCPW_REFERENCE_ROOT``, else
  ``/root/reference`` (the checkout of the machine the fixtures were made on).
  The staged copy is git-ignored, and it is what travels to a machine without
  the checkout, so the reference builds there too.
* ``oracle/_ref/libfcpw_ref.so``: the staged reference headers compiled against
  the Eigen API shim in oracle/compat, with the driver ref_driver.cpp
  (scalar ``Bvh``, the reference's comparator configuration, vectorize=false).
* ``oracle/_ref/libfcpw_ref_simd.so``: the same with ``FCPW_USE_ENOKI`` and
  ``FCPW_SIMD_WIDTH=4`` (the reference's setting for NEON / SSE hosts), so that
  ``Scene::build(..., vectorize=true)`` makes the reference's Mbvh. Timing only.

The scalar builds are compiled without floating-point contraction, so their
float results do not depend on the host ISA.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_LIB = BUILD / "liboracle.so"
REF_LIB = REF_OUT / "libfcpw_ref.so"
REF_SIMD_LIB = REF_OUT / "libfcpw_ref_simd.so"
REF_SIMD_ERROR = REF_OUT / "libfcpw_ref_simd.error.txt"  # why the vectorised build failed on this host
STAGED = REPO / "baseline" / "_ref"
STAGED_INCLUDE = STAGED / "include"
STAGED_ENOKI = STAGED / "deps" / "enoki" / "include"


def reference_root() -> Path:
    return Path(os.environ.get("FCPW_REFERENCE_ROOT", "/root/reference"))


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


_staged_this_process = False


def stage_reference() -> bool:
    """Copies the reference's headers into baseline/_ref when the checkout is
    present (replacing an older copy, once per process); True when a staged
    copy exists."""
    global _staged_this_process
    root = reference_root()
    src_inc = root / "include" / "fcpw"
    if not _staged_this_process and (src_inc / "fcpw.h").exists():
        _staged_this_process = True
        for src, dst in ((src_inc, STAGED_INCLUDE / "fcpw"),
                         (root / "deps" / "enoki" / "include" / "enoki", STAGED_ENOKI / "enoki")):
            if not src.exists():
                continue
            if dst.exists():
                shutil.rmtree(dst)
            shutil.copytree(src, dst)
    return (STAGED_INCLUDE / "fcpw" / "fcpw.h").exists()


def reference_include() -> Path | None:
    """The staged reference include directory, staging it first where possible."""
    return STAGED_INCLUDE if stage_reference() else None


def _deps():
    return [HERE / "ref_driver.cpp"] + list((HERE / "compat" / "Eigen").glob("*"))


def _build_ref(out: Path, extra: list[str], force: bool) -> Path | None:
    inc = reference_include()
    if inc is None:
        return None
    REF_OUT.mkdir(parents=True, exist_ok=True)
    newest = max(p.stat().st_mtime for p in _deps() + [inc / "fcpw" / "fcpw.h"])
    if not force and out.exists() and out.stat().st_mtime >= newest:
        return out
    tmp = out.with_suffix(".so.tmp")
    cmd = [_cxx(), "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-Wno-psabi", *extra,
           "-I", str(HERE / "compat"), "-I", str(inc), str(HERE / "ref_driver.cpp"), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        errors = [ln for ln in r.stderr.splitlines() if "error" in ln]
        if out == REF_SIMD_LIB:
            REF_SIMD_ERROR.write_text("\n".join(errors[:4]) + "\n")
        raise RuntimeError(f"reference build failed ({out.name}):\n" + "\n".join(errors[:20]) + "\n" +
                           r.stderr[-3000:])
    os.replace(tmp, out)
    return out


def build_reference(force: bool = False) -> Path | None:
    """Compiles the reference CPU path (scalar Bvh) where its headers are staged; None otherwise."""
    return _build_ref(REF_LIB, ["-ffp-contract=off"], force)


def build_reference_simd(force: bool = False) -> Path | None:
    """The reference with Enoki packets of 4 floats (its Mbvh, vectorize=true), where the
    staged copy includes Enoki; None otherwise. Enoki's NEON backend needs no flag on
    aarch64; elsewhere the build takes whatever vector ISA the compiler's default enables."""
    if reference_include() is None or not (STAGED_ENOKI / "enoki" / "array.h").exists():
        return None
    if REF_SIMD_ERROR.exists():
        REF_SIMD_ERROR.unlink()
    extra = ["-DFCPW_USE_ENOKI", "-DFCPW_SIMD_WIDTH=4", "-I", str(STAGED_ENOKI), "-O3"]
    if host_isa() in ("aarch64", "arm64"):
        # Enoki's NEON backend converts between vector register types implicitly, which GCC 13 rejects
        # unless told otherwise
        extra += ["-flax-vector-conversions", "-fpermissive"]
    return _build_ref(REF_SIMD_LIB, extra, force)


def host_isa() -> str:
    return platform.machine()


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
    try:
        print(build_reference_simd(force=True))
    except RuntimeError as e:
        print(e)
