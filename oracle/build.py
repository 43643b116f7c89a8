"""Build recipes for the oracle (test infrastructure, never shipped).

* ``build_oracle()`` compiles the C restatement ``oracle/gl_oracle.c`` into
  ``oracle/_build/libgl_oracle.so``.  It is self-contained and builds on any
  host with gcc (this container and the GPU host alike).
* ``build_ref()`` compiles the reference's own CPU sources for the flare path
  (JaydenB/ghostlight ``ghostlight/src``: trace.cpp, ghost.cpp, spectral.cpp,
  lens_calibration.cpp, spawn_probe.cpp, source_map.cpp, optical_system.cpp)
  from where they lie, together with ``oracle/ref_driver.cpp``, into
  ``oracle/_ref/libghostlight_ref.so``.  It needs the reference checkout and
  is skipped when that is absent.

Both use ``-ffp-contract=off`` so the float arithmetic is the reference
host build's (x86-64 g++ has no FMA contraction by default) on every machine.
"""
from __future__ import annotations

import os
import pathlib
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE_ROOT = pathlib.Path(os.environ.get("GHOSTLIGHT_REFERENCE", "/root/reference"))

ORACLE_LIB = BUILD / "libgl_oracle.so"
REF_LIB = REF_OUT / "libghostlight_ref.so"

REF_SOURCES = ["trace.cpp", "ghost.cpp", "spectral.cpp", "lens_calibration.cpp",
               "spawn_probe.cpp", "source_map.cpp", "optical_system.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(map(str, cmd)), r.stdout, r.stderr))


def _stale(target: pathlib.Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(pathlib.Path(d).stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "gl_oracle.c"]
    deps = srcs + [HERE / "gl_oracle_impl.h", REPO / "include" / "ghostlight_gb300.h"]
    if force or _stale(ORACLE_LIB, deps):
        tmp = ORACLE_LIB.with_suffix(".so.tmp%d" % os.getpid())
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-std=c11", "-I", str(REPO / "include"), *map(str, srcs),
              "-o", str(tmp), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_available() -> bool:
    return (REFERENCE_ROOT / "ghostlight" / "src" / "trace.cpp").exists()


def build_ref(force: bool = False):
    """Build oracle/_ref from the reference sources; None when absent."""
    if not reference_available():
        return None
    REF_OUT.mkdir(exist_ok=True)
    src_dir = REFERENCE_ROOT / "ghostlight" / "src"
    srcs = [HERE / "ref_driver.cpp"] + [src_dir / s for s in REF_SOURCES]
    if force or _stale(REF_LIB, srcs + [REPO / "include" / "ghostlight_gb300.h"]):
        tmp = REF_LIB.with_suffix(".so.tmp%d" % os.getpid())
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
              "-ffp-contract=off",
              "-I", str(src_dir), "-I", str(REFERENCE_ROOT / "ghostlight" / "third_party"),
              "-I", str(REPO / "include"), *map(str, srcs), "-o", str(tmp)])
        os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
