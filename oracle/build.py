"""Build recipes for the oracle (test infrastructure, never shipped).

* ``build_oracle()`` compiles the C restatement ``oracle/gl_oracle.c`` into
  ``oracle/_build/libgl_oracle.so``.  It is self-contained and builds on any
  host with gcc (this container and the GPU host alike).
* ``build_ref()`` compiles the reference's own CPU sources for the flare path
  (JaydenB/ghostlight ``ghostlight/src``: trace.cpp, ghost.cpp, spectral.cpp,
  lens_calibration.cpp, spawn_probe.cpp, source_map.cpp, optical_system.cpp),
  together with ``oracle/ref_driver.cpp``, into
  ``oracle/_ref/libghostlight_ref.so``.
* ``build_ref_gpu()`` compiles the reference's whole core library (its CUDA
  renderers included, for sm_103a, with the reference's own fast-math flags
  from ghostlight/CMakeLists.txt:97-109 and cuFFT) with the same driver into
  ``oracle/_ref/libghostlight_ref_gpu.so``: the reference GPU renderer.

The reference sources are read from the staged, git-ignored copy in
``baseline/_ref/`` (``oracle/stage_ref.py`` makes it from a checkout), so the
same recipes run on every host that carries the working tree; both builds are
skipped (None) where no staged copy exists.  The CPU builds use
``-ffp-contract=off`` so the float arithmetic is the reference host build's
(x86-64 g++ has no FMA contraction by default) on every machine.
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
REFERENCE_ROOT = REPO / "baseline" / "_ref"      # staged by oracle/stage_ref.py

ORACLE_LIB = BUILD / "libgl_oracle.so"
REF_LIB = REF_OUT / "libghostlight_ref.so"
REF_GPU_LIB = REF_OUT / "libghostlight_ref_gpu.so"

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


def _stage():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_gl_stage_ref", HERE / "stage_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.stage()


def reference_available() -> bool:
    return (REFERENCE_ROOT / "ghostlight" / "src" / "trace.cpp").exists()


def build_ref(force: bool = False):
    """Build oracle/_ref from the reference sources; None when absent."""
    _stage()
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


REF_GPU_CU = ["ghost_render.cu", "psf_render.cu", "starburst_render.cu", "mdft_render.cu", "veil_render.cu",
              "gate_render.cu", "fft_cufft.cu", "aperture_textures.cu", "coating_upload.cu"]
REF_GPU_CPP = ["PointFlareRenderer.cpp", "SourceFlareRenderer.cpp", "PSFRenderer.cpp", "lens_calibration.cpp",
               "spawn_probe.cpp", "source_map.cpp", "spectral.cpp", "optical_system.cpp", "trace.cpp",
               "ghost.cpp", "aperture_sdf.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return "nvcc"


def build_ref_gpu(force: bool = False):
    """The reference's core library with its CUDA renderers, built for
    sm_103a from the staged sources (about a minute on 16 cores); None when
    the sources are absent."""
    import concurrent.futures as cf
    _stage()
    if not reference_available():
        return None
    src_dir = REFERENCE_ROOT / "ghostlight" / "src"
    third = REFERENCE_ROOT / "ghostlight" / "third_party"
    obj_dir = REF_OUT / "gpu_obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    headers = sorted(src_dir.glob("*.h")) + [REPO / "include" / "ghostlight_gb300.h"]
    cuda_home = pathlib.Path(_nvcc()).resolve().parent.parent
    nv = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
          "--expt-relaxed-constexpr", "--prec-div=false", "--prec-sqrt=false", "--ftz=true",
          "-I", str(src_dir), "-I", str(third), "-I", str(REPO / "include")]
    cxx = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-DREF_GPU",
           "-I", str(src_dir), "-I", str(third), "-I", str(REPO / "include"), "-I", str(cuda_home / "include")]
    jobs = [(nv + ["-c", str(src_dir / f)], src_dir / f) for f in REF_GPU_CU]
    jobs += [(cxx + ["-c", str(src_dir / f)], src_dir / f) for f in REF_GPU_CPP]
    jobs += [(cxx + ["-c", str(HERE / "ref_driver.cpp")], HERE / "ref_driver.cpp")]
    todo, objs = [], []
    for cmd, src in jobs:
        obj = obj_dir / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            todo.append(cmd + ["-o", str(obj)])
    if todo:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 1))) as ex:
            list(ex.map(_run, todo))
    if force or todo or not REF_GPU_LIB.exists():
        tmp = REF_GPU_LIB.with_suffix(".so.tmp%d" % os.getpid())
        _run(["g++", "-shared", "-fopenmp", *map(str, objs), "-o", str(tmp),
              "-L", str(cuda_home / "lib64"), "-L", str(cuda_home / "lib"), "-lcufft", "-lcudart",
              "-Wl,-rpath," + str(cuda_home / "lib64")])
        os.replace(tmp, REF_GPU_LIB)
    return REF_GPU_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    if "--gpu" in sys.argv:
        print(build_ref_gpu(force="--force" in sys.argv))
