"""Build recipe of libghostlight_gb300.so (in-tree, sm_103a only).

Each translation unit gets the floating-point mode its job needs:

* gl_host.cpp  — host builders; -ffp-contract=off so float arithmetic is the
  reference host build's on x86-64 and aarch64 alike.
* gl_filter.cu — the culler; IEEE-exact device arithmetic (-fmad=false,
  IEEE division/sqrt, no flush-to-zero) so its decisions can be re-checked
  bit-for-bit on the host.
* the render / starburst / convolution units — throughput flags
  (flush-to-zero, approximate division and square root), the reference GPU
  build's own mode (ghostlight/CMakeLists.txt:97-109).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libghostlight_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I", str(REPO / "include"), "-I", str(CSRC)]
FAST = ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
EXACT = ["-fmad=false", "-ftz=false", "-prec-div=true", "-prec-sqrt=true"]

UNITS = {
    "gl_host.cpp": [],
    "gl_setup.cpp": [],
    "gl_coat.cpp": [],
    "gl_filter.cu": EXACT,
    "gl_ghost.cu": FAST,
    "gl_mdft.cu": FAST,
    "gl_conv.cu": FAST,
    "gl_serve.cu": FAST,
    "gl_veil.cu": FAST,
    "gl_psf.cu": FAST,
    "gl_sprite.cu": FAST,
}
# Occupancy target of the render kernel (CTAs of 128 threads per SM); an
# environment override lets a tuning sweep rebuild with another value.
for _var in ("GL_RENDER_MIN_BLOCKS",):
    if os.environ.get(_var):
        UNITS["gl_ghost.cu"] = UNITS["gl_ghost.cu"] + ["-D%s=%d" % (_var, int(os.environ[_var]))]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _compile(src: pathlib.Path, extra, verbose=False):
    obj = BUILD / (src.name + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *HOST_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "cu", *ARCH, *COMMON, *HOST_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src.name, r.stdout, r.stderr))
    return obj, r.stderr


def _deps():
    return [CSRC / u for u in UNITS] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list(CSRC.glob("*.inc")) + [REPO / "include" / "ghostlight_gb300.h", pathlib.Path(__file__)]


STAMP = BUILD / "flags.txt"


def _flags_stamp() -> str:
    """The per-unit flags the library was built with: a change (an
    environment override) forces a rebuild even when no source changed."""
    return "\n".join("%s %s" % (u, " ".join(f)) for u, f in sorted(UNITS.items()))


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    stamp = _flags_stamp()
    if not force and LIB.exists() and STAMP.exists() and STAMP.read_text() == stamp:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in _deps()):
            return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(UNITS))) as ex:
        futs = [ex.submit(_compile, CSRC / u, f, verbose) for u, f in UNITS.items()]
        results = [f.result() for f in futs]
    if verbose:
        for _, log in results:
            print(log)
    tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
    cmd = [nvcc(), *ARCH, "-shared", *[str(o) for o, _ in results], "-o", str(tmp), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    STAMP.write_text(stamp)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
