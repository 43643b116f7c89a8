"""Recipe: stage the reference's flare-path sources for the reference arm.

The reference (JaydenB/ghostlight) has no installable package at its root (no
setup.py or pyproject.toml), and its Python package under
ghostlight/bindings/python builds its extension with CMake for the building
host's architecture, which does not run on an Arm GPU host.  The reference arm
and the oracle's reference builds (oracle/build.py) therefore compile the
reference's own C++/CUDA sources directly, on whichever host they run.  This
recipe copies those sources, unmodified, from a reference checkout into the
git-ignored ``baseline/_ref/`` so that they travel with the working tree:

  baseline/_ref/ghostlight/src/           every source of the core library
  baseline/_ref/ghostlight/third_party/   the vendored JSON reader it includes

The checkout is taken from the first argument, else from
``GHOSTLIGHT_REFERENCE``, else from the checkout path of the build container.
Nothing here is product code and nothing is committed.

    python oracle/stage_ref.py [/path/to/ghostlight-checkout]
"""
from __future__ import annotations

import os
import pathlib
import shutil
import sys

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent
STAGE = REPO / "baseline" / "_ref"
DIRS = ("ghostlight/src", "ghostlight/third_party")


def checkout(path: str | None = None) -> pathlib.Path:
    return pathlib.Path(path or os.environ.get("GHOSTLIGHT_REFERENCE") or "/root/reference")


def stage(path: str | None = None) -> pathlib.Path | None:
    """Copy the sources when the checkout exists and the stage is missing or
    older; return the stage root, or None when neither is available."""
    root = checkout(path)
    if not (root / "ghostlight" / "src" / "trace.cpp").exists():
        return STAGE if (STAGE / "ghostlight" / "src" / "trace.cpp").exists() else None
    for d in DIRS:
        src, dst = root / d, STAGE / d
        for f in src.rglob("*"):
            if not f.is_file():
                continue
            out = dst / f.relative_to(src)
            if out.exists() and out.stat().st_mtime >= f.stat().st_mtime and out.stat().st_size == f.stat().st_size:
                continue
            out.parent.mkdir(parents=True, exist_ok=True)
            shutil.copy2(f, out)
    return STAGE


if __name__ == "__main__":
    print(stage(sys.argv[1] if len(sys.argv) > 1 else None))
