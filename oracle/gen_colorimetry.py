"""Write ghostlight_gb300/csrc/gl_colorimetry.inc: the CIE 1931 2-degree
standard-observer table (CIE 15:2004, 380-780 nm at 5 nm) and the resolved
input/output colour-space matrices (ACES AP1, sRGB/Rec.709, DCI-P3 D65/D60,
Bradford E->D60) as exact float32 hex literals, read from the reference's
public API (spectral.cpp get_sensor_profile / resolve_*_matrix) so the
spectral tables built from them are bit-identical.  Run once where the
reference checkout exists; the output is committed.
"""
import pathlib
import sys

import numpy as np

REPO = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))
from oracle import ref  # noqa: E402


def hx(v):
    return float(np.float32(v)).hex() + "f"


def main():
    wl, x, y, z = ref.cie_profile()
    lines = ["/* Generated by oracle/gen_colorimetry.py: CIE 1931 2-degree standard",
             " * observer (CIE 15:2004, 5 nm) and resolved colour-space matrices.",
             " * Standard data; values are the float32 ones the flare path uses. */",
             "#define GL_CIE_COUNT %d" % len(wl)]
    for name, arr in (("GL_CIE_WL", wl), ("GL_CIE_X", x), ("GL_CIE_Y", y), ("GL_CIE_Z", z)):
        body = ", ".join(hx(v) for v in arr)
        lines.append("static const float %s[GL_CIE_COUNT] = {%s};" % (name, body))
    outs, ins = [], []
    for cs in range(5):
        _, mo = ref.color_matrices(0, cs)
        outs.append(mo.reshape(-1))
    for cs in range(2):
        mi, _ = ref.color_matrices(cs, 0)
        ins.append(mi.reshape(-1))
    lines.append("static const float GL_OUTPUT_MATRICES[5][9] = {%s};" %
                 ", ".join("{" + ", ".join(hx(v) for v in m) + "}" for m in outs))
    lines.append("static const float GL_INPUT_MATRICES[2][9] = {%s};" %
                 ", ".join("{" + ", ".join(hx(v) for v in m) + "}" for m in ins))
    out = REPO / "ghostlight_gb300" / "csrc" / "gl_colorimetry.inc"
    out.write_text("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
