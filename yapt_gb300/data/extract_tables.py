"""Regenerate the published data tables this package ships under ``yapt_gb300/data``.

The tables are standard published data, not code:

* ``cie1931_2deg_d65_1nm.txt`` -- CIE 1931 2-degree colour-matching functions and
  the CIE standard illuminant D65, 360..830 nm at 1 nm (471 rows). These are the
  same values the reference renderer ships in
  ``Source/Renderer/inc/Renderer/Shared/Utility/SpectralData.h:10-268``; spectral
  film parity needs the identical numbers.
* ``joe_kuo_6_21201_first256.txt`` -- the first 256 rows of the Joe & Kuo (2008)
  Sobol initial direction numbers ``new-joe-kuo-6.21201`` (dimensions 2..257 of
  their numbering). The reference derives its generator matrices from this file
  (``Tools/generate_sobol_matrices.py:37-53``); only 256 dimensions are used per
  sample (``Source/Renderer/shaders/raytracing/raytraceCommon.hlsl:11-12``).

Usage: ``python yapt_gb300/data/extract_tables.py <reference checkout>``.
The outputs are committed; nothing at run time reads the reference checkout.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _parse_array(text, name):
    m = re.search(r"constexpr double %s\[[^\]]*\]\s*=\s*\{(.*?)\};" % re.escape(name), text, re.S)
    if not m:
        raise RuntimeError("array %s not found" % name)
    vals = [float(v) for v in re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", m.group(1))]
    return vals


def extract_cie(ref_root):
    path = os.path.join(ref_root, "Source/Renderer/inc/Renderer/Shared/Utility/SpectralData.h")
    text = open(path).read()
    x = _parse_array(text, "c_cieDeg2X")
    y = _parse_array(text, "c_cieDeg2Y")
    z = _parse_array(text, "c_cieDeg2Z")
    d65 = _parse_array(text, "c_cieD65StandardIllum")
    assert len(x) == len(y) == len(z) == len(d65) == 471, (len(x), len(y), len(z), len(d65))
    out = os.path.join(HERE, "cie1931_2deg_d65_1nm.txt")
    with open(out, "w") as f:
        f.write("# CIE 1931 2-degree colour matching functions and CIE D65 SPD, 1 nm steps\n")
        f.write("# lambda_nm xbar ybar zbar d65\n")
        for i in range(471):
            f.write("%d %.12g %.12g %.12g %.12g\n" % (360 + i, x[i], y[i], z[i], d65[i]))
    return out


def extract_joe_kuo(ref_root, count=256):
    path = os.path.join(ref_root, "Tools/new-joe-kuo-6.21201")
    out = os.path.join(HERE, "joe_kuo_6_21201_first256.txt")
    rows = []
    with open(path) as f:
        header = None
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            if header is None:
                header = s
                continue
            rows.append(s)
            if len(rows) == count:
                break
    with open(out, "w") as f:
        f.write("# First %d rows of the Joe & Kuo Sobol direction numbers new-joe-kuo-6.21201\n" % count)
        f.write("# (S. Joe and F. Y. Kuo, SIAM J. Sci. Comput. 30, 2635-2654, 2008)\n")
        f.write("# columns: d s a m_i...\n")
        for r in rows:
            f.write(" ".join(r.split()) + "\n")
    return out


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("YAPT_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: extract_tables.py <reference checkout>")
    print(extract_cie(root))
    print(extract_joe_kuo(root))
