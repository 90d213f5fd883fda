"""Write the golden fixtures under tests/golden from the reference checkout.

``sobol_matrices_dims0_255.u32``: the reference's own Sobol generator matrices
(``Source/Common/inc/Math/SobolMatrices.h:5-7``, produced there by
``Tools/generate_sobol_matrices.py``) for dimensions 0..255, 32 little-endian
uint32 columns per dimension. The library derives its matrices from the Joe & Kuo
direction numbers itself; this fixture pins that derivation to the reference's table.

Usage: ``python tests/golden/make_golden.py <reference checkout>``.
"""
import os
import re
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(root):
    text = open(os.path.join(root, "Source/Common/inc/Math/SobolMatrices.h")).read()
    body = text.split("SOBOL_MATRICES[SOBOL_MATRIX_COUNT * SOBOL_MATRIX_ROW_COUNT] =", 1)[1]
    vals = [int(v, 16) for v in re.findall(r"0x([0-9a-fA-F]+)u", body)]
    assert len(vals) == 513 * 32, len(vals)
    out = os.path.join(HERE, "sobol_matrices_dims0_255.u32")
    with open(out, "wb") as f:
        f.write(struct.pack("<%dI" % (256 * 32), *vals[: 256 * 32]))
    print(out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["YAPT_REFERENCE_ROOT"])
