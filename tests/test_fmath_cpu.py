"""include/yapt_fmath.h (the deterministic sin, cos, exp, log and pow that the device code and
the oracle share) against float64 references, within the error bounds its header states.

The functions are restated from published methods (Cody-Waite reduction, Taylor and atanh
series) instead of calling CUDA's math library, whose results are not specified bit for bit;
this checks them on a C build of the header over the ranges the tracer uses."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "yapt_fmath.h"
/* reads (x, y) float pairs from stdin; writes sin x, cos x, exp x, log x, pow(x, y) */
int main(void)
{
    float xy[2];
    while (fread(xy, sizeof(float), 2, stdin) == 2)
    {
        float o[5] = {ygm_sinf(xy[0]), ygm_cosf(xy[0]), ygm_expf(xy[0]), ygm_logf(xy[0]), ygm_powf(xy[0], xy[1])};
        fwrite(o, sizeof(float), 5, stdout);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def fmath():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    tmp = tempfile.mkdtemp()
    src, exe = os.path.join(tmp, "fmath.c"), os.path.join(tmp, "fmath")
    with open(src, "w") as f:
        f.write(PROGRAM)
    subprocess.run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), src, "-o", exe, "-lm"],
                   check=True)

    def run(x, y=None):
        y = np.zeros_like(x) if y is None else y
        data = np.stack([x, y], 1).astype(np.float32).tobytes()
        out = subprocess.run([exe], input=data, capture_output=True, check=True).stdout
        return np.frombuffer(out, np.float32).reshape(-1, 5)

    yield run
    shutil.rmtree(tmp, ignore_errors=True)


def ulps(got, ref):
    """|got - ref| in units of the float32 spacing at ref."""
    return np.abs(got.astype(np.float64) - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)


RNG = np.random.default_rng(2024)
N = 200000


def test_sin_and_cos(fmath):
    x = RNG.uniform(-1024.0, 1024.0, N).astype(np.float32)
    o, xd = fmath(x), x.astype(np.float64)
    assert np.abs(o[:, 0] - np.sin(xd)).max() < 1e-7
    assert np.abs(o[:, 1] - np.cos(xd)).max() < 1e-7
    x = RNG.uniform(-np.pi, np.pi, N).astype(np.float32)
    o, xd = fmath(x), x.astype(np.float64)
    assert ulps(o[:, 0], np.sin(xd)).max() <= 2.0
    assert ulps(o[:, 1], np.cos(xd)).max() <= 2.0
    # exact at the origin, as the tracer's rotations expect
    o = fmath(np.array([0.0], np.float32))
    assert o[0, 0] == 0.0 and o[0, 1] == 1.0


def test_exp(fmath):
    x = RNG.uniform(-87.0, 88.0, N).astype(np.float32)
    o = fmath(x)
    assert ulps(o[:, 2], np.exp(x.astype(np.float64))).max() <= 1.0
    assert fmath(np.array([0.0], np.float32))[0, 2] == 1.0


def test_log(fmath):
    x = np.exp(RNG.uniform(np.log(1e-30), np.log(1e30), N)).astype(np.float32)
    o = fmath(x)
    ref = np.log(x.astype(np.float64))
    far = np.abs(ref) > 1e-3  # near x = 1 the result is tiny: judged absolutely below
    assert ulps(o[far, 3], ref[far]).max() <= 2.0
    assert np.abs(o[~far, 3] - ref[~far]).max() < 1e-9
    assert fmath(np.array([1.0], np.float32))[0, 3] == 0.0


def test_pow(fmath):
    x = np.exp(RNG.uniform(np.log(1e-3), np.log(1e3), N)).astype(np.float32)
    y = RNG.uniform(-4.0, 4.0, N).astype(np.float32)
    o = fmath(x, y)
    xd, yd = x.astype(np.float64), y.astype(np.float64)
    err = ulps(o[:, 4], np.power(xd, yd))
    assert np.all(err <= 2.0 + 2.0 * np.abs(yd * np.log(xd)))
    special = fmath(np.array([0.0, 0.0, 1.0, 2.0], np.float32), np.array([2.0, 0.0, 7.5, 0.0], np.float32))[:, 4]
    assert special[0] == 0.0 and special[1] == 1.0 and special[2] == 1.0 and special[3] == 1.0
