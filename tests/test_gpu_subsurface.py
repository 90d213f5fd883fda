"""Subsurface scattering (the Christensen-Burley BSSRDF of subsurface.hlsl) on the device.

Per-sample parity with the FP32 oracle for the unidirectional and NEE integrators on a box
whose blocks and three icospheres scatter below their surfaces: probe rays against the
entry instance, the exit point's light connection and exit lobe. The megakernel and the
wavefront give the same samples. The bidirectional integrator's subsurface vertices are
covered in test_gpu_bdpt.py (per-sample parity and agreement with NEE).
"""
import numpy as np
import pytest

from yapt_gb300 import configs
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4


def compare(gpu, cpu, min_within=0.9995):
    assert np.array_equal(gpu[..., 0], cpu[..., 0]), "hero wavelengths differ"
    L_gpu, L_cpu = gpu[..., 1:5], cpu[..., 1:5]
    rel = np.abs(L_gpu - L_cpu) / np.maximum(np.abs(L_cpu), 1e-6)
    within = float(np.mean(np.all(rel <= REL_TOL, axis=-1)))
    assert np.all(np.isfinite(L_gpu))
    assert within >= min_within, within
    return within


@pytest.mark.parametrize("integrator", ["uni", "nee"])
def test_subsurface_per_sample_parity(built, host_luts, integrator):
    import pyoracle
    sc = configs.subsurface_box_scene(0)
    p = Context.params(integrator, 64, 64, spp_start=3, spp=4, max_depth=8, lambda_range=(380, 780), flags=256)
    with Context(0) as c:
        c.upload_scene(sc)
        gpu = c.render(p, dump=True)
    h = pyoracle.OracleSceneHandle(sc, host_luts, rgb_to_spd=N.host_table("rgb_to_spd", (380, 780)))
    cpu = h.render(p, precision=32)["records"]
    compare(gpu, cpu)


def test_subsurface_megakernel_equals_wavefront(built):
    sc = configs.subsurface_box_scene(1)
    with Context(0) as c:
        c.upload_scene(sc)
        a = c.render(c.params("nee", 48, 40, spp=3, max_depth=8, lambda_range=(380, 780), flags=256), dump=True)
        b = c.render(c.params("nee", 48, 40, spp=3, max_depth=8, lambda_range=(380, 780),
                              flags=256 | N.YG_FLAG_MEGAKERNEL), dump=True)
    assert np.array_equal(a, b)
