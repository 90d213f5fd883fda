"""Punctual lights (point, spot, directional; LightManager / lightSampling.hlsl:210-358) on
the GPU through the C ABI.

They have no geometry, so the path integrators sample them explicitly: NEE picks from the
one alias table over all lights, the unidirectional integrator from the table over the
punctual lights alone (rayHitDefault.hlsl:26-81); BDPT starts light subpaths at them
(samplePunctualLightEmission, BDPTCommon.hlsl:697-760). Checks: per-sample parity with the
FP32 oracle within 1e-4 relative (the same tolerance as the other integrator tests), the
wavefront and the megakernel giving identical samples, uni and BDPT agreeing with NEE block
by block within their combined standard error (all unbiased for the same image), and the
boundary's validation."""
import ctypes as C

import numpy as np
import pytest

from yapt_gb300 import _native as N
from yapt_gb300 import configs
from yapt_gb300.runtime import Context

import test_gpu_bdpt as B
import test_gpu_parity as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("integrator", ["uni", "nee", "bdpt"])
@pytest.mark.parametrize("area_light", [True, False])
def test_per_sample_parity_with_the_oracle(built, host_luts, integrator, area_light):
    import pyoracle
    sc = configs.punctual_box_scene(3, area_light=area_light)
    bdpt = integrator == "bdpt"
    p = Context.params(integrator, 48, 40, spp=4, max_depth=8, lambda_range=(380, 780), flags=256,
                       light_vertices=8 if bdpt else 0)
    with Context(0) as c:
        c.upload_scene(sc)
        gpu = c.render(p, dump=True)
        if not bdpt:
            p.flags = 256 | N.YG_FLAG_MEGAKERNEL
            mega = c.render(p, dump=True)
            p.flags = 256
            assert np.array_equal(gpu, mega)
    rgb = N.host_table("rgb_to_spd", (380, 780))  # the lights' intensities are RGB
    orc = pyoracle.OracleSceneHandle(sc, host_luts, rgb).render(p, precision=32)["records"]
    T.compare(gpu, orc, min_within=0.999)
    if bdpt:  # light-tracing splats (point and spot light paths reach the camera) land in XYZ
        rel = np.abs(gpu[..., 5:8] - orc[..., 5:8]) / np.maximum(np.abs(orc[..., 5:8]), 1e-6)
        assert float(np.mean(np.all(rel <= T.REL_TOL, axis=-1))) >= 0.999


@pytest.mark.parametrize("other", ["uni", "bdpt"])
@pytest.mark.parametrize("area_light", [True, False])
def test_integrators_estimate_the_same_image(built, other, area_light):
    sc = configs.punctual_box_scene(1, area_light=area_light)
    W = H = 32
    with Context(0) as c:
        c.upload_scene(sc)
        common = dict(spp=512, max_depth=16, regularize=False, lambda_range=(380, 780), flags=256)
        oth = c.render(c.params(other, W, H, **common), dump=True)
        nee = c.render(c.params("nee", W, H, **common), dump=True)
    assert np.all(np.isfinite(oth))
    mu, su = B.block_stats(oth, 8)
    mn, sn = B.block_stats(nee, 8)
    z = np.abs(mu - mn) / np.sqrt(su ** 2 + sn ** 2 + 1e-30)
    gu, gn = float(oth[..., 6].mean()), float(nee[..., 6].mean())
    assert gn > 0
    assert abs(gu - gn) / gn < B.MEAN_REL_TOL, (gu, gn)
    assert float(z.max()) < B.Z_MAX, float(z.max())


def test_lights_update_without_a_rebuild_and_validation(built):
    sc = configs.punctual_box_scene(2, area_light=False)
    with Context(0) as c:
        c.upload_scene(sc)
        p = c.params("nee", 24, 24, spp=2, max_depth=6, lambda_range=(380, 780), flags=256)
        a = c.render(p, dump=True)
        # brighter point light: the table is rebuilt on the spot and the image changes
        sc.punctual_lights[0]["intensity"] = (3.0, 3.0, 3.0)
        arr = sc.punctual_structs()
        N.check(c.lib.yg_set_punctual_lights(c.h, arr, len(sc.punctual_lights)))
        b = c.render(p, dump=True)
        assert not np.array_equal(a, b)
        bad = (N.PunctualLight * 1)()
        bad[0].type = 9
        with pytest.raises(N.YaptError):
            N.check(c.lib.yg_set_punctual_lights(c.h, bad, 1))
        bad[0].type = N.YG_LIGHT_SPOT  # zero direction
        with pytest.raises(N.YaptError):
            N.check(c.lib.yg_set_punctual_lights(c.h, bad, 1))
        bd = c.render(c.params("bdpt", 24, 24, spp=2, max_depth=6, lambda_range=(380, 780), flags=256), dump=True)
        assert float(bd[..., 6].sum()) > 0.0  # BDPT light subpaths start at the punctual lights
        N.check(c.lib.yg_set_punctual_lights(c.h, None, 0))
        dark = c.render(p, dump=True)
        assert float(dark[..., 6].sum()) == 0.0  # no area light and no punctual light left


def test_py_yapt_lights_render(built, py_yapt):
    import pyyapt_util as U
    Y = py_yapt
    r = Y.Renderer()
    r.init()
    r.getRendererVariable("Generic.RenderResolution").setFromIntArray([24, 24])
    r.getRendererVariable("RenderPipeline").setSelectedOption(1)
    r.getRendererVariable("World.EnvIntensityScale").setFromFloatArray([0.0])
    sc = Y.Scene()
    sc.init(r)
    box = U.box(1)
    meshes, mats, objs = U.build_scene(Y, r, sc, box)
    sc.update(0.0, 2)
    base = float(np.frombuffer(r.readback(Y.ReadbackTarget.FilmXYZ).getData().getBytes(), np.float32)[1::4].mean())
    light = sc.createLight("spot", Y.Light.LightType.SPOT)
    light.setIntensity(4.0)
    light.setSpotConeAngles(0.3, 0.6)
    # under the ceiling, aimed at the floor (the light emits along its forward axis)
    light.getTransform().lookAt(Y.vec3([0.5, 0.9, 0.5]), Y.vec3([0.5, 0.0, 0.55]), Y.vec3([0.0, 0.0, 1.0]))
    assert abs(light.getTransform().forward()[1] + 1.0) < 0.01
    sc.update(0.0, 2)
    assert r.getAccumulatedFrames() == 2  # the new light restarted the accumulation
    lit = float(np.frombuffer(r.readback(Y.ReadbackTarget.FilmXYZ).getData().getBytes(), np.float32)[1::4].mean())
    assert lit > base
    sc.shutdown()
    r.shutdown()
