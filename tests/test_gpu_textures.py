"""Textures (albedo, normal, occlusion/roughness/metalness, emission; materialsCommon.hlsl:354-397)
and the longitude-latitude environment map (getSkyBoxColor, materialsCommonResources.hlsl:181-224)
on the GPU through the C ABI.

Textures are sampled bilinearly with wrapping in FP32 arithmetic on both sides, so the per-sample
records must match the FP32 oracle within 1e-4 relative like the other integrator tests. The
environment's direction-to-uv mapping calls atan2 and acos (CUDA's and the C library's float
functions), which may differ in the last bit; the 1e-4 bound covers that. BDPT must still agree
with NEE block by block on a textured scene."""
import ctypes as C

import numpy as np
import pytest

from yapt_gb300 import _native as N
from yapt_gb300 import configs
from yapt_gb300.runtime import Context

import test_gpu_bdpt as B
import test_gpu_parity as T

pytestmark = pytest.mark.gpu


def scene(name):
    if name == "textured":
        return configs.textured_box_scene(1), 0.0
    if name == "cube":
        return configs.cube_sky_scene(3), 1.0
    return configs.environment_sky_scene(2), 1.0


@pytest.mark.parametrize("integrator", ["uni", "nee", "bdpt"])
@pytest.mark.parametrize("name", ["textured", "environment", "cube"])
def test_per_sample_parity_with_the_oracle(built, host_luts, integrator, name):
    import pyoracle
    sc, env = scene(name)
    bdpt = integrator == "bdpt"
    p = Context.params(integrator, 48, 40, spp=4, max_depth=8, lambda_range=(380, 780), flags=256, env_scale=env,
                       light_vertices=8 if bdpt else 0)
    with Context(0) as c:
        c.upload_scene(sc)
        gpu = c.render(p, dump=True)
        if not bdpt:
            p.flags = 256 | N.YG_FLAG_MEGAKERNEL
            assert np.array_equal(gpu, c.render(p, dump=True))
            p.flags = 256
    rgb = N.host_table("rgb_to_spd", (380, 780))
    orc = pyoracle.OracleSceneHandle(sc, host_luts, rgb).render(p, precision=32)["records"]
    T.compare(gpu, orc, min_within=0.999)
    if bdpt:
        rel = np.abs(gpu[..., 5:8] - orc[..., 5:8]) / np.maximum(np.abs(orc[..., 5:8]), 1e-6)
        assert float(np.mean(np.all(rel <= T.REL_TOL, axis=-1))) >= 0.999


def test_textures_change_the_image_and_bdpt_agrees_with_nee(built):
    W = H = 32
    with Context(0) as c:
        common = dict(spp=512, max_depth=16, regularize=False, lambda_range=(380, 780), flags=256)
        c.upload_scene(configs.box_scene(1))
        plain = c.render(c.params("nee", W, H, **common), dump=True)
        c.upload_scene(configs.textured_box_scene(1))
        nee = c.render(c.params("nee", W, H, **common), dump=True)
        bd = c.render(c.params("bdpt", W, H, **common), dump=True)
    assert abs(float(nee[..., 6].mean()) / float(plain[..., 6].mean()) - 1.0) > 0.05
    mn, sn = B.block_stats(nee, 8)
    mb, sb = B.block_stats(bd, 8)
    z = np.abs(mb - mn) / np.sqrt(sn ** 2 + sb ** 2 + 1e-30)
    assert abs(float(bd[..., 6].mean()) / float(nee[..., 6].mean()) - 1.0) < B.MEAN_REL_TOL
    assert float(z.max()) < B.Z_MAX, float(z.max())


def test_texture_validation(built):
    with Context(0) as c:
        sc = configs.box_scene(0)
        c.upload_scene(sc)
        tid = C.c_uint32()
        px = np.zeros((2, 2, 4), np.uint8)
        with pytest.raises(N.YaptError):
            N.check(c.lib.yg_upload_texture(c.h, 2, 2, 9, px.ctypes.data_as(C.c_void_p), C.byref(tid)))  # format
        with pytest.raises(N.YaptError):
            N.check(c.lib.yg_upload_texture(c.h, 0, 2, 0, px.ctypes.data_as(C.c_void_p), C.byref(tid)))  # size
        bad = np.full((2, 2, 4), np.nan, np.float32)
        with pytest.raises(N.YaptError):
            N.check(c.lib.yg_upload_texture(c.h, 2, 2, N.YG_TEXTURE_RGBA32_FLOAT, bad.ctypes.data_as(C.c_void_p), C.byref(tid)))
        with pytest.raises(N.YaptError):
            N.check(c.lib.yg_set_environment_texture(c.h, 1))  # no texture uploaded
        sc.materials[0]["albedo_texture"] = 3  # refers to a texture that does not exist
        c.upload_scene(sc)
        with pytest.raises(N.YaptError):
            c.render(c.params("nee", 8, 8, spp=1, flags=256))


@pytest.mark.parametrize("integrator", ["nee", "bdpt"])
def test_gltf_scene_renders_with_parity(built, host_luts, tmp_path, integrator):
    """A scene loaded from glTF (textured cube, emissive lamp, spot light) through the C ABI."""
    import pyoracle
    import gltf_util as G
    from yapt_gb300 import gltf
    path = str(tmp_path / "s.glb")
    G.write_scene(path, binary=True)
    sc = gltf.load(path)
    p = Context.params(integrator, 40, 32, spp=4, max_depth=8, lambda_range=(380, 780), flags=256,
                       light_vertices=8 if integrator == "bdpt" else 0)
    with Context(0) as c:
        c.upload_scene(sc)
        gpu = c.render(p, dump=True)
    rgb = N.host_table("rgb_to_spd", (380, 780))
    orc = pyoracle.OracleSceneHandle(sc, host_luts, rgb).render(p, precision=32)["records"]
    T.compare(gpu, orc, min_within=0.999)
