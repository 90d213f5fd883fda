"""Alpha-tested (cutout) geometry on the GPU through the C ABI: the traversal drops a candidate
hit whose albedo alpha is below the material's cutoff (alphaTestPasses,
hitShadersCommon.hlsl:162-183), reading the triangle's cutout record written by the scene
build. Per-sample parity with the FP32 oracle (1e-4 relative), for every integrator."""
import numpy as np
import pytest

from yapt_gb300 import _native as N
from yapt_gb300 import configs
from yapt_gb300.runtime import Context

import test_gpu_parity as T

pytestmark = pytest.mark.gpu


def params(integrator, W=48, H=40, spp=4):
    return Context.params(integrator, W, H, spp=spp, max_depth=8, lambda_range=(380, 780), flags=256,
                          light_vertices=8 if integrator == "bdpt" else 0)


@pytest.mark.parametrize("integrator", ["uni", "nee", "bdpt"])
def test_per_sample_parity_with_the_oracle(built, host_luts, integrator):
    import pyoracle
    sc = configs.cutout_box_scene(2)
    p = params(integrator)
    with Context(0) as c:
        c.upload_scene(sc)
        gpu = c.render(p, dump=True)
        if integrator != "bdpt":
            p.flags = 256 | N.YG_FLAG_MEGAKERNEL
            assert np.array_equal(gpu, c.render(p, dump=True))
            p.flags = 256
    rgb = N.host_table("rgb_to_spd", (380, 780))
    orc = pyoracle.OracleSceneHandle(sc, host_luts, rgb).render(p, precision=32)["records"]
    T.compare(gpu, orc, min_within=0.999)
    if integrator == "bdpt":
        rel = np.abs(gpu[..., 5:8] - orc[..., 5:8]) / np.maximum(np.abs(orc[..., 5:8]), 1e-6)
        assert float(np.mean(np.all(rel <= T.REL_TOL, axis=-1))) >= 0.999


def test_fully_cut_panels_vanish_and_opaque_panels_block(built):
    p = params("nee")
    with Context(0) as c:
        c.upload_scene(configs.cutout_box_scene(0, cutoff=1.5))
        cut = c.render(p, dump=True)
        sc = configs.cutout_box_scene(0, cutoff=1.5)
        sc.instances = sc.instances[:-2]
        c.upload_scene(sc)
        gone = c.render(p, dump=True)
        c.upload_scene(configs.cutout_box_scene(0, cutoff=0.0))
        opaque = c.render(p, dump=True)
        c.upload_scene(configs.cutout_box_scene(0, cutoff=0.5))
        half = c.render(p, dump=True)
    assert np.array_equal(cut, gone)
    differs = lambda a, b: float(np.mean(np.any(a[..., 1:5] != b[..., 1:5], axis=-1)))
    assert differs(half, opaque) > 0.05 and differs(half, gone) > 0.05


def test_clearing_textures_requires_a_new_build(built):
    from yapt_gb300._native import YaptError
    with Context(0) as c:
        c.upload_scene(configs.cutout_box_scene(0))
        p = params("nee", 16, 16, 1)
        first = c.render(p, dump=True)
        # the cutout records point into texture memory: clearing the textures unbuilds the scene
        N.check(c.lib.yg_clear_textures(c.h))
        with pytest.raises(YaptError):
            c.render(p, dump=True)
        c.upload_scene(configs.cutout_box_scene(0))
        assert np.array_equal(first, c.render(p, dump=True))
    with Context(0) as c:
        # an opaque scene keeps its build when the textures are cleared
        c.upload_scene(configs.box_scene(0))
        p = params("nee", 16, 16, 1)
        a = c.render(p, dump=True)
        N.check(c.lib.yg_clear_textures(c.h))
        assert np.array_equal(a, c.render(p, dump=True))


def cutout_spheres(seed, cutoff, n_spheres=120):
    """``random_shapes_scene`` with every icosphere alpha-tested: spherical uvs and an 8 x 4
    checker of alpha 0 and 1 on each sphere material (the spheres come first, then the ground
    and the lights)."""
    from yapt_gb300 import _native as N
    sc = configs.random_shapes_scene(seed, n_spheres=n_spheres)
    ico = sc.instances[0][1]
    p = sc.meshes[ico]["positions"].astype(np.float64)
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    sc.meshes[ico]["uvs"] = np.stack([np.arctan2(p[:, 2], p[:, 0]) / (2 * np.pi) + 0.5,
                                      np.arccos(np.clip(p[:, 1], -1, 1)) / np.pi], 1).astype(np.float32)
    ij = np.indices((16, 32)).sum(axis=0) // 4
    checker = np.zeros((16, 32, 4), np.uint8)
    checker[..., :3] = 200
    checker[..., 3] = np.where(ij % 2 == 0, 255, 0)
    tex = sc.add_texture(checker, N.YG_TEXTURE_RGBA8_UNORM)
    n = sum(1 for inst in sc.instances if inst[1] == ico)
    for (_, mesh, _, mat) in sc.instances[:n]:
        sc.materials[mat].update(albedo_texture=tex, alpha_cutoff=cutoff)
    return sc, n


def test_cut_spheres_parity_with_the_oracle(built, host_luts):
    import pyoracle
    sc, _ = cutout_spheres(1, 0.5)
    p = Context.params("nee", 128, 128, spp=2, max_depth=12, lambda_range=(380, 780), crop=(32, 40, 64, 48), flags=256)
    with Context(0) as c:
        c.upload_scene(sc)
        gpu = c.render(p, dump=True)
    rgb = N.host_table("rgb_to_spd", (380, 780))
    orc = pyoracle.OracleSceneHandle(sc, host_luts, rgb).render(p, precision=32)["records"]
    T.compare(gpu, orc, min_within=0.999)


def test_fully_cut_spheres_vanish_at_the_bench_scene_size(built):
    """All 500 icospheres of the NEE bench scene (160,008 triangles) cut away: the image equals
    the one without them, which exercises the cutout record offsets over the whole triangle
    array."""
    sc, n = cutout_spheres(0, 1.5, n_spheres=500)
    p = Context.params("nee", 256, 256, spp=2, max_depth=12, lambda_range=(380, 780), flags=256)
    with Context(0) as c:
        c.upload_scene(sc)
        cut = c.render(p, dump=True)
        sc.instances = sc.instances[n:]
        c.upload_scene(sc)
        gone = c.render(p, dump=True)
    same = float(np.mean(np.all(cut == gone, axis=-1)))
    assert same >= 0.9999, same
    assert np.any(gone[..., 1:5] > 0)
