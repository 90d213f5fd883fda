"""Alpha-tested (cutout) geometry in the oracle: alphaTestPasses (hitShadersCommon.hlsl:162-183)
drops a candidate hit where the albedo alpha at the hit's uv is below the material's cutoff,
for camera, bounce and shadow rays alike (PROCEED_ALPHA_TESTED, rayHitDefault.hlsl:101,130;
BDPTCommon.hlsl:1157).

A cutoff above every alpha cuts a panel away completely, so the image must equal, sample by
sample, the scene without the panels; a cutoff of 0 turns the test off (the panels are opaque).

Also the cube-map environment (getSkyBoxColor with ENVIRONMENT_TYPE_CUBE) against a
longitude-latitude map of the same constant colour."""
import numpy as np
import pytest

from yapt_gb300 import _native as N
from yapt_gb300 import configs
from yapt_gb300.runtime import Context


def render(sc, integrator, host_luts, precision=32):
    import pyoracle
    p = Context.params(integrator, 24, 20, spp=2, max_depth=6, lambda_range=(380, 780), flags=256,
                       light_vertices=4 if integrator == "bdpt" else 0)
    rgb = N.host_table("rgb_to_spd", (380, 780))
    return pyoracle.OracleSceneHandle(sc, host_luts, rgb).render(p, precision=precision)["records"]


def without_panels(sc):
    sc.instances = sc.instances[:-2]
    return sc


@pytest.mark.parametrize("integrator", ["uni", "nee", "bdpt"])
def test_fully_cut_panels_vanish(built, host_luts, integrator):
    cut = render(configs.cutout_box_scene(0, cutoff=1.5), integrator, host_luts)
    ref = render(without_panels(configs.cutout_box_scene(0, cutoff=1.5)), integrator, host_luts)
    assert np.array_equal(cut, ref)
    assert np.any(ref[..., 1:5] > 0)


def test_cutouts_change_the_image_between_opaque_and_absent(built, host_luts):
    half = render(configs.cutout_box_scene(0, cutoff=0.5), "nee", host_luts)
    opaque = render(configs.cutout_box_scene(0, cutoff=0.0), "nee", host_luts)
    gone = render(without_panels(configs.cutout_box_scene(0, cutoff=0.5)), "nee", host_luts)
    differs = lambda a, b: float(np.mean(np.any(a[..., 1:5] != b[..., 1:5], axis=-1)))
    # some samples see through the holes (as without the panels), others hit the screen
    assert differs(half, opaque) > 0.05
    assert differs(half, gone) > 0.05
    # the hero wavelengths do not depend on the geometry
    assert np.array_equal(half[..., 0], opaque[..., 0])


def test_fp32_and_fp64_oracles_agree_on_cutouts(built, host_luts):
    sc = configs.cutout_box_scene(1)
    a = render(sc, "nee", host_luts, 32)
    b = render(sc, "nee", host_luts, 64)
    rel = np.abs(a[..., 1:5] - b[..., 1:5]) / np.maximum(np.abs(b[..., 1:5]), 1e-3)
    assert float(np.mean(np.all(rel < 1e-2, axis=-1))) > 0.98


def test_scene_carries_the_cutout_materials():
    sc = configs.cutout_box_scene(0)
    mats = sc.materials[-2:]
    assert all(m["alpha_cutoff"] == 0.5 and m["albedo_texture"] > 0 for m in mats)
    assert all(sc.meshes[mesh].get("uvs") is not None for (_, mesh, _, _) in sc.instances[-2:])


def test_constant_cube_map_matches_a_constant_longitude_latitude_map(built, host_luts):
    """A cube map and a longitude-latitude map of one colour light the scene alike (up to the
    last-bit rounding of the bilinear weights); a cube map read from the wrong face or texel
    would not."""
    colour = np.array([0.7, 0.45, 0.3, 1.0], np.float32)
    cube = configs.cube_sky_scene(1, face=8)
    cube.textures[-1] = (8, 48, N.YG_TEXTURE_RGBA32_FLOAT, np.tile(colour, (48, 8, 1)))
    flat = configs.environment_sky_scene(1)
    flat.textures[-1] = (16, 8, N.YG_TEXTURE_RGBA32_FLOAT, np.tile(colour, (8, 16, 1)))
    import pyoracle
    p = Context.params("nee", 24, 20, spp=2, max_depth=6, lambda_range=(380, 780), flags=256, env_scale=1.0)
    rgb = N.host_table("rgb_to_spd", (380, 780))
    a = pyoracle.OracleSceneHandle(cube, host_luts, rgb).render(p, precision=32)["records"]
    b = pyoracle.OracleSceneHandle(flat, host_luts, rgb).render(p, precision=32)["records"]
    assert np.any(b[..., 1:5] > 0)
    assert np.allclose(a[..., 1:5], b[..., 1:5], rtol=1e-5, atol=1e-7)
