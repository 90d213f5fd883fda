"""The glTF loader (the reference's scene_loader.py restated over this build's scene), on the CPU:
the PNG decoder against an encoder that uses all five row filters, and a written scene whose
hierarchy, camera, light, materials (factors, textures, extensions) and meshes must come back."""
import numpy as np
import pytest

import gltf_util as G
from yapt_gb300 import _native as N
from yapt_gb300 import gltf


@pytest.mark.parametrize("channels", [1, 2, 3, 4])
def test_png_roundtrip(channels):
    px = np.random.default_rng(channels).integers(0, 256, (11, 7, channels)).astype(np.uint8)
    out = gltf.decode_png(G.encode_png(px))
    rgb = px[..., :1].repeat(3, 2) if channels <= 2 else px[..., :3]
    alpha = px[..., -1:] if channels in (2, 4) else np.full((11, 7, 1), 255, np.uint8)
    assert np.array_equal(out, np.concatenate([rgb, alpha], 2))


@pytest.mark.parametrize("binary", [False, True])
def test_scene_loads(tmp_path, binary):
    path = str(tmp_path / ("s.glb" if binary else "s.gltf"))
    tex = G.write_scene(path, binary)
    sc = gltf.load(path)
    assert len(sc.instances) == 3 and len(sc.meshes) == 3
    # the cube: parent T * R(45 deg about y) * child S(0.5)
    o2w = sc.instances[0][0]
    c, s = np.cos(np.pi / 4), np.sin(np.pi / 4)
    want = np.array([[c, 0, s, 0.2], [0, 1, 0, 0.5], [-s, 0, c, -0.1], [0, 0, 0, 1]]) @ np.diag([0.5, 0.5, 0.5, 1])
    np.testing.assert_allclose(o2w, want, atol=1e-6)
    p, n, uv, idx = G.cube_arrays()
    m = sc.meshes[sc.instances[0][1]]
    assert np.array_equal(m["positions"], p) and np.array_equal(m["indices"], idx) and np.array_equal(m["uvs"], uv)
    t = m["tangents"]
    np.testing.assert_allclose(np.abs(np.sum(t[:, :3] * n, 1)), 0, atol=1e-6)  # tangents orthogonal to the normals
    np.testing.assert_allclose(np.linalg.norm(t[:, :3], axis=1), 1, atol=1e-6)
    cube = sc.materials[sc.instances[0][3]]
    assert cube["albedo"] == (0.8, 0.6, 0.4) and cube["metalness"] == 0.0 and cube["roughness"] == 0.5
    assert cube["clear_coat_amount"] == 0.7 and cube["clear_coat_ior"] == 1.5
    w, h, fmt, px = sc.textures[cube["albedo_texture"] - 1]
    assert fmt == N.YG_TEXTURE_RGBA8_SRGB and np.array_equal(px, tex)
    floor = sc.materials[sc.instances[1][3]]
    assert floor["material_mask"] & N.YG_MATERIAL_TWO_SIDED
    glow = sc.materials[sc.instances[2][3]]
    np.testing.assert_allclose(glow["emissive"], (4.0, 3.6, 3.2))
    np.testing.assert_allclose(sc.instances[2][0][:3, 3], (0, 2.5, 0))
    # camera 15 degrees down from (0, 1.5, 4); spot light pointing straight down
    np.testing.assert_allclose(sc.camera.world[:3, 3], (0, 1.5, 4), atol=1e-6)
    assert abs(sc.camera.fovy - 0.9) < 1e-9
    L = sc.punctual_lights[0]
    assert L["type"] == N.YG_LIGHT_SPOT
    np.testing.assert_allclose(L["direction"], (0, -1, 0), atol=1e-6)
    np.testing.assert_allclose(L["intensity"], (3.0, 2.7, 2.1))
    assert abs(L["cos_inner"] - np.cos(0.3)) < 1e-9 and abs(L["cos_outer"] - np.cos(0.6)) < 1e-9


def test_unsupported_images_raise(tmp_path):
    import json
    path = str(tmp_path / "s.gltf")
    G.write_scene(path)
    g = json.load(open(path))
    g["images"] = [{"uri": "data:image/jpeg;base64,/9j/4AAQ", "mimeType": "image/jpeg"}]
    json.dump(g, open(path, "w"))
    with pytest.raises(ValueError):
        gltf.load(path)
