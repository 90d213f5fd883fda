"""py_yapt on the GPU: a scene built through the reference's Python surface renders the same
film, bit for bit, as the C ABI given the records py_yapt committed (the tolerance is zero:
both go through yg_render with identical inputs); frames accumulate in sample order, so
three frames then two equal five in one call; changes restart the accumulation."""
import ctypes as C

import numpy as np
import pytest

import pyyapt_util as U
from yapt_gb300 import _native as N
from yapt_gb300.runtime import Context

pytestmark = pytest.mark.gpu


def setup_renderer(Y, w=48, h=40, pipeline=1):
    r = Y.Renderer()
    r.init()
    r.getRendererVariable("Generic.RenderResolution").setFromIntArray([w, h])
    r.getRendererVariable("RenderPipeline").setSelectedOption(pipeline)
    r.getRendererVariable("Generic.MaxDepth").setFromIntArray([6])
    r.getRendererVariable("Generic.SpectralRange").setFromFloatArray([380.0, 780.0])
    r.getRendererVariable("World.EnvIntensityScale").setFromFloatArray([0.0])
    return r


def film_of(Y, r):
    rb = r.readback(Y.ReadbackTarget.FilmXYZ)
    assert rb.isReady()
    d = rb.getData()
    assert d.getFormat() == Y.ResourceFormat.RGBA32_SFLOAT and d.getTexelSizeInBytes() == 16
    a = np.frombuffer(d.getBytes(), np.float32).reshape(d.getHeight(), d.getWidth(), 4)
    rb.release()
    assert rb.getState() == Y.ReadbackState.Freed
    return a


def c_abi_film(Y, records, meshes, w, h, spp, integrator="nee"):
    """Renders the committed records through the C ABI on a context of its own."""
    inst = (N.Instance * (len(records["instances"]) // C.sizeof(N.Instance))).from_buffer_copy(records["instances"])
    mats = (N.Material * (len(records["materials"]) // C.sizeof(N.Material))).from_buffer_copy(records["materials"])
    spec = np.frombuffer(records["spectra"], np.float32)
    cam = N.Camera.from_buffer_copy(records["camera"])
    with Context(0) as c:
        lib, h_ = c.lib, c.h
        for m in meshes:
            d = m._decoded()
            pos = np.array(d["positions"], np.float32)
            nrm = np.array(d["normals"], np.float32)
            tan = np.array(d["tangents"], np.float32) if d["tangents"] else None
            idx = np.array(d["indices"], np.uint32)
            sub = np.array(d["submeshes"], np.uint32)
            desc = N.MeshDesc()
            desc.positions = pos.ctypes.data_as(C.POINTER(C.c_float))
            desc.normals = nrm.ctypes.data_as(C.POINTER(C.c_float))
            desc.tangents = tan.ctypes.data_as(C.POINTER(C.c_float)) if tan is not None else None
            desc.uvs = None
            desc.vertex_count = len(pos) // 3
            desc.indices = idx.ctypes.data_as(C.c_void_p)
            desc.index_count = len(idx)
            desc.index_bits = 32
            desc.submesh_ranges = sub.ctypes.data_as(C.POINTER(C.c_uint32))
            desc.submesh_count = len(sub) // 2
            mid = C.c_uint32()
            N.check(lib.yg_upload_mesh(h_, C.byref(desc), C.byref(mid)))
        N.check(lib.yg_upload_materials(h_, mats, len(mats)))
        if len(spec):
            N.check(lib.yg_upload_spectra(h_, spec.ctypes.data_as(C.POINTER(C.c_float)), len(spec) // 81, 81, 380.0, 780.0))
        N.check(lib.yg_set_instances(h_, inst, len(inst)))
        N.check(lib.yg_set_camera(h_, C.byref(cam)))
        N.check(lib.yg_build_scene(h_))
        c.film_clear(w, h)
        c.render(c.params(integrator, w, h, spp_start=0, spp=spp, max_depth=6, lambda_range=(380, 780)))
        xyz, cnt = c.film()
    return xyz, cnt


def used_meshes(objs):
    out, seen = [], set()
    for o in objs:
        m = o.getMesh()
        if m.getName() not in seen:
            seen.add(m.getName())
            out.append(m)
    return out


def test_box_scene_through_py_yapt_equals_the_c_abi(built, py_yapt):
    Y = py_yapt
    W, H = 48, 40
    r = setup_renderer(Y, W, H)
    sc = Y.Scene()
    sc.init(r)
    meshes, mats, objs = U.build_scene(Y, r, sc, U.box(1))
    sc.update(0.016, 3)
    sc.update(0.016, 2)
    assert r.getAccumulatedFrames() == 5
    got = film_of(Y, r)
    rec = sc._debugRecords()
    assert len(rec["instances"]) // C.sizeof(N.Instance) == 8  # 5 wall submeshes, 2 cubes, 1 light
    xyz, cnt = c_abi_film(Y, rec, used_meshes(objs), W, H, 5)
    assert np.all(got[..., 3] == 5) and np.array_equal(cnt, got[..., 3])
    assert np.array_equal(xyz, got[..., :3]), float(np.abs(xyz - got[..., :3]).max())
    assert float(got[..., 1].mean()) > 0.0
    sc.shutdown()
    r.shutdown()


def test_accumulation_restarts_and_readback_targets(built, py_yapt):
    Y = py_yapt
    r = setup_renderer(Y, 32, 24)
    sc = Y.Scene()
    sc.init(r)
    meshes, mats, objs = U.build_scene(Y, r, sc, U.box(2))
    sc.update(0.0, 2)
    assert r.getAccumulatedFrames() == 2
    sc.update(0.0)
    assert r.getAccumulatedFrames() == 3
    mats[0].setAlbedo(Y.vec3([0.2, 0.3, 0.4]))  # any change restarts
    sc.update(0.0)
    assert r.getAccumulatedFrames() == 1
    objs[-1].getTransform().addTranslation(Y.vec3([0.0, -0.001, 0.0]))
    sc.update(0.0)
    assert r.getAccumulatedFrames() == 1
    r.getRendererVariable("Generic.Seed").setFromIntArray([7])
    sc.update(0.0)
    assert r.getAccumulatedFrames() == 1
    fc = r.readback(Y.ReadbackTarget.FinalColor).getData()
    assert fc.getFormat() == Y.ResourceFormat.RGBA8_UNORM and fc.getSizeInBytes() == 32 * 24 * 4
    assert fc.getRowPitchInBytes() == 32 * 4
    assert r.readback(Y.ReadbackTarget.Features).getState() == Y.ReadbackState.Failed  # features off
    r.getRendererVariable("Generic.Features").setSelectedOption(1)
    sc.update(0.0, 2)
    f = r.readback(Y.ReadbackTarget.Features).getData()
    assert f.getDepthOrSlices() == 2
    feats = np.frombuffer(f.getBytes(), np.float32).reshape(2, 24, 32, 4)
    assert np.all(feats[0, ..., 3] > 0)  # depth of first hits inside the closed box
    rgb = np.frombuffer(r.readback(Y.ReadbackTarget.FilmRGB).getData().getBytes(), np.float32).reshape(24, 32, 4)
    xyz = film_of(Y, r)
    M = np.array([[3.2406, -1.5372, -0.4986], [-0.9689, 1.8758, 0.0415], [0.0557, -0.2040, 1.0570]], np.float32)
    np.testing.assert_allclose(rgb[..., :3], xyz[..., :3] @ M.T, rtol=1e-5, atol=1e-6)
    # dropping the last Python reference to a render object removes it from the scene
    n_before = len(sc._debugRecords()["instances"])
    del objs[-1]
    assert len(sc._debugRecords()["instances"]) < n_before
    sc.shutdown()
    r.shutdown()


def test_bdpt_pipeline_and_unsupported_features_raise(built, py_yapt):
    Y = py_yapt
    r = setup_renderer(Y, 24, 24, pipeline=2)
    r.getRendererVariable("BDPT.LightVertices").setFromIntArray([6])
    sc = Y.Scene()
    sc.init(r)
    meshes, mats, objs = U.build_scene(Y, r, sc, U.box(3))
    sc.update(0.0, 2)
    xyz = film_of(Y, r)
    assert np.all(np.isfinite(xyz)) and float(xyz[..., 1].mean()) > 0.0
    light = sc.createLight("point", Y.Light.LightType.POINT)
    light.getTransform().setTranslation(Y.vec3([0.5, 0.8, 0.5]))
    sc.update(0.0)  # BDPT light subpaths from the point light
    assert r.getAccumulatedFrames() == 1
    light.setIntensity(0.0)  # a dark light is left out
    sc.update(0.0)
    r.getRendererVariable("RenderPipeline").setSelectedOption(3)
    with pytest.raises(Y.YaptError):
        sc.update(0.0)  # debug pipelines are not built
    assert r.getRendererVariable("No.Such.Variable") is None
    assert "RenderPipeline" in r.getAllRendererVariableNames()
    with pytest.raises(Y.YaptError):
        r.createTexture("t", Y.ResourceDimension.TEXTURE_3D, Y.ResourceFormat.RGBA8_UNORM, 0, 4, 4, 1, 1)
    with pytest.raises(Y.YaptError):
        r.createTexture("t", Y.ResourceDimension.TEXTURE_2D, Y.ResourceFormat.R32_SFLOAT, 0, 4, 4, 1, 1)
    sc.shutdown()
    r.shutdown()


def test_textures_and_skybox(built, py_yapt):
    """A white albedo texture leaves the film bit for bit unchanged (albedo x 1); a coloured one
    and a skybox change it; every texture change restarts the accumulation."""
    Y = py_yapt
    r = setup_renderer(Y, 32, 24)
    sc = Y.Scene()
    sc.init(r)
    meshes, mats, objs = U.build_scene(Y, r, sc, U.box(2))
    # an RGB-albedo material on the walls (a texture modulates the RGB albedo; materials whose
    # albedo is a tabulated curve ignore it)
    wall = r.createMaterial("wall")
    wall.setAlbedo(Y.vec3([0.7, 0.7, 0.7]))
    wall.setMetalness(0.0)
    wall.setRoughness(1.0)
    objs[0].setMaterials([wall] * len(objs[0].getMaterials()))
    mats = [wall]
    sc.update(0.0, 2)
    base = film_of(Y, r)
    white = np.full((4, 4, 4), 255, np.uint8)
    t = r.createTexture("white", Y.ResourceDimension.TEXTURE_2D, Y.ResourceFormat.RGBA8_UNORM, 0, 4, 4, 1, 1)
    t.upload(0, 0, 1, 1, 16, white.ctypes.data, 0)
    assert t.getName() == "white"
    mats[0].setAlbedoTexture(t, Y.vec2([2.0, 2.0]))
    sc.update(0.0, 2)
    assert r.getAccumulatedFrames() == 2
    same = film_of(Y, r)
    assert np.array_equal(same, base)
    red = np.zeros((4, 4, 4), np.uint8)
    red[..., 0] = 255
    red[..., 3] = 255
    t.upload(0, 0, 1, 1, 16, red.ctypes.data, 0)  # new content: a new upload
    sc.update(0.0, 2)
    assert r.getAccumulatedFrames() == 2
    assert not np.array_equal(film_of(Y, r), base)
    sky = np.ones((8, 16, 4), np.float32)
    k = r.createTexture("sky", Y.ResourceDimension.TEXTURE_2D, Y.ResourceFormat.RGBA32_SFLOAT, 0, 16, 8, 1, 1)
    k.upload(0, 0, 1, 1, 16 * 16, sky.ctypes.data, 0)
    var = r.getRendererVariable("World.Skycube")
    assert var.getTexture() is None
    var.setTexture(k)
    assert var.getTexture().getName() == "sky"
    r.getRendererVariable("World.EnvIntensityScale").setFromFloatArray([1.0])
    sc.update(0.0, 2)
    img = film_of(Y, r)
    assert np.all(np.isfinite(img)) and float(img[..., 1].mean()) > 0.0
    # a cube map of the same constant sky, its faces uploaded in two ranges of slices, lights
    # the scene alike (up to the last-bit rounding of the bilinear weights)
    cube = r.createTexture("cube", Y.ResourceDimension.TEXTURE_CUBEMAP, Y.ResourceFormat.RGBA32_SFLOAT, 0, 8, 8, 1, 6)
    faces = np.ones((6, 8, 8, 4), np.float32)
    cube.upload(0, 0, 1, 2, 8 * 16, faces.ctypes.data, 0)
    cube.upload(0, 2, 1, 4, 8 * 16, faces.ctypes.data, 2 * 8 * 8 * 16)
    with pytest.raises(Y.YaptError):
        cube.upload(0, 4, 1, 3, 8 * 16, faces.ctypes.data, 0)  # slices 4..6 of six
    with pytest.raises(Y.YaptError):
        mats[0].setAlbedoTexture(cube, Y.vec2([1.0, 1.0]))
    with pytest.raises(Y.YaptError):
        r.createTexture("c", Y.ResourceDimension.TEXTURE_CUBEMAP, Y.ResourceFormat.RGBA8_UNORM, 0, 8, 4, 1, 6)
    var.setTexture(cube)
    sc.update(0.0, 2)
    assert np.allclose(film_of(Y, r), img, rtol=1e-5, atol=1e-7)
    sc.shutdown()
    r.shutdown()
