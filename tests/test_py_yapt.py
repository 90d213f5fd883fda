"""py_yapt without a device: the reference's Python names, vector types, transform and camera
math, mesh layout decoding and material presets.

Transform and camera conventions follow Source/Scene/inc/Scene/Transform.inl (object matrix
T * R(q) * S, parent * child, look-at along local -z) and Camera.inl (glm::perspective); the
camera constants must agree with yapt_gb300.scene.CameraDesc (the path the parity tests use)
to 1e-6 relative."""
import numpy as np
import pytest

from yapt_gb300.scene import CameraDesc

# class -> methods of the reference bindings (Source/Python/srcBindings/*.cpp)
REFERENCE_SURFACE = {
    "Renderer": ["init", "shutdown", "getRendererVariable", "getAllRendererVariableNames", "setRenderOutputToSurface",
                 "resetRenderOutput", "createTexture", "createBuffer", "createMesh", "createMaterial", "readback"],
    "Scene": ["init", "shutdown", "update", "createRenderObject", "createSceneObject", "createLight", "getMainCamera"],
    "Material": ["setFromMaterialPreset", "getName", "setTransparency", "getTransparency", "setMetalness", "getMetalness",
                 "setAlbedo", "getAlbedo", "setSpecularTint", "getSpecularTint", "setAbsorption", "getAbsorption",
                 "setEmission", "getEmission", "setEmissionFocus", "getEmissionFocus", "setDielectricIOR",
                 "getDielectricIOR", "setRoughness", "getRoughness", "setAnisotropy", "getAnisotropy",
                 "setAnisotropyRotation", "getAnisotropyRotation", "setTwoSided", "getTwoSided", "setSpecularAmount",
                 "getSpecularAmount", "setClearCoatAmount", "getClearCoatAmount", "setClearCoatRoughness",
                 "getClearCoatRoughness", "setClearCoatIOR", "getClearCoatIOR", "setSheenRoughness", "getSheenRoughness",
                 "setSheenTint", "getSheenTint", "setSheenAmount", "getSheenAmount", "setAlphaCutoff", "getAlphaCutoff",
                 "setAlphaBlend", "getAlphaBlend", "setThinFilmThicknessNM", "getThinFilmThicknessNM",
                 "setCauchysCoefficients", "getCauchysCoefficients", "setEnableDispersion", "getEnableDispersion",
                 "setSubsurfaceAmount", "getSubsurfaceAmount", "setSubsurfaceRadius", "getSubsurfaceRadius",
                 "setSubsurfaceRadiusScale", "getSubsurfaceRadiusScale", "setAlbedoTexture", "setNormalTexture",
                 "setORMTexture", "setEmissiveTexture"],
    "Mesh": ["getName", "setVertexBuffer", "setIndexBuffer", "setSubmesh", "getSubmeshCount",
             "calculateBoundsFromVertexBuffer"],
    "MeshAttribute": ["format", "semanticName", "semanticIndex"],
    "VertexBufferLayout": ["attributes", "vertexStrideInBytes", "STRIDE_TIGHTLY_PACKED"],
    "Buffer": ["upload", "getName"],
    "SceneObject": ["getName", "getTransform"],
    "RenderObject": ["setMesh", "setMaterial", "setMaterials", "getMaterials", "getMesh", "getName", "getTransform"],
    "Light": ["setType", "getType", "setColor", "getColor", "setIntensity", "getIntensity", "setSpotConeAngles",
              "getSpotInnerAngle", "getSpotOuterAngle"],
    "Camera": ["setProjectionPerspective", "setProjectionOrthographic", "setFOVY", "setAspectRatio", "setNearPlane",
               "setFarPlane", "setOrthographicSize", "setProjectionType", "getFOVY", "getAspectRatio", "getNearPlane",
               "getFarPlance", "getOrthographicSize", "getProjectionType", "getTransform"],
    "Transform": ["setTranslation", "addTranslation", "getTranslation", "setScale", "addScale", "getScale",
                  "setOrientation", "addOrientation", "getOrientation", "lookAt", "right", "up", "forward", "setParent",
                  "getId", "getParentId"],
    "RendererVariable": ["setFromFloatArray", "setFromIntArray", "getAsFloatArray", "getAsIntArray", "getLimitsFloat",
                         "getLimitsInt", "getComponentCount", "getOptions", "getSelectedOption", "setSelectedOption",
                         "getType"],
    "ReadbackObject": ["getState", "isReady", "release", "getData"],
    "ReadbackData": ["getWidth", "getHeight", "getDepthOrSlices", "getTexelSizeInBytes", "getRowPitchInBytes",
                     "getSizeInBytes", "getFormat", "getDimensions", "getBytes"],
    "RendererCache": ["getDefaultRendererCache"],
}
ENUMS = {
    ("Material", "MaterialPreset"): ["BLANK", "METAL_GOLD", "METAL_SILVER", "METAL_COPPER", "METAL_BRASS",
                                     "METAL_ALUMINIUM", "GLASS", "PLASTIC"],
    ("Light", "LightType"): ["POINT", "SPOT", "DIRECTIONAL"],
    ("Camera", "ProjectionType"): ["PERSPECTIVE", "ORTHOGRAPHIC"],
    (None, "ReadbackTarget"): ["FinalColor", "FilmXYZ", "FilmRGB", "Features"],
    (None, "ReadbackState"): ["Created", "Pending", "Ready", "Failed", "Freed"],
    (None, "RendererVariableType"): ["FLOAT", "INT", "TEXTURE", "BUFFER", "OPTIONS"],
    (None, "AttributeSemanticName"): ["UNKNOWN", "POSITION", "TEXCOORD", "NORMAL", "TANGENT", "COLOR"],
    (None, "ResourceUsageBits"): ["COPY_DESTINATION", "VERTEX_BUFFER", "INDEX_BUFFER",
                                  "ACCELERATION_STRUCTURE_BUILD_INPUT", "SAMPLED_TEXTURE"],
    (None, "ResourceFormat"): ["RGB32_SFLOAT", "RGBA32_SFLOAT", "RG32_SFLOAT", "RGBA8_UNORM", "R16_UINT", "R32_UINT"],
}


def test_reference_names_are_all_present(py_yapt):
    Y = py_yapt
    for cls, methods in REFERENCE_SURFACE.items():
        c = getattr(Y, cls)
        missing = [m for m in methods if not hasattr(c, m)]
        assert not missing, (cls, missing)
    for (owner, enum), values in ENUMS.items():
        e = getattr(getattr(Y, owner) if owner else Y, enum)
        assert all(hasattr(e, v) for v in values), enum
    for v in ("vec2", "vec3", "vec4", "ivec2", "ivec3", "ivec4"):
        assert hasattr(Y, v)


def test_vectors(py_yapt):
    Y = py_yapt
    a = Y.vec3([1.0, 2.0, 3.0])
    b = Y.vec3(2.0)
    assert list(a + b) == [3.0, 4.0, 5.0] and list(a * b) == [2.0, 4.0, 6.0] and list(a / 2.0) == [0.5, 1.0, 1.5]
    assert len(Y.vec4()) == 4 and a[2] == 3.0
    a[0] = 7.0
    assert a[0] == 7.0
    with pytest.raises(IndexError):
        a[3]
    assert list(Y.ivec2([3, -4])) == [3, -4]


def quat_matrix(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def scene_with_objects(Y):
    sc = Y.Scene()  # objects can be made and edited before init; rendering needs it
    return sc, sc.createRenderObject("a"), sc.createSceneObject("parent")


def test_transform_matrices(py_yapt):
    Y = py_yapt
    sc, ro, parent = scene_with_objects(Y)
    t = ro.getTransform()
    q = np.array([0.1, -0.3, 0.2, 0.9])
    q /= np.linalg.norm(q)
    t.setTranslation(Y.vec3([1.0, 2.0, -3.0]))
    t.setScale(Y.vec3([2.0, 0.5, 1.5]))
    t.setOrientation(Y.vec4([float(v) for v in q]))
    qf = np.array(list(t.getOrientation()), np.float64)
    M = np.eye(4)
    M[:3, :3] = quat_matrix(qf) @ np.diag([2.0, 0.5, 1.5])
    M[:3, 3] = [1.0, 2.0, -3.0]
    np.testing.assert_allclose(np.array(t.getMatrixWS()), M, rtol=0, atol=1e-12)
    # parenting composes parent * child
    pt = parent.getTransform()
    pt.setTranslation(Y.vec3([0.0, 10.0, 0.0]))
    t.setParent(pt)
    assert t.getParentId() == pt.getId() != 0
    P = np.eye(4)
    P[1, 3] = 10.0
    np.testing.assert_allclose(np.array(t.getMatrixWS()), P @ M, atol=1e-12)
    with pytest.raises(Y.YaptError):
        pt.setParent(t)  # cycle
    t.setParent(None)
    # the reference's addScale assigns; addTranslation adds; addOrientation multiplies
    t.addScale(Y.vec3([3.0, 3.0, 3.0]))
    assert list(t.getScale()) == [3.0, 3.0, 3.0]
    t.addTranslation(Y.vec3([1.0, 1.0, 1.0]))
    assert list(t.getTranslation()) == [2.0, 3.0, -2.0]
    t.setOrientation(Y.vec4([0.0, 0.0, 0.0, 1.0]))
    r = [0.0, np.sin(0.25), 0.0, np.cos(0.25)]
    t.addOrientation(Y.vec4(r))
    t.addOrientation(Y.vec4(r))
    np.testing.assert_allclose(list(t.getOrientation()), [0.0, np.sin(0.5), 0.0, np.cos(0.5)], atol=1e-6)


def test_look_at_and_axes(py_yapt):
    Y = py_yapt
    sc = Y.Scene()
    t = sc.getMainCamera().getTransform()
    eye, at = np.array([0.5, 0.7, 2.1]), np.array([0.4, 0.5, 0.0])
    t.lookAt(Y.vec3(list(eye)), Y.vec3(list(at)), Y.vec3([0.0, 1.0, 0.0]))
    want = CameraDesc(eye=eye, target=at).world
    np.testing.assert_allclose(np.array(t.getMatrixWS()), want, atol=2e-6)
    f = (at - eye) / np.linalg.norm(at - eye)
    np.testing.assert_allclose(list(t.forward()), f, atol=2e-6)
    np.testing.assert_allclose(list(t.right()), want[:3, 0], atol=2e-6)
    np.testing.assert_allclose(list(t.up()), want[:3, 1], atol=2e-6)


def test_camera_constants_match_the_scene_camera(py_yapt):
    Y = py_yapt
    sc = Y.Scene()
    cam = sc.getMainCamera()
    assert abs(cam.getFOVY() - np.pi * 0.3) < 1e-6 and cam.getNearPlane() == pytest.approx(0.1)
    cam.setProjectionPerspective(float(np.pi * 0.22), 1.25, 0.1, 1000.0)
    eye, at = [0.5, 0.5, 2.1], [0.5, 0.5, 0.0]
    cam.getTransform().lookAt(Y.vec3(eye), Y.vec3(at), Y.vec3([0.0, 1.0, 0.0]))
    got = cam._constants(0.02, 3.0)
    desc = CameraDesc(eye=eye, target=at, fovy=np.float32(np.pi * 0.22), aspect=1.25)
    desc.world = np.array(cam.getTransform().getMatrixWS())
    want = desc.matrices()
    for k in ("uv_to_view", "view_to_uv", "world_to_view", "view_to_world"):
        np.testing.assert_allclose(np.array(got[k]).reshape(4, 4), np.asarray(want[k], np.float32), rtol=1e-6,
                                   atol=1e-6)
    assert got["z_sign"] == want["z_sign"]
    cam.setProjectionType(Y.Camera.ProjectionType.ORTHOGRAPHIC)
    with pytest.raises(Y.YaptError):
        cam._constants(0.0, 1.0)


def test_mesh_layouts_offsets_strides_and_submeshes(py_yapt):
    Y = py_yapt
    F, S = Y.ResourceFormat, Y.AttributeSemanticName
    r = Y.Renderer()  # resource creation needs no device
    n = 6
    rng = np.random.default_rng(0)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    uv = rng.uniform(size=(n, 2)).astype(np.float32)
    tan = rng.normal(size=(n, 4)).astype(np.float32)
    # one interleaved buffer, stride 64 with padding, explicit and inferred offsets:
    # position @0, uv @12 (inferred), normal @24 (explicit), tangent @36 (inferred)
    inter = np.zeros((n, 16), np.float32)
    inter[:, 0:3], inter[:, 3:5], inter[:, 6:9], inter[:, 9:13] = pos, uv, nrm, tan
    layout = Y.VertexBufferLayout([Y.MeshAttribute(F.RGB32_SFLOAT, S.POSITION, 0),
                                   Y.MeshAttribute(F.RG32_SFLOAT, S.TEXCOORD, 0),
                                   Y.MeshAttribute(F.RGB32_SFLOAT, S.NORMAL, 0, 24),
                                   Y.MeshAttribute(F.RGBA32_SFLOAT, S.TANGENT, 0)], 64)
    vb = r.createBuffer("v", int(Y.ResourceUsageBits.VERTEX_BUFFER), inter.nbytes + 16)
    vb.upload(16, inter.nbytes, inter.ctypes.data, 0)  # data at a 16-byte buffer offset
    idx = np.array([0, 1, 2, 0, 1, 2, 1, 2, 0], np.uint16)  # second submesh uses vertex offset 3
    ib = r.createBuffer("i", int(Y.ResourceUsageBits.INDEX_BUFFER), idx.nbytes)
    ib.upload(0, idx.nbytes, idx.ctypes.data, 0)
    mesh = r.createMesh("m", [layout], n, 2, True)
    mesh.setVertexBuffer(0, vb, 16)
    mesh.setIndexBuffer(ib, 0)
    lo, hi = Y.Mesh.calculateBoundsFromVertexBuffer(pos.ctypes.data, idx.ctypes.data, 0, 3, 0, 12, True)
    np.testing.assert_array_equal(list(lo), pos[:3].min(0))
    np.testing.assert_array_equal(list(hi), pos[:3].max(0))
    mesh.setSubmesh(0, 0, 3, 0, lo, hi)
    with pytest.raises(Y.YaptError):
        mesh._decoded()  # submesh 1 not set
    mesh.setSubmesh(1, 3, 6, 3, lo, hi)
    d = mesh._decoded()
    np.testing.assert_array_equal(np.array(d["positions"]).reshape(n, 3), pos)
    np.testing.assert_array_equal(np.array(d["normals"]).reshape(n, 3), nrm)
    np.testing.assert_array_equal(np.array(d["uvs"]).reshape(n, 2), uv)
    np.testing.assert_array_equal(np.array(d["tangents"]).reshape(n, 4), tan)
    assert d["indices"] == [0, 1, 2, 3, 4, 5, 4, 5, 3]
    assert d["submeshes"] == [0, 3, 3, 6]
    with pytest.raises(Y.YaptError):
        vb.upload(inter.nbytes, 32, inter.ctypes.data, 0)  # outside the buffer


def test_material_presets_defaults_and_spectra(py_yapt):
    Y = py_yapt
    r = Y.Renderer()
    m = r.createMaterial("m")
    # MaterialParameters() defaults
    assert list(m.getAlbedo()) == [1.0, 1.0, 1.0] and m.getMetalness() == 1.0
    assert m.getRoughness() == pytest.approx(0.1) and m.getDielectricIOR() == pytest.approx(1.5)
    np.testing.assert_allclose(list(m.getCauchysCoefficients()), [1.5046, 0.0042], rtol=1e-6)
    m.setFromMaterialPreset(Y.Material.MaterialPreset.METAL_GOLD)
    want = np.power(np.array([0.9451, 0.7294, 0.37255]), 2.2).astype(np.float32)
    np.testing.assert_array_equal(np.array(list(m.getAlbedo()), np.float32), want)
    assert m.getRoughness() == 0.0 and m.getMetalness() == 1.0 and m.getTransparency() == 0.0
    m.setFromMaterialPreset(Y.Material.MaterialPreset.GLASS)
    assert m.getTransparency() == 1.0 and m.getMetalness() == 0.0 and list(m.getAlbedo()) == [1.0, 1.0, 1.0]
    m.setTwoSided(True)
    m.setEnableDispersion(True)
    assert m.getTwoSided() and m.getEnableDispersion()
    # tabulated spectra resampled like numpy.interp onto the 5 nm grid
    lam, val = [400.0, 500.0, 650.0], [0.2, 0.8, 0.4]
    m.setAlbedoSpectrum(lam, val)
    grid = np.linspace(380, 780, 81)
    np.testing.assert_array_equal(np.array(m.getAlbedoSpectrum(), np.float32), np.interp(grid, lam, val).astype(np.float32))
    m.setEmissionBlackbody(3000.0)
    from yapt_gb300.configs import blackbody_spectrum
    np.testing.assert_allclose(m.getEmissionSpectrum(), blackbody_spectrum(3000.0), rtol=1e-6)
    with pytest.raises(TypeError):  # a Texture from Renderer.createTexture is required
        m.setAlbedoTexture(None, Y.vec2(1.0))


def test_lights_variables_and_headless_errors(py_yapt):
    Y = py_yapt
    sc = Y.Scene()
    light = sc.createLight("l", Y.Light.LightType.SPOT)
    assert light.getType() == Y.Light.LightType.SPOT and light.getIntensity() == 1.0
    light.setSpotConeAngles(2.0, 3.0)  # clamped: outer to pi/2, inner to outer
    assert light.getSpotOuterAngle() == pytest.approx(np.pi / 2) and light.getSpotInnerAngle() == pytest.approx(np.pi / 2)
    r = Y.Renderer()
    with pytest.raises(Y.YaptError):
        r.getRendererVariable("RenderPipeline")  # not initialised
    with pytest.raises(Y.YaptError):
        sc.update(0.016)  # scene not initialised
    with pytest.raises(Y.YaptError):
        r.setRenderOutputToSurface(64, 64, 0)
