"""Scene construction through py_yapt the way the reference's scripts do it
(Source/Python/pythonScripts/yapt/mesh_utils.py:325-390): a tightly packed position
buffer, an interleaved normal (+ tangent) buffer, an index buffer, one setSubmesh per
submesh; render objects with a transform and per-submesh materials."""
import numpy as np

from yapt_gb300 import configs
from yapt_gb300.scene import MATERIAL_DEFAULTS, SPECTRUM_LMAX, SPECTRUM_LMIN, SPECTRUM_POINTS

GRID = list(np.linspace(SPECTRUM_LMIN, SPECTRUM_LMAX, SPECTRUM_POINTS))


def make_buffer(Y, renderer, name, data, usage):
    data = np.ascontiguousarray(data)
    buf = renderer.createBuffer(name, int(usage), data.nbytes)
    buf.upload(0, data.nbytes, data.ctypes.data, 0)
    return buf


def upload_mesh(Y, renderer, name, positions, normals, indices, submeshes=None, tangents=None, use16=False):
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, np.uint16 if use16 else np.uint32).reshape(-1)
    usage = Y.ResourceUsageBits.COPY_DESTINATION | Y.ResourceUsageBits.VERTEX_BUFFER
    F, S = Y.ResourceFormat, Y.AttributeSemanticName
    layouts = [Y.VertexBufferLayout([Y.MeshAttribute(F.RGB32_SFLOAT, S.POSITION, 0)], Y.VertexBufferLayout.STRIDE_TIGHTLY_PACKED)]
    attrs = [Y.MeshAttribute(F.RGB32_SFLOAT, S.NORMAL, 0)]
    cols = [nrm]
    if tangents is not None:
        attrs.append(Y.MeshAttribute(F.RGBA32_SFLOAT, S.TANGENT, 0))
        cols.append(np.ascontiguousarray(tangents, np.float32).reshape(-1, 4))
    layouts.append(Y.VertexBufferLayout(attrs, Y.VertexBufferLayout.STRIDE_TIGHTLY_PACKED))
    buffers = [make_buffer(Y, renderer, name + "_positions", pos, usage),
               make_buffer(Y, renderer, name + "_attrs", np.concatenate(cols, axis=1), usage)]
    ib = make_buffer(Y, renderer, name + "_indices", idx, Y.ResourceUsageBits.INDEX_BUFFER)
    if submeshes is None:
        submeshes = [(0, len(idx))]
    mesh = renderer.createMesh(name, layouts, len(pos), len(submeshes), use16)
    for i, b in enumerate(buffers):
        mesh.setVertexBuffer(i, b, 0)
    mesh.setIndexBuffer(ib, 0)
    for k, (first, count) in enumerate(submeshes):
        lo, hi = Y.Mesh.calculateBoundsFromVertexBuffer(pos.ctypes.data, idx.ctypes.data, first, count, 0, 12, use16)
        mesh.setSubmesh(k, first, count, 0, lo, hi)
    return mesh


def quaternion(R):
    """Unit quaternion (x, y, z, w) of a rotation matrix."""
    w = np.sqrt(max(0.0, 1.0 + R[0, 0] + R[1, 1] + R[2, 2])) / 2
    x = np.sqrt(max(0.0, 1.0 + R[0, 0] - R[1, 1] - R[2, 2])) / 2
    y = np.sqrt(max(0.0, 1.0 - R[0, 0] + R[1, 1] - R[2, 2])) / 2
    z = np.sqrt(max(0.0, 1.0 - R[0, 0] - R[1, 1] + R[2, 2])) / 2
    x = np.copysign(x, R[2, 1] - R[1, 2])
    y = np.copysign(y, R[0, 2] - R[2, 0])
    z = np.copysign(z, R[1, 0] - R[0, 1])
    return [x, y, z, w]


def set_material(Y, mat, params):
    """Principled parameters (scene.MATERIAL_DEFAULTS names) through the Material setters."""
    p = dict(MATERIAL_DEFAULTS)
    p.update(params)
    v3 = lambda v: Y.vec3([float(x) for x in v])  # noqa: E731
    mat.setAlbedo(v3(p["albedo"]))
    mat.setTransparency(p["transparency"])
    mat.setSpecularTint(v3(p["specular"]))
    mat.setMetalness(p["metalness"])
    mat.setAbsorption(v3(p["absorption"]))
    mat.setDielectricIOR(p["dielectric_ior"])
    mat.setEmission(v3(p["emissive"]))
    mat.setRoughness(p["roughness"])
    mat.setAnisotropy(p["anisotropy"])
    mat.setAnisotropyRotation(p["anisotropy_rotation"])
    mat.setTwoSided(bool(p["material_mask"] & 1))
    mat.setEnableDispersion(bool(p["material_mask"] & 2))
    mat.setThinFilmThicknessNM(p["thin_film_thickness_nm"])
    mat.setCauchysCoefficients(Y.vec2([float(c) for c in p["cauchy"]]))
    mat.setSheenAmount(p["sheen_amount"])
    mat.setEmissionFocus(p["emission_focus"])
    mat.setSheenTint(v3(p["sheen_tint"]))
    mat.setSheenRoughness(p["sheen_roughness"])
    mat.setSpecularAmount(p["specular_amount"])
    mat.setClearCoatAmount(p["clear_coat_amount"])
    mat.setClearCoatIOR(p["clear_coat_ior"])
    mat.setClearCoatRoughness(p["clear_coat_roughness"])


def build_scene(Y, renderer, scene, sc):
    """Rebuilds a yapt_gb300.scene.Scene through py_yapt. Returns the objects (they must stay
    referenced: a render object whose last reference is dropped leaves the scene)."""
    meshes = [upload_mesh(Y, renderer, "mesh%d" % i, m["positions"], m["normals"], m["indices"], m["submeshes"],
                          m["tangents"]) for i, m in enumerate(sc.meshes)]
    mats = []
    for i, params in enumerate(sc.materials):
        mat = renderer.createMaterial("mat%d" % i)
        set_material(Y, mat, params)
        for key, setter in (("albedo_spectrum", mat.setAlbedoSpectrum), ("specular_spectrum", mat.setSpecularSpectrum),
                            ("emission_spectrum", mat.setEmissionSpectrum)):
            sid = params.get(key, -1)
            if sid >= 0:
                setter(GRID, [float(v) for v in sc.spectra[sid]])
        mats.append(mat)
    # group consecutive instances that cover all submeshes of one mesh with one transform
    # into one render object with a material per submesh
    groups = []
    for (o2w, mesh, sub, mat) in sc.instances:
        g = groups[-1] if groups else None
        if g and g["mesh"] == mesh and np.array_equal(g["o2w"], o2w) and sub == len(g["mats"]):
            g["mats"].append(mat)
        else:
            groups.append(dict(mesh=mesh, o2w=np.asarray(o2w, float), first_sub=sub, mats=[mat]))
    objs = []
    for k, g in enumerate(groups):
        ro = scene.createRenderObject("obj%d" % k)
        M = g["o2w"]
        scale = np.linalg.norm(M[:3, :3], axis=0)
        R = M[:3, :3] / scale
        t = ro.getTransform()
        t.setTranslation(Y.vec3([float(x) for x in M[:3, 3]]))
        t.setScale(Y.vec3([float(x) for x in scale]))
        t.setOrientation(Y.vec4([float(x) for x in quaternion(R)]))
        m = sc.meshes[g["mesh"]]
        if g["first_sub"] == 0 and len(g["mats"]) == len(m["submeshes"]):
            ro.setMesh(meshes[g["mesh"]])
        else:  # a view of the one submesh this instance draws
            assert len(g["mats"]) == 1
            first, count = m["submeshes"][g["first_sub"]]
            ro.setMesh(upload_mesh(Y, renderer, "mesh%d_%d" % (g["mesh"], g["first_sub"]), m["positions"],
                                   m["normals"], m["indices"][first:first + count], None, m["tangents"]))
        ro.setMaterials([mats[i] for i in g["mats"]])
        objs.append(ro)
    cam = scene.getMainCamera()
    c = sc.camera
    cam.setProjectionPerspective(float(c.fovy), float(c.aspect), float(c.near), float(c.far))
    W = c.world
    eye = W[:3, 3]
    cam.getTransform().lookAt(Y.vec3([float(x) for x in eye]), Y.vec3([float(x) for x in eye - W[:3, 2]]),
                              Y.vec3([0.0, 1.0, 0.0]))
    return meshes, mats, objs


def box(seed=1):
    return configs.box_scene(seed)
