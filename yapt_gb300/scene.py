"""Scene description on the host: meshes, materials, spectra, instances, camera.

A Scene is plain numpy data. ``upload`` hands it to a native context through the
C ABI (yg_upload_mesh / yg_upload_materials / yg_set_instances / yg_set_camera);
``pooled`` returns the same data flattened the way a per-instance consumer (the
oracle, a checker) reads it.

Camera conventions follow YAPT: view = inverse(camera world matrix), projection
glm::perspective (right handed, NDC z in [-1, 1]) mapped to the DX12 platform NDC
and then to texture space with v pointing down
(Source/Renderer/inc/Renderer/Shared/Utility/RenderAPIAbstractionUtility.h:18-58,
RaytraceCommonResources.cpp:64-140, Source/Scene/inc/Scene/Camera.inl:46-51).
"""
import ctypes as C

import numpy as np

from . import _native as N

# defaults of MaterialParameters (Source/Renderer/inc/Renderer/Shared/MaterialInternal.h:41-77)
MATERIAL_DEFAULTS = dict(
    albedo=(1.0, 1.0, 1.0), transparency=0.0, specular=(1.0, 1.0, 1.0), metalness=1.0,
    absorption=(0.0, 0.0, 0.0), dielectric_ior=1.5, emissive=(0.0, 0.0, 0.0), roughness=0.1,
    anisotropy=0.0, anisotropy_rotation=0.0, material_mask=0, thin_film_thickness_nm=0.0,
    cauchy=(1.5046, 0.00420), sheen_amount=0.0, emission_focus=0.0, sheen_tint=(1.0, 1.0, 1.0),
    sheen_roughness=0.5, specular_amount=1.0, clear_coat_amount=0.0, clear_coat_ior=1.5,
    clear_coat_roughness=0.1, subsurface_radius=(1.0, 0.2, 0.1), subsurface_amount=0.0,
    subsurface_radius_scale=1.0, alpha_cutoff=0.0, albedo_spectrum=-1, specular_spectrum=-1,
    emission_spectrum=-1,
    # texture id + 1 (0: none) and uv scale per slot
    albedo_texture=0, normal_texture=0, orm_texture=0, emissive_texture=0,
    albedo_uv_scale=(1.0, 1.0), normal_uv_scale=(1.0, 1.0), orm_uv_scale=(1.0, 1.0), emissive_uv_scale=(1.0, 1.0),
)

# the spectral grid every tabulated curve is stored on (5 nm steps)
SPECTRUM_LMIN, SPECTRUM_LMAX, SPECTRUM_POINTS = 380.0, 780.0, 81


def material_struct(params):
    m = N.Material()
    p = dict(MATERIAL_DEFAULTS)
    unknown = set(params) - set(p)
    if unknown:
        raise ValueError("unknown material parameters: %s" % sorted(unknown))
    p.update(params)
    for k, v in p.items():
        if isinstance(v, (tuple, list, np.ndarray)):
            arr = getattr(m, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        elif k in ("material_mask",):
            setattr(m, k, int(v))
        elif k.endswith("_spectrum") or k.endswith("_texture"):
            setattr(m, k, int(v))
        else:
            setattr(m, k, float(v))
    return m


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def affine(translation=(0, 0, 0), rotation=None, scale=(1, 1, 1)):
    """4x4 float64 object-to-world matrix T * R * S."""
    M = np.eye(4)
    R = np.eye(3) if rotation is None else np.asarray(rotation, dtype=np.float64)
    M[:3, :3] = R @ np.diag(np.asarray(scale, dtype=np.float64))
    M[:3, 3] = translation
    return M


def rotation_x(angle):
    c, s = np.cos(angle), np.sin(angle)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def rotation_y(angle):
    c, s = np.cos(angle), np.sin(angle)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def look_at_world(eye, target, up=(0, 1, 0)):
    """Camera world matrix: the camera looks down its local -z (right handed)."""
    eye = np.asarray(eye, float)
    f = np.asarray(target, float) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, float))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    M = np.eye(4)
    M[:3, 0], M[:3, 1], M[:3, 2], M[:3, 3] = r, u, -f, eye
    return M


def perspective(fovy, aspect, near, far):
    """glm::perspective (right handed, clip z in [-1, 1])."""
    t = np.tan(fovy / 2.0)
    P = np.zeros((4, 4))
    P[0, 0] = 1.0 / (aspect * t)
    P[1, 1] = 1.0 / t
    P[2, 2] = -(far + near) / (far - near)
    P[2, 3] = -(2.0 * far * near) / (far - near)
    P[3, 2] = -1.0
    return P


NDC_TO_DX12 = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0.5, 0.5], [0, 0, 0, 1.0]])
DX12_NDC_TO_UV = np.array([[0.5, 0, 0, 0.5], [0, -0.5, 0, 0.5], [0, 0, 1, 0], [0, 0, 0, 1.0]])


class CameraDesc:
    def __init__(self, eye, target, up=(0, 1, 0), fovy=np.pi * 0.3, aspect=1.0, near=0.1, far=1000.0,
                 aperture_radius=0.0, focus_distance=10.0):
        self.world = look_at_world(eye, target, up)
        self.fovy, self.aspect, self.near, self.far = fovy, aspect, near, far
        self.aperture_radius, self.focus_distance = aperture_radius, focus_distance

    def matrices(self):
        view = np.linalg.inv(self.world)
        view_to_uv = DX12_NDC_TO_UV @ NDC_TO_DX12 @ perspective(self.fovy, self.aspect, self.near, self.far)
        uv_to_view = np.linalg.inv(view_to_uv)
        c = uv_to_view @ np.array([0.5, 0.5, 0.0, 1.0])
        zsign = -1.0 if c[2] / c[3] < 0 else 1.0
        return dict(uv_to_view=uv_to_view, view_to_uv=view_to_uv, world_to_view=view, view_to_world=self.world,
                    z_sign=zsign)

    def struct(self):
        m = self.matrices()
        cam = N.Camera()
        for k in ("uv_to_view", "view_to_uv", "world_to_view", "view_to_world"):
            arr = getattr(cam, k)
            for i, v in enumerate(np.asarray(m[k], np.float32).reshape(-1)):
                arr[i] = float(v)
        cam.aperture_radius = max(0.0, self.aperture_radius)
        cam.focus_distance = max(1e-4, self.focus_distance)
        cam.view_forward_z_sign = m["z_sign"]
        return cam


class Scene:
    def __init__(self):
        self.meshes = []      # dict(positions, normals, tangents, indices, submeshes)
        self.materials = []   # dict of parameters
        self.spectra = []     # arrays of SPECTRUM_POINTS values
        self.instances = []   # (o2w 4x4 float64, mesh, submesh, material)
        self.camera = None
        self.name = "scene"
        self.punctual_lights = []  # dict(type, position, direction, intensity, cos_inner, cos_outer)
        self.textures = []         # (width, height, format, texel array)
        self.env_texture = 0       # texture id + 1 of the environment (longitude-latitude map)
        self.env_cube = False      # True: env_texture is a cube map, faces stacked +X, -X, +Y, -Y, +Z, -Z

    # -- building --------------------------------------------------------
    def add_texture(self, texels, fmt=None):
        """texels: (h, w, 4) uint8 (fmt RGBA8_UNORM or RGBA8_SRGB, default sRGB) or float32
        (RGBA32_FLOAT). Returns the id + 1 that materials and env_texture refer to."""
        a = np.ascontiguousarray(texels)
        assert a.ndim == 3 and a.shape[2] == 4
        if a.dtype == np.uint8:
            fmt = N.YG_TEXTURE_RGBA8_SRGB if fmt is None else fmt
        else:
            a = np.ascontiguousarray(a, np.float32)
            fmt = N.YG_TEXTURE_RGBA32_FLOAT
        self.textures.append((a.shape[1], a.shape[0], fmt, a))
        return len(self.textures)

    def add_mesh(self, positions, normals, indices, submeshes=None, tangents=None, uvs=None):
        pos = _f32(positions).reshape(-1, 3)
        nrm = _f32(normals).reshape(-1, 3)
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32).reshape(-1))
        if submeshes is None:
            submeshes = [(0, len(idx))]
        tan = None if tangents is None else _f32(tangents).reshape(-1, 4)
        uv = None if uvs is None else _f32(uvs).reshape(-1, 2)
        self.meshes.append(dict(positions=pos, normals=nrm, indices=idx, submeshes=list(submeshes), tangents=tan, uvs=uv))
        return len(self.meshes) - 1

    def add_material(self, **params):
        self.materials.append(dict(params))
        return len(self.materials) - 1

    def add_spectrum(self, values):
        v = np.asarray(values, dtype=np.float32).reshape(-1)
        if v.size != SPECTRUM_POINTS:
            raise ValueError("spectra are stored on %d points (380..780 nm)" % SPECTRUM_POINTS)
        self.spectra.append(v)
        return len(self.spectra) - 1

    def add_punctual_light(self, kind, position=(0, 0, 0), direction=(0, -1, 0), intensity=(1, 1, 1), cos_inner=1.0,
                           cos_outer=0.0):
        """kind: "point", "spot" or "directional" (RGB intensity; irradiance for directional)."""
        t = {"point": N.YG_LIGHT_POINT, "spot": N.YG_LIGHT_SPOT, "directional": N.YG_LIGHT_DIRECTIONAL}[kind]
        self.punctual_lights.append(dict(type=t, position=tuple(position), direction=tuple(direction),
                                         intensity=tuple(intensity), cos_inner=float(cos_inner),
                                         cos_outer=float(cos_outer)))
        return len(self.punctual_lights) - 1

    def punctual_structs(self):
        arr = (N.PunctualLight * max(1, len(self.punctual_lights)))()
        for i, L in enumerate(self.punctual_lights):
            arr[i].type = L["type"]
            for k in range(3):
                arr[i].position[k] = float(L["position"][k])
                arr[i].direction[k] = float(L["direction"][k])
                arr[i].intensity[k] = float(L["intensity"][k])
            arr[i].cos_inner, arr[i].cos_outer = L["cos_inner"], L["cos_outer"]
        return arr

    def add_instance(self, mesh, material, o2w=None, submesh=0):
        o2w = np.eye(4) if o2w is None else np.asarray(o2w, dtype=np.float64)
        self.instances.append((o2w, mesh, submesh, material))
        return len(self.instances) - 1

    def triangle_count(self):
        return sum(self.meshes[m]["submeshes"][s][1] // 3 for (_, m, s, _) in self.instances)

    # -- native ----------------------------------------------------------
    def instance_structs(self):
        arr = (N.Instance * max(1, len(self.instances)))()
        for i, (o2w, mesh, sub, mat) in enumerate(self.instances):
            w2o = np.linalg.inv(o2w)
            a = np.asarray(o2w[:3, :], np.float32).reshape(-1)
            b = np.asarray(w2o[:3, :], np.float32).reshape(-1)
            for k in range(12):
                arr[i].obj_to_world[k] = float(a[k])
                arr[i].world_to_obj[k] = float(b[k])
            arr[i].mesh, arr[i].submesh, arr[i].material = mesh, sub, mat
        return arr

    def material_structs(self):
        arr = (N.Material * max(1, len(self.materials)))()
        for i, p in enumerate(self.materials):
            arr[i] = material_struct(p)
        return arr

    def spectra_array(self):
        if not self.spectra:
            return np.zeros((0, SPECTRUM_POINTS), np.float32)
        return np.ascontiguousarray(np.stack(self.spectra).astype(np.float32))

    def upload(self, lib, ctx):
        """Uploads everything through the C ABI and builds the acceleration structure."""
        for m in self.meshes:
            d = N.MeshDesc()
            d.positions = m["positions"].ctypes.data_as(C.POINTER(C.c_float))
            d.normals = m["normals"].ctypes.data_as(C.POINTER(C.c_float))
            d.tangents = m["tangents"].ctypes.data_as(C.POINTER(C.c_float)) if m["tangents"] is not None else None
            d.uvs = m["uvs"].ctypes.data_as(C.POINTER(C.c_float)) if m.get("uvs") is not None else None
            d.vertex_count = len(m["positions"])
            d.indices = m["indices"].ctypes.data_as(C.c_void_p)
            d.index_count = len(m["indices"])
            d.index_bits = 32
            rng = np.asarray(m["submeshes"], dtype=np.uint32).reshape(-1)
            d.submesh_ranges = rng.ctypes.data_as(C.POINTER(C.c_uint32))
            d.submesh_count = len(m["submeshes"])
            mid = C.c_uint32()
            N.check(lib.yg_upload_mesh(ctx, C.byref(d), C.byref(mid)))
        mats = self.material_structs()
        N.check(lib.yg_upload_materials(ctx, mats, len(self.materials)))
        spec = self.spectra_array()
        if len(spec):
            N.check(lib.yg_upload_spectra(ctx, spec.ctypes.data_as(C.POINTER(C.c_float)), len(spec), SPECTRUM_POINTS,
                                          SPECTRUM_LMIN, SPECTRUM_LMAX))
        inst = self.instance_structs()
        N.check(lib.yg_set_instances(ctx, inst, len(self.instances)))
        if self.camera is not None:
            cam = self.camera.struct()
            N.check(lib.yg_set_camera(ctx, C.byref(cam)))
        N.check(lib.yg_set_punctual_lights(ctx, self.punctual_structs(), len(self.punctual_lights)))
        N.check(lib.yg_clear_textures(ctx))
        for (w, h, fmt, a) in self.textures:
            tid = C.c_uint32()
            N.check(lib.yg_upload_texture(ctx, w, h, fmt, a.ctypes.data_as(C.c_void_p), C.byref(tid)))
        if self.env_cube:
            N.check(lib.yg_set_environment_cube(ctx, self.env_texture))
        else:
            N.check(lib.yg_set_environment_texture(ctx, self.env_texture))
        N.check(lib.yg_build_scene(ctx))

    def pooled(self):
        """Vertex/index pools and per-instance records (first index, prim count, vertex base)."""
        pos, nrm, tan, idx, uvs = [], [], [], [], []
        vbase, ibase = [], []
        nv = ni = 0
        for m in self.meshes:
            vbase.append(nv)
            ibase.append(ni)
            pos.append(m["positions"])
            nrm.append(m["normals"])
            t = m["tangents"] if m["tangents"] is not None else np.tile(np.float32([1, 0, 0, 1]), (len(m["positions"]), 1))
            tan.append(t)
            uvs.append(m["uvs"] if m.get("uvs") is not None else np.full((len(m["positions"]), 2), 0.5, np.float32))
            idx.append(m["indices"])
            nv += len(m["positions"])
            ni += len(m["indices"])
        inst = []
        for (o2w, mesh, sub, mat) in self.instances:
            first, count = self.meshes[mesh]["submeshes"][sub]
            inst.append(dict(o2w=o2w, first_index=ibase[mesh] + first, prim_count=count // 3, vertex_base=vbase[mesh],
                             material=mat, has_tangents=self.meshes[mesh]["tangents"] is not None,
                             has_uvs=self.meshes[mesh].get("uvs") is not None))
        return dict(positions=np.concatenate(pos), normals=np.concatenate(nrm), tangents=np.concatenate(tan),
                    uvs=np.concatenate(uvs), indices=np.concatenate(idx), instances=inst)
