"""Seeded synthetic scenes for the benchmark configurations.

There is no public dataset for this path; the scenes are generated from one
numpy PCG64 generator per configuration, with the shapes, sizes and value
distributions of the benchmark definitions:

* ``box_scene``      closed-on-5-sides unit box (10 triangles), two rotated inner boxes
                     (12 triangles each), a 0.25 x 0.25 ceiling quad light with a
                     D65-shaped spectrum, diffuse principled materials with 8-point
                     reflectance spectra U(0.05, 0.85) over 380..780 nm. The front (z = 1)
                     is open; the camera looks in from outside. Env.IntensityScale = 0.
* ``random_shapes_scene``  N icospheres (subdivision 2, 320 triangles) with centres
                     U([-10,10] x [0,4] x [-10,10]) (y up), radii U(0.2, 1.0), on a
                     40 x 40 ground quad, lit by 3 quad lights with blackbody spectra,
                     T ~ U(2700 K, 6500 K); roughness U(0.05, 1), metallic ~ Bernoulli(0.3),
                     20% dispersive dielectrics (Cauchy A = 1.5, B = 0.0042 um^2).
"""
import numpy as np

from . import _native as N
from .scene import (SPECTRUM_LMAX, SPECTRUM_LMIN, SPECTRUM_POINTS, CameraDesc, Scene, affine, rotation_x,
                    rotation_y)

GRID = np.linspace(SPECTRUM_LMIN, SPECTRUM_LMAX, SPECTRUM_POINTS)


def control_point_spectrum(rng, n=8, lo=0.05, hi=0.85):
    """Piecewise-linear reflectance through n seeded control points over 380..780 nm."""
    lam = np.linspace(SPECTRUM_LMIN, SPECTRUM_LMAX, n)
    vals = rng.uniform(lo, hi, size=n)
    return np.interp(GRID, lam, vals).astype(np.float32)


def blackbody_spectrum(T):
    """Planck's law sampled on the spectral grid, normalised to a peak of 1 in 380..780 nm."""
    h, c, k = 6.62607015e-34, 2.99792458e8, 1.380649e-23
    lam = GRID * 1e-9
    b = (2 * h * c * c) / (lam ** 5) / np.expm1(h * c / (lam * k * T))
    return (b / b.max()).astype(np.float32)


def quad(w, h):
    """Unit quad in the xz plane facing -y (a ceiling light), centred at the origin."""
    p = np.array([[-w / 2, 0, -h / 2], [w / 2, 0, -h / 2], [w / 2, 0, h / 2], [-w / 2, 0, h / 2]], np.float32)
    n = np.tile(np.float32([0, -1, 0]), (4, 1))
    # winding so that cross(p1 - p0, p2 - p0) points along -y
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    e = np.cross(p[1] - p[0], p[2] - p[0])
    if e[1] > 0:
        idx = np.array([0, 2, 1, 0, 3, 2], np.uint32)
    return p, n, idx


def cuboid():
    """Axis-aligned unit cube centred at the origin, 12 triangles, outward flat normals."""
    faces = []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sgn
            u = np.zeros(3)
            u[(axis + 1) % 3] = 1.0
            v = np.cross(n, u)
            c = n * 0.5
            corners = [c - u * 0.5 - v * 0.5, c + u * 0.5 - v * 0.5, c + u * 0.5 + v * 0.5, c - u * 0.5 + v * 0.5]
            faces.append((np.array(corners), n))
    pos, nrm, idx = [], [], []
    for (cs, n) in faces:
        b = len(pos)
        pos.extend(cs)
        nrm.extend([n] * 4)
        tri = [b, b + 1, b + 2, b, b + 2, b + 3]
        if np.dot(np.cross(cs[1] - cs[0], cs[2] - cs[0]), n) < 0:
            tri = [b, b + 2, b + 1, b, b + 3, b + 2]
        idx.extend(tri)
    return np.array(pos, np.float32), np.array(nrm, np.float32), np.array(idx, np.uint32)


def flat_tangents(normals):
    """One unit tangent per vertex, perpendicular to its normal (w = 1). The shading frame is
    built from the normal and the tangent (constructBasisTransform, commonMath.hlsl:124-129);
    a mesh without tangents gets (1, 0, 0) (hitShadersCommon.hlsl:197), which is parallel to
    a face whose normal is +-x and leaves that frame degenerate (NaN), so the box walls and
    cuboids carry tangents, as meshes loaded by the reference's asset scripts do
    (pythonScripts/yapt/mesh_utils.py:12-60)."""
    n = np.asarray(normals, np.float64).reshape(-1, 3)
    a = np.where(np.abs(n[:, 1:2]) < 0.9, [[0.0, 1.0, 0.0]], [[0.0, 0.0, 1.0]])
    t = np.cross(a, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    return np.concatenate([t, np.ones((len(t), 1))], 1).astype(np.float32)


def scaled_cuboid(sc, size):
    """A cuboid mesh with its extent in the vertices, so that its instance transform stays a
    rotation and translation. The reference samples and evaluates BSDFs in object space and
    maps directions with the object-to-world matrix in the path tracers
    (rayHitDefault.hlsl:429-431) but with the normal matrix in BDPT
    (BDPTTraceLightPath.comp:182-185, 324); under a non-uniform scale the integrators then
    estimate slightly different images, so the synthetic scenes keep instance scales uniform."""
    p, n, i = cuboid()
    p = (p * np.asarray(size, np.float32)).astype(np.float32)
    return sc.add_mesh(p, n, i, tangents=flat_tangents(n))


def icosphere(subdiv=2):
    """Unit icosphere: 20 * 4^subdiv triangles, outward winding, smooth normals."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, float) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
             (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    pos = np.array(verts, np.float32)
    idx = []
    for (a, b, c) in faces:
        n = np.cross(pos[b] - pos[a], pos[c] - pos[a])
        if np.dot(n, pos[a] + pos[b] + pos[c]) < 0:
            b, c = c, b
        idx += [a, b, c]
    return pos, pos.copy(), np.array(idx, np.uint32)


def diffuse(spectrum_id):
    # diffuse principled layer set as in the reference's test scenes
    # (Tests/IntegratorCompare/focused_emission_scene.py:52-56): no metal, no specular, rough
    return dict(albedo=(0.5, 0.5, 0.5), albedo_spectrum=spectrum_id, metalness=0.0, transparency=0.0,
                specular_amount=0.0, roughness=1.0)


def box_scene(seed=0, light_intensity=12.0, aspect=1.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene()
    sc.name = "box(seed=%d)" % seed
    # the five walls: floor, ceiling, back, left, right; normals point into the box
    wall_defs = [((0.5, 0.0, 0.5), (0, 1, 0)), ((0.5, 1.0, 0.5), (0, -1, 0)), ((0.5, 0.5, 0.0), (0, 0, 1)),
                 ((0.0, 0.5, 0.5), (1, 0, 0)), ((1.0, 0.5, 0.5), (-1, 0, 0))]
    pos, nrm, idx = [], [], []
    for (c, n) in wall_defs:
        c, n = np.array(c, float), np.array(n, float)
        u = np.array([1.0, 0, 0]) if abs(n[0]) < 0.5 else np.array([0, 0, 1.0])
        v = np.cross(n, u)
        cs = [c - 0.5 * u - 0.5 * v, c + 0.5 * u - 0.5 * v, c + 0.5 * u + 0.5 * v, c - 0.5 * u + 0.5 * v]
        b = len(pos)
        pos.extend(cs)
        nrm.extend([n] * 4)
        tri = [b, b + 1, b + 2, b, b + 2, b + 3]
        if np.dot(np.cross(cs[1] - cs[0], cs[2] - cs[0]), n) < 0:
            tri = [b, b + 2, b + 1, b, b + 3, b + 2]
        idx.extend(tri)
    walls = sc.add_mesh(np.array(pos), np.array(nrm), np.array(idx), submeshes=[(6 * i, 6) for i in range(5)],
                        tangents=flat_tangents(nrm))
    for i in range(5):
        sid = sc.add_spectrum(control_point_spectrum(rng))
        mat = sc.add_material(**diffuse(sid))
        sc.add_instance(walls, mat, submesh=i)
    for k in range(2):
        sid = sc.add_spectrum(control_point_spectrum(rng))
        mat = sc.add_material(**diffuse(sid))
        h = rng.uniform(0.25, 0.6)
        w = rng.uniform(0.18, 0.3)
        x = 0.3 if k == 0 else 0.7
        z = rng.uniform(0.3, 0.6)
        o2w = affine(translation=(x, h / 2, z), rotation=rotation_y(rng.uniform(0, np.pi)))
        sc.add_instance(scaled_cuboid(sc, (w, h, w)), mat, o2w)
    qp, qn, qi = quad(0.25, 0.25)
    light = sc.add_mesh(qp, qn, qi)
    lmat = sc.add_material(albedo=(0.0, 0.0, 0.0), emissive=(light_intensity,) * 3, metalness=0.0, specular_amount=0.0,
                           roughness=1.0)
    sc.add_instance(light, lmat, affine(translation=(0.5, 0.999, 0.5)))
    sc.camera = CameraDesc(eye=(0.5, 0.5, 2.1), target=(0.5, 0.5, 0.0), fovy=np.pi * 0.22, aspect=aspect)
    return sc


def layered_box_scene(seed=0, light_intensity=12.0, aspect=1.0):
    """``box_scene`` with the principled BSDF's layered lobes switched on: a sheen floor, a
    clear-coated plastic back wall, a brushed (anisotropic, rotated tangent frame) metal
    block and a clear-coated metal block under a thin film, so that every layer of the
    reference's BSDF (Shaders/Bsdfs/layeredBsdf.hlsl, miscBrdf.hlsl, thinFilm.hlsl) carries
    energy into the image. Materials 0..4 are the walls, 5 and 6 the blocks, 7 the light."""
    sc = box_scene(seed, light_intensity, aspect)
    sc.name = "layered_box(seed=%d)" % seed
    m = sc.materials
    m[0].update(sheen_amount=0.8, sheen_tint=(0.9, 0.6, 0.3), sheen_roughness=0.35)
    m[2].update(clear_coat_amount=1.0, clear_coat_ior=1.6, clear_coat_roughness=0.05, roughness=0.6)
    m[5].update(metalness=1.0, roughness=0.35, specular=(0.95, 0.8, 0.6), specular_amount=1.0,
                anisotropy=0.7, anisotropy_rotation=0.2)
    m[6].update(metalness=1.0, roughness=0.2, specular=(0.9, 0.9, 0.9), specular_amount=1.0,
                clear_coat_amount=1.0, clear_coat_ior=1.45, clear_coat_roughness=0.1, thin_film_thickness_nm=420.0)
    return sc


def subsurface_box_scene(seed=0, light_intensity=12.0, aspect=1.0):
    """``box_scene`` whose two blocks scatter below their surfaces (the Christensen-Burley
    subsurface layer of subsurface.hlsl): one a pale, fully subsurface block with an RGB mean
    free path of (1.0, 0.5, 0.25) x 0.06 under a glossy specular layer, the other a half
    subsurface, half diffuse block with a clear coat and sheen and a grey radius of 0.02, plus
    three subsurface icospheres (subdivision 3) on the floor. Closed meshes, so every probe ray
    finds the surface it starts in."""
    sc = box_scene(seed, light_intensity, aspect)
    sc.name = "subsurface_box(seed=%d)" % seed
    m = sc.materials
    m[5].update(albedo_spectrum=-1, albedo=(0.85, 0.55, 0.4), subsurface_amount=1.0, subsurface_radius=(1.0, 0.5, 0.25),
                subsurface_radius_scale=0.06, specular_amount=0.5, roughness=0.35, dielectric_ior=1.4)
    m[6].update(subsurface_amount=0.5, subsurface_radius=(1.0, 1.0, 1.0), subsurface_radius_scale=0.02,
                clear_coat_amount=0.6, clear_coat_roughness=0.2, sheen_amount=0.4, sheen_roughness=0.5)
    rng = np.random.Generator(np.random.PCG64(2000 + seed))
    ball = sc.add_mesh(*icosphere(3))
    for k in range(3):
        mat = sc.add_material(**diffuse(sc.add_spectrum(control_point_spectrum(rng))))
        sc.materials[mat].update(subsurface_amount=1.0, subsurface_radius=tuple(rng.uniform(0.3, 1.0, 3)),
                                 subsurface_radius_scale=0.04, specular_amount=0.3, roughness=0.5)
        r = 0.07
        sc.add_instance(ball, mat, affine(translation=(0.2 + 0.3 * k, r, 0.8), scale=(r, r, r)))
    return sc


def textured_box_scene(seed=0, aspect=1.0):
    """``box_scene`` with textures in every material slot the reference has
    (materialsCommon.hlsl:354-397): an 8 x 8 checker albedo (sRGB, uv scale 3) on the floor,
    a bump normal map plus an occlusion/roughness/metalness map (linear) on a metallic back
    wall, and an emission gradient on the ceiling light. Quad faces get uv (0,0)-(1,1)."""
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    sc = box_scene(seed, aspect=aspect)
    sc.name = "textured_box(seed=%d)" % seed
    for m in sc.meshes:
        m["uvs"] = np.tile(np.float32([[0, 0], [1, 0], [1, 1], [0, 1]]), (len(m["positions"]) // 4, 1))
    ij = np.indices((64, 64)).sum(axis=0) // 8
    c0, c1 = rng.integers(40, 250, 3), rng.integers(40, 250, 3)
    checker = np.where((ij % 2 == 0)[..., None], c0, c1).astype(np.uint8)
    checker = np.concatenate([checker, np.full((64, 64, 1), 255, np.uint8)], axis=2)
    y, x = np.mgrid[0:32, 0:32] / 32.0
    nx, ny = 0.35 * np.cos(2 * np.pi * 3 * x), 0.35 * np.sin(2 * np.pi * 2 * y)
    n = np.stack([nx, ny, np.ones_like(nx)], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    normal = np.concatenate([np.round((n * 0.5 + 0.5) * 255), np.full((32, 32, 1), 255)], -1).astype(np.uint8)
    orm = np.stack([0.5 + 0.5 * x, 0.3 + 0.7 * y, (x > 0.5).astype(float), np.ones_like(x)], -1)
    orm = np.round(orm * 255).astype(np.uint8)
    glow = np.stack([0.3 + 0.7 * x[:16, :16] * 2, np.full((16, 16), 0.8), 0.5 + 0.5 * y[:16, :16] * 2, np.ones((16, 16))], -1)
    glow = np.round(np.clip(glow, 0, 1) * 255).astype(np.uint8)
    t_checker = sc.add_texture(checker)
    t_normal = sc.add_texture(normal, N.YG_TEXTURE_RGBA8_UNORM)
    t_orm = sc.add_texture(orm, N.YG_TEXTURE_RGBA8_UNORM)
    t_glow = sc.add_texture(glow, N.YG_TEXTURE_RGBA8_UNORM)
    m = sc.materials
    m[0].update(albedo_spectrum=-1, albedo=(0.9, 0.9, 0.9), albedo_texture=t_checker, albedo_uv_scale=(3.0, 3.0))
    m[2].update(metalness=1.0, specular=(0.9, 0.85, 0.8), specular_amount=1.0, roughness=0.6, normal_texture=t_normal,
                orm_texture=t_orm)
    m[7].update(emissive_texture=t_glow)
    return sc


def cutout_box_scene(seed=0, cutoff=0.5, aspect=1.0):
    """``box_scene`` with two alpha-tested panels (the reference's alpha cutoff, applied in the
    any-hit stage by alphaTestPasses, hitShadersCommon.hlsl:162-183): a two-sided vertical
    screen with round holes between the camera and the blocks, and a grate of slots just
    under the ceiling light, so that camera, bounce and shadow rays all pass through
    cutouts. Their albedo texture's alpha is 0 in the holes and 1 elsewhere, with a soft
    edge; the panels are the last two instances, material ids 8 and 9."""
    sc = box_scene(seed, aspect=aspect)
    sc.name = "cutout_box(seed=%d, cutoff=%g)" % (seed, cutoff)
    uv = np.float32([[0, 0], [1, 0], [1, 1], [0, 1]])
    y, x = (np.mgrid[0:64, 0:64] + 0.5) / 64.0
    r = np.hypot(x - 0.5, y - 0.5)
    holes = np.clip((r - 0.3) / 0.06, 0.0, 1.0)
    screen = np.stack([0.2 + 0.6 * x, 0.5 + 0.0 * x, 0.8 - 0.5 * y, holes], -1)
    slots = np.clip(np.abs(x - 0.5) * 8.0 - 1.0, 0.0, 1.0)
    grate = np.stack([0.6 + 0.0 * x, 0.6 + 0.0 * x, 0.6 + 0.0 * x, slots], -1)
    t_screen = sc.add_texture(np.round(screen * 255).astype(np.uint8), N.YG_TEXTURE_RGBA8_UNORM)
    t_grate = sc.add_texture(np.round(grate * 255).astype(np.uint8), N.YG_TEXTURE_RGBA8_UNORM)
    qp, qn, qi = quad(0.7, 0.6)
    screen_mesh = sc.add_mesh(qp, qn, qi, tangents=flat_tangents(qn), uvs=uv)
    m_screen = sc.add_material(albedo=(0.8, 0.8, 0.8), metalness=0.0, transparency=0.0, specular_amount=0.0,
                               roughness=1.0, albedo_texture=t_screen, albedo_uv_scale=(3.0, 2.0), alpha_cutoff=cutoff,
                               material_mask=N.YG_MATERIAL_TWO_SIDED)
    # the xz quad turned to face +z, at z = 0.85
    sc.add_instance(screen_mesh, m_screen, affine(translation=(0.5, 0.45, 0.85), rotation=rotation_x(-np.pi / 2)))
    qp, qn, qi = quad(0.4, 0.4)
    grate_mesh = sc.add_mesh(qp, qn, qi, tangents=flat_tangents(qn), uvs=uv)
    m_grate = sc.add_material(albedo=(0.6, 0.6, 0.6), metalness=0.0, transparency=0.0, specular_amount=0.0,
                              roughness=1.0, albedo_texture=t_grate, albedo_uv_scale=(2.0, 1.0), alpha_cutoff=cutoff,
                              material_mask=N.YG_MATERIAL_TWO_SIDED)
    sc.add_instance(grate_mesh, m_grate, affine(translation=(0.5, 0.93, 0.5)))
    return sc


def environment_sky_scene(seed=0, aspect=1.0):
    """``sky_scene`` under a longitude-latitude environment map (getSkyBoxColor with
    ENVIRONMENT_TYPE_LONGLAT): a float RGBA gradient sky with a warm band near the horizon."""
    sc = sky_scene(seed, aspect=aspect)
    sc.name = "environment_sky(seed=%d)" % seed
    v, u = np.mgrid[0:32, 0:64] / np.array([32.0, 64.0])[:, None, None]
    sky = np.stack([0.4 + 0.6 * np.exp(-((v - 0.5) / 0.1) ** 2) + 0.2 * u, 0.5 + 0.3 * (1 - v), 0.9 - 0.5 * v, np.ones_like(u)],
                   -1).astype(np.float32)
    sc.env_texture = sc.add_texture(sky)
    return sc


def cube_sky_scene(seed=0, aspect=1.0, face=16):
    """``sky_scene`` under a cube-map environment (getSkyBoxColor with ENVIRONMENT_TYPE_CUBE):
    six float RGBA faces, each a distinct tint with a gradient across it, so that the face
    selection and the in-face coordinates both show in the image."""
    sc = sky_scene(seed, aspect=aspect)
    sc.name = "cube_sky(seed=%d)" % seed
    t, s = (np.mgrid[0:face, 0:face] + 0.5) / face
    tints = [(1.0, 0.5, 0.4), (0.4, 1.0, 0.5), (0.9, 0.9, 1.2), (0.3, 0.25, 0.2), (0.5, 0.6, 1.0), (1.0, 0.8, 0.3)]
    faces = [np.stack([r * (0.6 + 0.4 * s), g * (0.6 + 0.4 * t), b * (1.0 - 0.3 * s * t), np.ones_like(s)], -1)
             for (r, g, b) in tints]
    sc.env_texture = sc.add_texture(np.concatenate(faces, 0).astype(np.float32))
    sc.env_cube = True
    return sc


def punctual_box_scene(seed=0, area_light=True, aspect=1.0):
    """``box_scene`` lit by punctual lights (LightManager's point, spot and directional
    lights): a point light in the upper left, a spot light under the ceiling aimed at the
    floor (inner 20, outer 35 degrees) and a directional light entering through the open
    front; the ceiling's area light stays unless ``area_light`` is False."""
    sc = box_scene(seed, aspect=aspect)
    sc.name = "punctual_box(seed=%d%s)" % (seed, "" if area_light else ", no area light")
    if not area_light:
        sc.instances.pop()  # the ceiling light quad is the last instance
    sc.add_punctual_light("point", position=(0.25, 0.8, 0.6), intensity=(0.35, 0.3, 0.22))
    sc.add_punctual_light("spot", position=(0.7, 0.95, 0.45), direction=(0.0, -1.0, 0.1), intensity=(1.2, 1.1, 0.9),
                          cos_inner=float(np.cos(np.radians(20.0))), cos_outer=float(np.cos(np.radians(35.0))))
    sc.add_punctual_light("directional", direction=(-0.3, -0.45, -1.0), intensity=(0.5, 0.55, 0.65))
    return sc


def random_shapes_scene(seed=0, n_spheres=500, light_intensity=25.0, aspect=1.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene()
    sc.name = "random_shapes(seed=%d, n=%d)" % (seed, n_spheres)
    ico = sc.add_mesh(*icosphere(2))
    for _ in range(n_spheres):
        c = (rng.uniform(-10, 10), rng.uniform(0, 4), rng.uniform(-10, 10))
        r = rng.uniform(0.2, 1.0)
        rough = rng.uniform(0.05, 1.0)
        metallic = rng.uniform() < 0.3
        dielectric = (not metallic) and rng.uniform() < (0.2 / 0.7)
        sid = sc.add_spectrum(control_point_spectrum(rng))
        if metallic:
            mat = sc.add_material(albedo=(0.8, 0.8, 0.8), albedo_spectrum=sid, specular=(1.0, 1.0, 1.0), metalness=1.0,
                                  roughness=rough)
        elif dielectric:
            mat = sc.add_material(albedo=(1.0, 1.0, 1.0), transparency=1.0, metalness=0.0, specular_amount=1.0,
                                  roughness=rough, material_mask=2, cauchy=(1.5, 0.0042), dielectric_ior=1.5)
        else:
            mat = sc.add_material(albedo=(0.5, 0.5, 0.5), albedo_spectrum=sid, metalness=0.0, specular_amount=1.0,
                                  roughness=rough)
        sc.add_instance(ico, mat, affine(translation=c, scale=(r, r, r)))
    gp, gn, gi = quad(40.0, 40.0)
    gn = -gn
    gi = gi[[0, 2, 1, 3, 5, 4]]
    ground = sc.add_mesh(gp, gn, gi)
    gsid = sc.add_spectrum(control_point_spectrum(rng))
    sc.add_instance(ground, sc.add_material(**diffuse(gsid)))
    lp, ln, li = quad(3.0, 3.0)
    light = sc.add_mesh(lp, ln, li)
    for k in range(3):
        T = rng.uniform(2700.0, 6500.0)
        sid = sc.add_spectrum(blackbody_spectrum(T))
        lmat = sc.add_material(albedo=(0.0, 0.0, 0.0), emissive=(light_intensity,) * 3, emission_spectrum=sid,
                               metalness=0.0, specular_amount=0.0, roughness=1.0)
        pos = (rng.uniform(-8, 8), rng.uniform(7, 9), rng.uniform(-8, 8))
        sc.add_instance(light, lmat, affine(translation=pos))
    sc.camera = CameraDesc(eye=(0.0, 7.0, 19.0), target=(0.0, 1.0, 0.0), fovy=np.pi * 0.3, aspect=aspect)
    return sc


def caustic_box_scene(seed=0, n_spheres=150, n_lights=10, sphere_subdiv=3, light_intensity=12.0,
                      sphere_light_intensity=3.0, aspect=1.0):
    """The box layout of ``box_scene`` (same seed, same walls, blocks and ceiling light) filled
    with ``n_spheres`` small icospheres, 60% of them dispersive dielectrics (Cauchy A = 1.5,
    B = 0.0042 um^2; half of those smooth, half with roughness U(0.05, 0.3)) and 40% diffuse,
    plus ``n_lights`` emissive spheres of radius 0.05 with a D65-shaped spectrum. With the
    defaults the scene holds about 196k triangles."""
    sc = box_scene(seed, light_intensity=light_intensity, aspect=aspect)
    sc.name = "caustic_box(seed=%d, n=%d)" % (seed, n_spheres)
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    ball = sc.add_mesh(*icosphere(sphere_subdiv))
    for _ in range(n_spheres):
        r = rng.uniform(0.03, 0.08)
        c = (rng.uniform(0.05 + r, 0.95 - r), rng.uniform(r, 0.85), rng.uniform(0.05 + r, 0.95 - r))
        if rng.uniform() < 0.6:
            rough = 0.0 if rng.uniform() < 0.5 else rng.uniform(0.05, 0.3)
            mat = sc.add_material(albedo=(1.0, 1.0, 1.0), transparency=1.0, metalness=0.0, specular_amount=1.0,
                                  roughness=rough, material_mask=2, cauchy=(1.5, 0.0042), dielectric_ior=1.5)
        else:
            mat = sc.add_material(**diffuse(sc.add_spectrum(control_point_spectrum(rng))))
        sc.add_instance(ball, mat, affine(translation=c, scale=(r, r, r)))
    bulb = sc.add_mesh(*icosphere(2))
    lmat = sc.add_material(albedo=(0.0, 0.0, 0.0), emissive=(sphere_light_intensity,) * 3, metalness=0.0,
                           specular_amount=0.0, roughness=1.0)
    for _ in range(n_lights):
        c = (rng.uniform(0.1, 0.9), rng.uniform(0.6, 0.9), rng.uniform(0.1, 0.9))
        sc.add_instance(bulb, lmat, affine(translation=c, scale=(0.05, 0.05, 0.05)))
    return sc


def sky_scene(seed=0, aspect=1.0):
    """No lights: a diffuse ground quad and three diffuse blocks under the analytic sky of the
    reference's miss shader (|dir| x Env.IntensityScale), for the environment light paths."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sc = Scene()
    sc.name = "sky(seed=%d)" % seed
    gp, gn, gi = quad(6.0, 6.0)
    gn = -gn
    gi = gi[[0, 2, 1, 3, 5, 4]]
    ground = sc.add_mesh(gp, gn, gi)
    sc.add_instance(ground, sc.add_material(**diffuse(sc.add_spectrum(control_point_spectrum(rng)))))
    for k in range(3):
        mat = sc.add_material(**diffuse(sc.add_spectrum(control_point_spectrum(rng))))
        h = rng.uniform(0.5, 1.5)
        o2w = affine(translation=(-1.2 + 1.2 * k, h / 2, rng.uniform(-0.5, 0.5)), rotation=rotation_y(rng.uniform(0, np.pi)))
        sc.add_instance(scaled_cuboid(sc, (0.6, h, 0.6)), mat, o2w)
    sc.camera = CameraDesc(eye=(0.0, 2.5, 5.0), target=(0.0, 0.5, 0.0), fovy=np.pi * 0.3, aspect=aspect)
    return sc


SERVE_TRIANGLES = (10_000, 21_000, 45_000, 96_000, 205_000, 437_000, 935_000, 2_000_000)


def serve_scene(variant, target_triangles=None):
    """Serving-configuration scene: the ``box_scene`` layout (seed = variant) filled with diffuse
    and dielectric icospheres (subdivision 3, 1280 triangles) until it holds about
    ``target_triangles`` (default SERVE_TRIANGLES[variant]: 10k to 2M over the 8 variants)."""
    target = SERVE_TRIANGLES[variant] if target_triangles is None else int(target_triangles)
    sc = box_scene(variant)
    sc.name = "serve(variant=%d, ~%d triangles)" % (variant, target)
    rng = np.random.Generator(np.random.PCG64(1000 + variant))
    base = sc.triangle_count()
    n = max(0, int(round((target - base) / 1280.0)))
    ball = sc.add_mesh(*icosphere(3))
    mats = [sc.add_material(**diffuse(sc.add_spectrum(control_point_spectrum(rng)))) for _ in range(6)]
    mats.append(sc.add_material(albedo=(1.0, 1.0, 1.0), transparency=1.0, metalness=0.0, specular_amount=1.0,
                                roughness=0.1, material_mask=2, cauchy=(1.5, 0.0042), dielectric_ior=1.5))
    r = float(np.clip(0.35 / max(n, 1) ** (1.0 / 3.0), 0.004, 0.06))
    for _ in range(n):
        c = (rng.uniform(0.05, 0.95), rng.uniform(0.02, 0.8), rng.uniform(0.05, 0.95))
        sc.add_instance(ball, mats[int(rng.integers(len(mats)))], affine(translation=c, scale=(r, r, r)))
    return sc
