"""glTF 2.0 scene loading into a :class:`yapt_gb300.scene.Scene`.

Follows the reference's loader (Source/Python/pythonScripts/yapt/scene_loader.py:29-421, with
mesh_utils.py for tangents): one instance per mesh primitive and node, node transforms composed
down the hierarchy, the first perspective camera, KHR_lights_punctual lights, and the material
mapping of ``_load_material_gltf`` (scene_loader.py:106-278): base colour, metallic and roughness
factors, emission with KHR_materials_emissive_strength, base colour / normal / emissive textures,
the metallic-roughness (or occlusion) texture as the ORM texture, alpha modes (MASK and cut-out
BLEND as an alpha cutoff, other BLEND as alpha-blended transparency), and the transmission,
specular, clearcoat, sheen, volume, iridescence and ior extensions.

Reads .gltf (buffers as files or data URIs) and .glb. Images: PNG (8-bit grey, grey+alpha, RGB,
RGBA; not interlaced), decoded here with zlib; JPEG and KTX images raise ValueError.
"""
import base64
import json
import math
import os
import struct
import zlib

import numpy as np

from . import _native as N
from .scene import CameraDesc, Scene

_COMPONENTS = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}
_DTYPES = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}


def decode_png(data):
    """PNG bytes -> (h, w, 4) uint8 RGBA (8-bit colour types 0, 2, 4, 6; no interlace)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG image")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + n
    w, h, depth, ctype, _, _, interlace = hdr
    channels = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if depth != 8 or channels is None or interlace:
        raise ValueError("PNG: only 8-bit grey/RGB(A) images without interlacing are supported")
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    stride = w * channels
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)].astype(np.int32)
        cur = np.zeros(stride, np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:  # 1: sub, 3: average, 4: Paeth, sequential over the row
            for x in range(stride):
                a = cur[x - channels] if x >= channels else 0
                b = prev[x]
                c = prev[x - channels] if x >= channels else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    px = out.reshape(h, w, channels).astype(np.uint8)
    if channels == 1:
        px = np.repeat(px, 3, axis=2)
    elif channels == 2:
        px = np.concatenate([np.repeat(px[..., :1], 3, axis=2), px[..., 1:]], axis=2)
    if px.shape[2] == 3:
        px = np.concatenate([px, np.full((h, w, 1), 255, np.uint8)], axis=2)
    return np.ascontiguousarray(px)


def _quat_to_matrix(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _node_matrix(node):
    if "matrix" in node:
        return np.array(node["matrix"], np.float64).reshape(4, 4).T  # column-major
    M = np.eye(4)
    R = _quat_to_matrix(node.get("rotation", [0, 0, 0, 1]))
    M[:3, :3] = R @ np.diag(node.get("scale", [1, 1, 1]))
    M[:3, 3] = node.get("translation", [0, 0, 0])
    return M


def compute_tangents(positions, indices, uvs, normals):
    """Per-vertex tangents from uv gradients (mesh_utils.py:12-60): accumulated per triangle,
    Gram-Schmidt against the normal, handedness in w; vertices without a usable uv gradient get
    a tangent perpendicular to the normal."""
    p, n, t = positions.astype(np.float64), normals.astype(np.float64), uvs.astype(np.float64)
    tan = np.zeros_like(p)
    bit = np.zeros_like(p)
    tri = indices.reshape(-1, 3)
    e1, e2 = p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]]
    d1, d2 = t[tri[:, 1]] - t[tri[:, 0]], t[tri[:, 2]] - t[tri[:, 0]]
    det = d1[:, 0] * d2[:, 1] - d2[:, 0] * d1[:, 1]
    ok = np.abs(det) > 1e-20
    r = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)[:, None]
    td = (e1 * d2[:, 1:2] - e2 * d1[:, 1:2]) * r
    bd = (e2 * d1[:, 0:1] - e1 * d2[:, 0:1]) * r
    for k in range(3):
        np.add.at(tan, tri[:, k], td)
        np.add.at(bit, tri[:, k], bd)
    tan = tan - n * np.sum(n * tan, axis=1, keepdims=True)
    ln = np.linalg.norm(tan, axis=1)
    fallback = np.cross(np.where(np.abs(n[:, 1:2]) < 0.9, [[0.0, 1.0, 0.0]], [[0.0, 0.0, 1.0]]), n)
    fallback /= np.maximum(np.linalg.norm(fallback, axis=1, keepdims=True), 1e-30)
    tan = np.where((ln > 1e-12)[:, None], tan / np.maximum(ln, 1e-30)[:, None], fallback)
    w = np.where(np.sum(np.cross(n, tan) * bit, axis=1) < 0, -1.0, 1.0)
    return np.concatenate([tan, w[:, None]], 1).astype(np.float32)


class _Loader:
    def __init__(self, path):
        self.dir = os.path.dirname(os.path.abspath(path))
        with open(path, "rb") as f:
            data = f.read()
        self.bin = None
        if data[:4] == b"glTF":
            length = struct.unpack("<I", data[8:12])[0]
            pos, js = 12, None
            while pos < length:
                n, kind = struct.unpack("<II", data[pos:pos + 8])
                chunk = data[pos + 8:pos + 8 + n]
                if kind == 0x4E4F534A:
                    js = json.loads(chunk.decode("utf-8"))
                elif kind == 0x004E4942:
                    self.bin = chunk
                pos += 8 + n
            self.g = js
        else:
            self.g = json.loads(data.decode("utf-8"))
        self.buffers = [self._buffer(b, i) for i, b in enumerate(self.g.get("buffers", []))]
        self.textures = {}

    def _uri(self, uri):
        if uri.startswith("data:"):
            return base64.b64decode(uri.split(",", 1)[1])
        with open(os.path.join(self.dir, uri), "rb") as f:
            return f.read()

    def _buffer(self, b, i):
        if "uri" not in b:
            return self.bin
        return self._uri(b["uri"])

    def accessor(self, i):
        a = self.g["accessors"][i]
        comps = _COMPONENTS[a["type"]]
        dt = np.dtype(_DTYPES[a["componentType"]])
        count = a["count"]
        if "bufferView" not in a:
            return np.zeros((count, comps), dt)
        v = self.g["bufferViews"][a["bufferView"]]
        buf = self.buffers[v["buffer"]]
        start = v.get("byteOffset", 0) + a.get("byteOffset", 0)
        stride = v.get("byteStride", 0) or comps * dt.itemsize
        raw = np.frombuffer(buf, np.uint8, count=(count - 1) * stride + comps * dt.itemsize, offset=start)
        rows = np.lib.stride_tricks.as_strided(raw, (count, comps * dt.itemsize), (stride, 1))
        out = np.ascontiguousarray(rows).view(dt).reshape(count, comps)
        if a.get("normalized") and dt.kind in "ui":
            out = out.astype(np.float32) / float(np.iinfo(dt).max)
        return out

    def image(self, ti, linear, sc):
        key = (ti, linear)
        if key in self.textures:
            return self.textures[key]
        tex = self.g["textures"][ti]
        img = self.g["images"][tex["source"]]
        mime = img.get("mimeType", "")
        if "bufferView" in img:
            v = self.g["bufferViews"][img["bufferView"]]
            data = bytes(self.buffers[v["buffer"]][v.get("byteOffset", 0):v.get("byteOffset", 0) + v["byteLength"]])
        else:
            data = self._uri(img["uri"])
            mime = mime or ("image/png" if img["uri"].lower().endswith(".png") else "")
        if data[:8] != b"\x89PNG\r\n\x1a\n":
            raise ValueError("glTF image %d: only PNG images can be decoded here (%s)" % (tex["source"], mime or "unknown"))
        px = decode_png(data)
        tid = sc.add_texture(px, N.YG_TEXTURE_RGBA8_UNORM if linear else N.YG_TEXTURE_RGBA8_SRGB)
        self.textures[key] = (tid, px)
        return self.textures[key]

    def material(self, mi, sc):
        """scene_loader.py:106-278 mapped onto this build's material parameters."""
        p = dict(albedo=(1.0, 1.0, 1.0), metalness=1.0, roughness=1.0, transparency=0.0)
        if mi is None:
            return sc.add_material(**p)
        m = self.g["materials"][mi]
        ext = m.get("extensions", {}) or {}
        strength = ext.get("KHR_materials_emissive_strength", {}).get("emissiveStrength", 1.0)
        if m.get("emissiveFactor"):
            p["emissive"] = tuple(c * strength for c in m["emissiveFactor"])
        if "emissiveTexture" in m:
            p["emissive_texture"] = self.image(m["emissiveTexture"]["index"], False, sc)[0]
        if "normalTexture" in m:
            p["normal_texture"] = self.image(m["normalTexture"]["index"], True, sc)[0]
        if "occlusionTexture" in m:
            p["orm_texture"] = self.image(m["occlusionTexture"]["index"], True, sc)[0]
        mask = N.YG_MATERIAL_TWO_SIDED if m.get("doubleSided") else 0
        pbr = m.get("pbrMetallicRoughness", {})
        color = pbr.get("baseColorFactor", [1, 1, 1, 1])
        p["albedo"] = tuple(color[:3])
        coverage, blended, transmission = 1.0, False, 0.0
        if "baseColorTexture" in pbr:
            tid, px = self.image(pbr["baseColorTexture"]["index"], False, sc)
            p["albedo_texture"] = tid
            min_alpha = px[..., 3].min() / 255.0
        else:
            min_alpha = 1.0
        mode = m.get("alphaMode", "OPAQUE")
        if mode == "MASK" and "baseColorTexture" in pbr:
            cutoff = m.get("alphaCutoff", 0.5)
            if min_alpha < cutoff:
                p["alpha_cutoff"] = cutoff
        elif mode == "BLEND":
            if min_alpha < 0.02:
                p["alpha_cutoff"] = 0.5
            elif min_alpha < 1.0 or (len(color) > 3 and color[3] < 1.0):
                coverage = color[3] if len(color) > 3 else 1.0
                if min_alpha < 1.0:
                    mask |= N.YG_MATERIAL_ALPHA_BLEND
                blended = True
        p["metalness"] = pbr.get("metallicFactor", 1.0)
        p["roughness"] = pbr.get("roughnessFactor", 1.0)
        if "metallicRoughnessTexture" in pbr:
            p["orm_texture"] = self.image(pbr["metallicRoughnessTexture"]["index"], True, sc)[0]
        if "KHR_materials_transmission" in ext:
            transmission = ext["KHR_materials_transmission"].get("transmissionFactor", 0.0)
            p["transparency"] = transmission
            vol = ext.get("KHR_materials_volume")
            if vol is None or vol.get("thicknessFactor", 0.0) == 0:
                mask |= N.YG_MATERIAL_TWO_SIDED
            else:
                mask &= ~N.YG_MATERIAL_TWO_SIDED
        if "KHR_materials_specular" in ext:
            p["specular_amount"] = ext["KHR_materials_specular"].get("specularFactor", 1.0)
        if "KHR_materials_clearcoat" in ext:
            cc = ext["KHR_materials_clearcoat"]
            p.update(clear_coat_amount=cc.get("clearcoatFactor", 0.0), clear_coat_roughness=cc.get("clearcoatRoughnessFactor", 0.0),
                     clear_coat_ior=1.5)
        if "KHR_materials_sheen" in ext:
            sh = ext["KHR_materials_sheen"]
            col = sh.get("sheenColorFactor", [0.0, 0.0, 0.0])
            amount = max(col)
            if amount > 0:
                r = sh.get("sheenRoughnessFactor", 0.0)
                p.update(sheen_amount=amount, sheen_tint=tuple(c / amount for c in col), sheen_roughness=r * r)
        if "KHR_materials_volume" in ext:
            vol = ext["KHR_materials_volume"]
            if vol.get("thicknessFactor", None) == 0:
                mask |= N.YG_MATERIAL_TWO_SIDED
            dist, col = vol.get("attenuationDistance", -1), vol.get("attenuationColor", [1, 1, 1])
            if dist > 0 and any(c != 1 for c in col):
                p["absorption"] = tuple(-math.log(c) / dist for c in col)
        if "KHR_materials_iridescence" in ext:
            ir = ext["KHR_materials_iridescence"]
            p.update(clear_coat_ior=ir.get("iridescenceIor", 1.3), clear_coat_amount=ir.get("iridescenceFactor", 0.0),
                     thin_film_thickness_nm=ir.get("iridescenceThicknessMaximum", 400))
        if "KHR_materials_ior" in ext:
            p["dielectric_ior"] = ext["KHR_materials_ior"].get("ior", 1.5)
        if blended:
            p["transparency"] = 1.0 - coverage * (1.0 - transmission)
            if transmission == 0.0:
                mask |= N.YG_MATERIAL_TWO_SIDED
        p["material_mask"] = mask
        return sc.add_material(**p)


def load(path, aspect=None):
    """Loads a .gltf or .glb file into a Scene (meshes, materials, textures, instances, the
    first perspective camera and KHR_lights_punctual lights)."""
    L = _Loader(path)
    g = L.g
    sc = Scene()
    sc.name = os.path.basename(path)
    materials = {}
    mesh_ids = {}

    def prim_mesh(mi, pi):
        key = (mi, pi)
        if key in mesh_ids:
            return mesh_ids[key]
        pr = g["meshes"][mi]["primitives"][pi]
        if pr.get("mode", 4) != 4:
            raise ValueError("mesh %d primitive %d: only triangle lists are supported" % (mi, pi))
        att = pr["attributes"]
        pos = L.accessor(att["POSITION"]).astype(np.float32)
        idx = L.accessor(pr["indices"]).reshape(-1).astype(np.uint32) if "indices" in pr else np.arange(len(pos), dtype=np.uint32)
        if "NORMAL" in att:
            nrm = L.accessor(att["NORMAL"]).astype(np.float32)
        else:  # flat normals from the triangles
            tri = idx.reshape(-1, 3)
            fn = np.cross(pos[tri[:, 1]] - pos[tri[:, 0]], pos[tri[:, 2]] - pos[tri[:, 0]])
            nrm = np.zeros_like(pos)
            for k in range(3):
                np.add.at(nrm, tri[:, k], fn)
            nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
        uvs = L.accessor(att["TEXCOORD_0"]).astype(np.float32) if "TEXCOORD_0" in att else None
        if "TANGENT" in att:
            tan = L.accessor(att["TANGENT"]).astype(np.float32)
        elif uvs is not None:
            tan = compute_tangents(pos, idx, uvs, nrm)
        else:
            from .configs import flat_tangents
            tan = flat_tangents(nrm)
        mesh_ids[key] = sc.add_mesh(pos, nrm, idx, tangents=tan, uvs=uvs)
        return mesh_ids[key]

    def material(mi):
        if mi not in materials:
            materials[mi] = L.material(mi, sc)
        return materials[mi]

    lights = g.get("extensions", {}).get("KHR_lights_punctual", {}).get("lights", [])
    camera = None

    def visit(ni, parent):
        nonlocal camera
        node = g["nodes"][ni]
        M = parent @ _node_matrix(node)
        if "mesh" in node:
            for pi, pr in enumerate(g["meshes"][node["mesh"]]["primitives"]):
                sc.add_instance(prim_mesh(node["mesh"], pi), material(pr.get("material")), M)
        if "camera" in node and camera is None:
            cam = g["cameras"][node["camera"]]
            if cam.get("type") == "perspective":
                pp = cam["perspective"]
                eye = M[:3, 3]
                fwd = -M[:3, 2] / np.linalg.norm(M[:3, 2])
                up = M[:3, 1] / np.linalg.norm(M[:3, 1])
                camera = CameraDesc(eye=tuple(eye), target=tuple(eye + fwd), up=tuple(up), fovy=pp["yfov"],
                                    aspect=aspect or pp.get("aspectRatio", 1.0), near=pp.get("znear", 0.1),
                                    far=pp.get("zfar", 1000.0))
        li = node.get("extensions", {}).get("KHR_lights_punctual", {}).get("light")
        if li is not None:
            d = lights[li]
            col = d.get("color", [1, 1, 1])
            inten = d.get("intensity", 1.0)
            fwd = -M[:3, 2] / max(np.linalg.norm(M[:3, 2]), 1e-30)
            kind = {"point": "point", "spot": "spot", "directional": "directional"}[d["type"]]
            spot = d.get("spot", {})
            sc.add_punctual_light(kind, position=tuple(M[:3, 3]), direction=tuple(fwd),
                                  intensity=tuple(c * inten for c in col),
                                  cos_inner=math.cos(spot.get("innerConeAngle", 0.0)),
                                  cos_outer=math.cos(spot.get("outerConeAngle", math.pi / 4)))
        for c in node.get("children", []):
            visit(c, M)

    scene_index = g.get("scene", 0)
    roots = g["scenes"][scene_index]["nodes"] if g.get("scenes") else range(len(g.get("nodes", [])))
    for ni in roots:
        visit(ni, np.eye(4))
    sc.camera = camera or CameraDesc(eye=(0.0, 0.0, 5.0), target=(0.0, 0.0, 0.0), aspect=aspect or 1.0)
    return sc
