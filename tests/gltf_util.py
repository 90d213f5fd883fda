"""Writes small glTF 2.0 files for the loader tests: a PNG encoder (zlib, all five row
filters) and a scene with a textured cube under a two-level node hierarchy, a camera and a
KHR_lights_punctual spot light."""
import base64
import json
import struct
import zlib

import numpy as np


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def encode_png(px):
    """(h, w, c) uint8, c in 1..4 (grey, grey+alpha, RGB, RGBA) -> PNG bytes; row y uses filter y % 5."""
    h, w, c = px.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    raw = bytearray()
    prev = np.zeros(w * c, np.int32)
    for y in range(h):
        line = px[y].reshape(-1).astype(np.int32)
        f = y % 5
        out = np.zeros_like(line)
        for x in range(len(line)):
            a = line[x - c] if x >= c else 0
            b = prev[x]
            cc = prev[x - c] if x >= c else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, cc)][f]
            out[x] = (line[x] - pred) & 255
        raw.append(f)
        raw += bytes(out.astype(np.uint8))
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b""))


def cube_arrays():
    from yapt_gb300.configs import cuboid
    p, n, i = cuboid()
    uv = np.tile(np.float32([[0, 0], [1, 0], [1, 1], [0, 1]]), (len(p) // 4, 1))
    return p.astype(np.float32), n.astype(np.float32), uv, i.astype(np.uint32)


def write_scene(path, binary=False):
    """A floor quad and a textured cube (child of a translated, rotated parent), a camera and a
    spot light. Returns the texture pixels and the parameters written."""
    p, n, uv, idx = cube_arrays()
    fp = np.float32([[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, 2]])
    fn = np.tile(np.float32([0, 1, 0]), (4, 1))
    fi = np.uint32([0, 2, 1, 0, 3, 2])
    blobs = [p, n, uv, idx, fp, fn, fi]
    rng = np.random.default_rng(3)
    tex = rng.integers(0, 256, (8, 8, 4)).astype(np.uint8)
    tex[..., 3] = 255
    png = encode_png(tex)
    buf = bytearray()
    views = []
    for b in blobs + [np.frombuffer(png, np.uint8)]:
        while len(buf) % 4:
            buf.append(0)
        views.append(dict(buffer=0, byteOffset=len(buf), byteLength=b.nbytes))
        buf += b.tobytes()
    acc = [
        dict(bufferView=0, componentType=5126, count=len(p), type="VEC3"),
        dict(bufferView=1, componentType=5126, count=len(n), type="VEC3"),
        dict(bufferView=2, componentType=5126, count=len(uv), type="VEC2"),
        dict(bufferView=3, componentType=5125, count=len(idx), type="SCALAR"),
        dict(bufferView=4, componentType=5126, count=4, type="VEC3"),
        dict(bufferView=5, componentType=5126, count=4, type="VEC3"),
        dict(bufferView=6, componentType=5125, count=6, type="SCALAR"),
    ]
    g = {
        "asset": {"version": "2.0"},
        "extensionsUsed": ["KHR_lights_punctual", "KHR_materials_clearcoat", "KHR_materials_emissive_strength"],
        "buffers": [{"byteLength": len(buf)}],
        "bufferViews": views,
        "accessors": acc,
        "images": [{"bufferView": 7, "mimeType": "image/png"}],
        "textures": [{"source": 0}],
        "materials": [
            {"name": "cube", "pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.6, 0.4, 1.0], "metallicFactor": 0.0,
                                                     "roughnessFactor": 0.5, "baseColorTexture": {"index": 0}},
             "extensions": {"KHR_materials_clearcoat": {"clearcoatFactor": 0.7, "clearcoatRoughnessFactor": 0.1}}},
            {"name": "floor", "pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.5, 0.5, 1.0], "metallicFactor": 0.0},
             "emissiveFactor": [0.0, 0.0, 0.0], "doubleSided": True},
            {"name": "glow", "emissiveFactor": [1.0, 0.9, 0.8],
             "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 4.0}}},
        ],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3, "material": 0}]},
                   {"primitives": [{"attributes": {"POSITION": 4, "NORMAL": 5}, "indices": 6, "material": 1}]},
                   {"primitives": [{"attributes": {"POSITION": 4, "NORMAL": 5}, "indices": 6, "material": 2}]}],
        "cameras": [{"type": "perspective", "perspective": {"yfov": 0.9, "aspectRatio": 1.0, "znear": 0.1, "zfar": 100.0}}],
        "extensions": {"KHR_lights_punctual": {"lights": [{"type": "spot", "color": [1.0, 0.9, 0.7], "intensity": 3.0,
                                                           "spot": {"innerConeAngle": 0.3, "outerConeAngle": 0.6}}]}},
        "nodes": [
            {"name": "parent", "translation": [0.2, 0.5, -0.1], "rotation": [0.0, 0.3826834, 0.0, 0.9238795], "children": [1]},
            {"name": "cube", "mesh": 0, "scale": [0.5, 0.5, 0.5]},
            {"name": "floor", "mesh": 1},
            {"name": "lamp", "mesh": 2, "matrix": [1, 0, 0, 0, 0, -1, 0, 0, 0, 0, -1, 0, 0, 2.5, 0, 1]},
            {"name": "camera", "camera": 0, "translation": [0.0, 1.5, 4.0], "rotation": [-0.1305262, 0.0, 0.0, 0.9914449]},
            {"name": "spot", "translation": [1.0, 2.0, 1.0], "rotation": [-0.7071068, 0.0, 0.0, 0.7071068],
             "extensions": {"KHR_lights_punctual": {"light": 0}}},
        ],
        "scenes": [{"nodes": [0, 2, 3, 4, 5]}],
        "scene": 0,
    }
    if binary:
        js = json.dumps(g).encode()
        while len(js) % 4:
            js += b" "
        while len(buf) % 4:
            buf.append(0)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(buf), 0x004E4942) + bytes(buf)
        with open(path, "wb") as f:
            f.write(b"glTF" + struct.pack("<II", 2, 12 + len(body)) + body)
    else:
        g["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(bytes(buf)).decode()
        with open(path, "w") as f:
            json.dump(g, f)
    return tex
