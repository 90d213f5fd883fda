"""ctypes bridge to the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline, never by the product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")

import sys  # noqa: E402

sys.path.insert(0, ROOT)
from yapt_gb300 import _native as N  # noqa: E402  (struct layouts of include/yapt_gpu.h)


class OracleInstance(C.Structure):
    _fields_ = [("o2w", C.c_float * 12), ("w2o", C.c_float * 12), ("first_index", C.c_uint32),
                ("prim_count", C.c_uint32), ("vertex_base", C.c_uint32), ("material", C.c_uint32),
                ("has_tangents", C.c_uint32), ("has_uvs", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class OracleTexture(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32),
                ("reserved", C.c_uint32)]


class OracleScene(C.Structure):
    _fields_ = [("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("tangents", C.POINTER(C.c_float)), ("indices", C.POINTER(C.c_uint32)),
                ("instances", C.POINTER(OracleInstance)), ("n_instances", C.c_uint32),
                ("materials", C.POINTER(N.Material)), ("n_materials", C.c_uint32),
                ("spectra", C.POINTER(C.c_float)), ("spec_points", C.c_uint32), ("spec_lmin", C.c_float),
                ("spec_lmax", C.c_float), ("camera", C.POINTER(N.Camera)), ("luts", C.POINTER(C.c_float) * 9),
                ("rgb_to_spd", C.POINTER(C.c_float)), ("data_dir", C.c_char_p),
                ("punctual", C.POINTER(N.PunctualLight)), ("n_punctual", C.c_uint32),
                ("uvs", C.POINTER(C.c_float)), ("textures", C.POINTER(OracleTexture)), ("n_textures", C.c_uint32),
                ("env_texture", C.c_uint32), ("env_cube", C.c_uint32)]


class OracleStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("seconds", C.c_double)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        lib.oracle_render.restype = C.c_int
        lib.oracle_render.argtypes = [C.POINTER(OracleScene), C.POINTER(N.RenderParams), C.c_int, C.c_int, C.c_void_p,
                                      C.c_void_p, C.POINTER(OracleStats)]
        lib.oracle_atrous_moments.restype = C.c_int
        lib.oracle_atrous_moments.argtypes = [C.POINTER(OracleScene), C.POINTER(N.RenderParams), C.c_int, C.c_void_p]
        lib.oracle_atrous.restype = C.c_int
        lib.oracle_atrous.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(N.Camera),
                                      C.POINTER(N.AtrousParams), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_render_strided.restype = C.c_int
        lib.oracle_render_strided.argtypes = [C.POINTER(OracleScene), C.POINTER(N.RenderParams), C.c_uint32, C.c_int,
                                              C.c_int, C.c_void_p, C.POINTER(OracleStats)]
        lib.oracle_needs_rgb_table.restype = C.c_int
        lib.oracle_needs_rgb_table.argtypes = [C.POINTER(OracleScene), C.POINTER(N.RenderParams)]
        lib.oracle_host_table.restype = C.c_int
        lib.oracle_host_table.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_size_t,
                                          C.POINTER(C.c_size_t)]
        lib.oracle_sobol_matrices.restype = C.c_int
        lib.oracle_sobol_matrices.argtypes = [C.c_char_p, C.c_void_p]
        _lib = lib
    return _lib


def sobol_matrices():
    out = np.zeros(256 * 32, np.uint32)
    rc = load().oracle_sobol_matrices(N.DATA_DIR.encode(), out.ctypes.data_as(C.c_void_p))
    assert rc == 0
    return out


LUT_NAMES = ["ss", "ss_avg", "ssms", "ssms_avg", "trans_denser", "trans_lighter", "trans_avg_denser",
             "trans_avg_lighter", "sheen"]


def host_table(name, lambda_range=(380, 700)):
    """A precomputed table generated by the oracle library itself (no GPU library loaded):
    "sobol", one of LUT_NAMES, or "rgb_to_spd" for the spectral range."""
    which = N.TABLES[name]
    n = C.c_size_t()
    lib = load()
    lo, hi = int(lambda_range[0]), int(lambda_range[1])
    if lib.oracle_host_table(N.DATA_DIR.encode(), which, lo, hi, None, 0, C.byref(n)) != 0:
        raise RuntimeError("oracle_host_table(%s) failed" % name)
    out = np.zeros(n.value, dtype=np.uint32 if name == "sobol" else np.float32)
    if lib.oracle_host_table(N.DATA_DIR.encode(), which, lo, hi, out.ctypes.data_as(C.c_void_p), out.size, C.byref(n)) != 0:
        raise RuntimeError("oracle_host_table(%s) failed" % name)
    return out


def own_luts():
    """The nine multiple-scattering / sheen LUTs, generated by the oracle library."""
    return {n: host_table(n) for n in LUT_NAMES}


def render_params(integrator="nee", width=64, height=64, spp_start=0, spp=1, max_depth=8, lambda_range=(380.0, 700.0),
                  crop=None, regularize_after=8, regularize=True, env_scale=0.0, seed=0, flags=0, light_paths=0,
                  light_vertices=0):
    """A yg_render_params request (struct layout of include/yapt_gpu.h), built without the
    GPU library."""
    p = N.RenderParams()
    p.integrator = N.INTEGRATORS[integrator] if isinstance(integrator, str) else int(integrator)
    p.width, p.height = int(width), int(height)
    p.spp_start, p.spp_count = int(spp_start), int(spp)
    p.max_depth = int(max_depth)
    p.regularize_after_vertices = int(regularize_after)
    p.regularize_enable = 1 if regularize else 0
    p.env_intensity_scale = float(env_scale)
    p.seed = int(seed)
    p.flags = int(flags)
    if crop is not None:
        p.crop_x, p.crop_y, p.crop_w, p.crop_h = [int(v) for v in crop]
    p.lambda_min, p.lambda_max = float(lambda_range[0]), float(lambda_range[1])
    p.bdpt_light_paths = int(light_paths)
    p.bdpt_light_vertices = int(light_vertices)
    return p


class OracleSceneHandle:
    """Keeps the numpy buffers alive while the oracle reads them."""

    def __init__(self, scene, luts, rgb_to_spd=None):
        pool = scene.pooled()
        self.keep = []

        def fp(a, dt=np.float32):
            a = np.ascontiguousarray(np.asarray(a, dtype=dt))
            self.keep.append(a)
            return a

        pos, nrm, tan = fp(pool["positions"]), fp(pool["normals"]), fp(pool["tangents"])
        idx = fp(pool["indices"], np.uint32)
        ninst = len(pool["instances"])
        inst = (OracleInstance * max(1, ninst))()
        for i, d in enumerate(pool["instances"]):
            a = np.asarray(d["o2w"][:3, :], np.float32).reshape(-1)
            b = np.asarray(np.linalg.inv(d["o2w"])[:3, :], np.float32).reshape(-1)
            for k in range(12):
                inst[i].o2w[k] = float(a[k])
                inst[i].w2o[k] = float(b[k])
            inst[i].first_index = d["first_index"]
            inst[i].prim_count = d["prim_count"]
            inst[i].vertex_base = d["vertex_base"]
            inst[i].material = d["material"]
            inst[i].has_tangents = 1 if d["has_tangents"] else 0
            inst[i].has_uvs = 1 if d["has_uvs"] else 0
        mats = scene.material_structs()
        spec = fp(scene.spectra_array() if len(scene.spectra) else np.zeros((1, 81), np.float32))
        cam = scene.camera.struct()
        s = OracleScene()
        s.positions = pos.ctypes.data_as(C.POINTER(C.c_float))
        s.normals = nrm.ctypes.data_as(C.POINTER(C.c_float))
        s.tangents = tan.ctypes.data_as(C.POINTER(C.c_float))
        s.indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
        s.instances = inst
        s.n_instances = ninst
        s.materials = mats
        s.n_materials = len(scene.materials)
        s.spectra = spec.ctypes.data_as(C.POINTER(C.c_float))
        s.spec_points = 81
        s.spec_lmin, s.spec_lmax = 380.0, 780.0
        s.camera = C.pointer(cam)
        for i, name in enumerate(LUT_NAMES):
            s.luts[i] = fp(luts[name]).ctypes.data_as(C.POINTER(C.c_float))
        s.rgb_to_spd = fp(rgb_to_spd).ctypes.data_as(C.POINTER(C.c_float)) if rgb_to_spd is not None else None
        s.data_dir = N.DATA_DIR.encode()
        pl = scene.punctual_structs()
        s.punctual = pl
        s.n_punctual = len(scene.punctual_lights)
        s.uvs = fp(pool["uvs"]).ctypes.data_as(C.POINTER(C.c_float))
        tx = (OracleTexture * max(1, len(scene.textures)))()
        for i, (w, h, fmt, a) in enumerate(scene.textures):
            self.keep.append(a)
            tx[i].data = a.ctypes.data_as(C.c_void_p)
            tx[i].width, tx[i].height, tx[i].format = w, h, fmt
        s.textures = tx
        s.n_textures = len(scene.textures)
        s.env_texture = scene.env_texture
        s.env_cube = 1 if getattr(scene, "env_cube", False) else 0
        self.keep += [inst, mats, cam, pl, tx]
        self.s = s

    def render(self, params, precision=32, threads=None, records=True, film=False):
        threads = threads or os.cpu_count() or 1
        cw = params.crop_w or params.width
        ch = params.crop_h or params.height
        rec = np.zeros((params.spp_count, ch, cw, 8), np.float32) if records else None
        fil = np.zeros((ch, cw, 3), np.float64) if film else None
        st = OracleStats()
        rc = load().oracle_render(C.byref(self.s), C.byref(params), precision, threads,
                                  rec.ctypes.data_as(C.c_void_p) if rec is not None else None,
                                  fil.ctypes.data_as(C.c_void_p) if fil is not None else None, C.byref(st))
        if rc != 0:
            raise RuntimeError("oracle_render failed: %d" % rc)
        return dict(records=rec, film=fil, rays=st.rays, seconds=st.seconds)

    def ensure_rgb_table(self, params):
        """Gives the scene the oracle's own RGB -> spectrum fit for the request's range when the
        request needs one (RGB colours, coloured lights or an environment)."""
        if self.s.rgb_to_spd or load().oracle_needs_rgb_table(C.byref(self.s), C.byref(params)) != 1:
            return self
        lo, hi = params.lambda_min, params.lambda_max
        if lo == 0.0 and hi == 0.0:
            lo, hi = 380.0, 700.0
        t = np.ascontiguousarray(host_table("rgb_to_spd", (lo, hi)), np.float32)
        self.keep.append(t)
        self.s.rgb_to_spd = t.ctypes.data_as(C.POINTER(C.c_float))
        return self

    def render_strided(self, params, stride, precision=32, threads=None, film=False):
        """Every stride-th pixel of the crop in x and y (uni/NEE): a bounded sample of a large
        request. film: mean XYZ (ceil(ch/stride), ceil(cw/stride), 3) in float64."""
        threads = threads or os.cpu_count() or 1
        cw = params.crop_w or params.width
        ch = params.crop_h or params.height
        fil = np.zeros(((ch + stride - 1) // stride, (cw + stride - 1) // stride, 3), np.float64) if film else None
        st = OracleStats()
        rc = load().oracle_render_strided(C.byref(self.s), C.byref(params), int(stride), precision, threads,
                                          fil.ctypes.data_as(C.c_void_p) if fil is not None else None, C.byref(st))
        if rc != 0:
            raise RuntimeError("oracle_render_strided failed: %d" % rc)
        return dict(film=fil, rays=st.rays, seconds=st.seconds)

    def atrous_moments(self, params, moments, threads=None):
        """Adds the first-camera-vertex feature moments of the request's samples onto
        `moments` (float32 (4, H, W, 4), layout of yg_atrous_read), in sample order."""
        assert moments.dtype == np.float32 and moments.flags.c_contiguous
        assert moments.shape == (4, params.height, params.width, 4)
        rc = load().oracle_atrous_moments(C.byref(self.s), C.byref(params), threads or os.cpu_count() or 1,
                                          moments.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise RuntimeError("oracle_atrous_moments failed: %d" % rc)
        return moments


def atrous(film_sum, odd_sum, moments, camera, params, threads=None):
    """The a-trous filter on float32 arrays film_sum/odd_sum (H, W, 4) and moments
    (4, H, W, 4); returns (xyzw (H, W, 4), variance (H, W), features (2, H, W, 4) uint32)."""
    h, w = film_sum.shape[:2]
    f = [np.ascontiguousarray(a, np.float32) for a in (film_sum, odd_sum, moments)]
    out = np.zeros((h, w, 4), np.float32)
    var = np.zeros((h, w), np.float32)
    feat = np.zeros((2, h, w, 4), np.uint32)
    rc = load().oracle_atrous(w, h, *[a.ctypes.data_as(C.c_void_p) for a in f], C.byref(camera), C.byref(params),
                              threads or os.cpu_count() or 1, out.ctypes.data_as(C.c_void_p),
                              var.ctypes.data_as(C.c_void_p), feat.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise RuntimeError("oracle_atrous failed: %d" % rc)
    return out, var, feat


def luts_from_context(ctx):
    return {n: ctx.table(n) for n in LUT_NAMES}
