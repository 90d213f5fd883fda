"""ctypes view of the C ABI in include/yapt_gpu.h (libyaptgpu.so).

This is the thin binding the Python API and the tests use to call the library;
struct layouts mirror the header field by field.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
DATA_DIR = os.path.join(HERE, "data")
LIB_PATH = os.path.join(HERE, "libyaptgpu.so")

YG_OK = 0
INTEGRATORS = {"uni": 0, "BPT": 0, "nee": 1, "BPT_WITH_NEE": 1, "bdpt": 2, "BDPT": 2}

YG_MATERIAL_TWO_SIDED = 1
YG_MATERIAL_DISPERSION = 2
YG_MATERIAL_ALPHA_BLEND = 4
YG_FLAG_DISABLE_TEXEL_JITTER = 1 << 1
YG_FLAG_NO_FILM = 1 << 8
YG_FLAG_FEATURES = 1 << 9
YG_FLAG_COUNT_TRAVERSAL = 1 << 10
YG_FLAG_MEGAKERNEL = 1 << 11
YG_FLAG_TIME_KERNELS = 1 << 12
YG_FLAG_ATROUS_FEATURES = 1 << 13
YG_TEXTURE_RGBA8_UNORM, YG_TEXTURE_RGBA8_SRGB, YG_TEXTURE_RGBA32_FLOAT = 0, 1, 2
YG_NN_CONV_MMA_SYNC = 0
YG_NN_CONV_TCGEN05 = 1
YG_NN_CONV_TCGEN05_TMA = 2

TABLES = {
    "sobol": 0, "ss": 1, "ss_avg": 2, "ssms": 3, "ssms_avg": 4, "trans_denser": 5, "trans_lighter": 6,
    "trans_avg_denser": 7, "trans_avg_lighter": 8, "sheen": 9, "cie": 10, "rgb_to_spd": 11,
}


class Material(C.Structure):
    _fields_ = [
        ("albedo", C.c_float * 3), ("transparency", C.c_float),
        ("specular", C.c_float * 3), ("metalness", C.c_float),
        ("absorption", C.c_float * 3), ("dielectric_ior", C.c_float),
        ("emissive", C.c_float * 3), ("roughness", C.c_float),
        ("anisotropy", C.c_float), ("anisotropy_rotation", C.c_float),
        ("material_mask", C.c_uint32), ("thin_film_thickness_nm", C.c_float),
        ("cauchy", C.c_float * 2), ("sheen_amount", C.c_float), ("emission_focus", C.c_float),
        ("sheen_tint", C.c_float * 3), ("sheen_roughness", C.c_float),
        ("specular_amount", C.c_float), ("clear_coat_amount", C.c_float),
        ("clear_coat_ior", C.c_float), ("clear_coat_roughness", C.c_float),
        ("subsurface_radius", C.c_float * 3), ("subsurface_amount", C.c_float),
        ("subsurface_radius_scale", C.c_float), ("alpha_cutoff", C.c_float),
        ("albedo_spectrum", C.c_int32), ("specular_spectrum", C.c_int32),
        ("emission_spectrum", C.c_int32), ("reserved", C.c_int32),
        ("albedo_texture", C.c_uint32), ("normal_texture", C.c_uint32), ("orm_texture", C.c_uint32),
        ("emissive_texture", C.c_uint32), ("albedo_uv_scale", C.c_float * 2), ("normal_uv_scale", C.c_float * 2),
        ("orm_uv_scale", C.c_float * 2), ("emissive_uv_scale", C.c_float * 2),
    ]


class MeshDesc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
        ("tangents", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
        ("vertex_count", C.c_uint32), ("indices", C.c_void_p), ("index_count", C.c_uint32),
        ("index_bits", C.c_uint32), ("submesh_ranges", C.POINTER(C.c_uint32)), ("submesh_count", C.c_uint32),
    ]


class Instance(C.Structure):
    _fields_ = [
        ("obj_to_world", C.c_float * 12), ("world_to_obj", C.c_float * 12),
        ("mesh", C.c_uint32), ("submesh", C.c_uint32), ("material", C.c_uint32), ("reserved", C.c_uint32),
    ]


class Camera(C.Structure):
    _fields_ = [
        ("uv_to_view", C.c_float * 16), ("view_to_uv", C.c_float * 16),
        ("world_to_view", C.c_float * 16), ("view_to_world", C.c_float * 16),
        ("aperture_radius", C.c_float), ("focus_distance", C.c_float),
        ("view_forward_z_sign", C.c_float), ("reserved", C.c_float),
    ]


YG_LIGHT_POINT, YG_LIGHT_SPOT, YG_LIGHT_DIRECTIONAL = 1, 2, 3


class PunctualLight(C.Structure):
    _fields_ = [
        ("type", C.c_uint32), ("position", C.c_float * 3), ("direction", C.c_float * 3), ("intensity", C.c_float * 3),
        ("cos_inner", C.c_float), ("cos_outer", C.c_float), ("reserved", C.c_float * 2),
    ]


class TonemapParams(C.Structure):
    _fields_ = [
        ("enable", C.c_uint32), ("auto_exposure", C.c_uint32), ("manual_exposure", C.c_float),
        ("exposure_compensation", C.c_float), ("eye_adaptation_speed", C.c_float), ("delta_time", C.c_float),
        ("reset", C.c_uint32), ("source", C.c_uint32),
    ]


class AtrousParams(C.Structure):
    _fields_ = [
        ("depth_sigma_scale", C.c_float), ("normal_sigma", C.c_float), ("material_sigma", C.c_float),
        ("color_sigma", C.c_float), ("feature_variance_scale", C.c_float), ("prefilter", C.c_uint32),
        ("passes", C.c_uint32), ("reserved", C.c_uint32),
    ]


class RenderParams(C.Structure):
    _fields_ = [
        ("integrator", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
        ("spp_start", C.c_uint32), ("spp_count", C.c_uint32), ("max_depth", C.c_uint32),
        ("regularize_after_vertices", C.c_uint32), ("regularize_enable", C.c_uint32),
        ("env_intensity_scale", C.c_float), ("seed", C.c_uint32), ("flags", C.c_uint32),
        ("crop_x", C.c_uint32), ("crop_y", C.c_uint32), ("crop_w", C.c_uint32), ("crop_h", C.c_uint32),
        ("lambda_min", C.c_float), ("lambda_max", C.c_float), ("bdpt_light_paths", C.c_uint32),
        ("bdpt_light_vertices", C.c_uint32), ("reserved", C.c_uint32 * 2),
    ]


class SampleRecord(C.Structure):
    _fields_ = [("lambda_hero", C.c_float), ("radiance", C.c_float * 4), ("xyz", C.c_float * 3)]


class KernelProfile(C.Structure):
    """yg_kernel_profile: per-kind device time of the last wavefront render."""
    _fields_ = [("ms", C.c_float * 4), ("launches", C.c_uint32 * 4),
                ("closest_rays", C.c_uint64), ("closest_nodes", C.c_uint64), ("closest_triangles", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("shadow_nodes", C.c_uint64), ("shadow_triangles", C.c_uint64),
                ("connect_ms", C.c_float), ("connect_launches", C.c_uint32), ("connection_record_bytes", C.c_uint32),
                ("reserved", C.c_uint32)]


KERNEL_KINDS = ("trace", "regroup", "shade", "shadow")


class ServerOptions(C.Structure):
    _fields_ = [
        ("memory_budget_bytes", C.c_uint64), ("max_active", C.c_uint32), ("wave_capacity", C.c_uint32),
        ("round_samples", C.c_uint32), ("max_depth", C.c_uint32), ("lambda_min", C.c_float),
        ("lambda_max", C.c_float), ("use_graphs", C.c_uint32), ("persistent", C.c_uint32),
        ("barrier_polls", C.c_uint32), ("reserved", C.c_uint32 * 3),
    ]


class Request(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("reserved", C.c_uint32), ("params", RenderParams)]


class RequestInfo(C.Structure):
    _fields_ = [
        ("state", C.c_int32), ("error", C.c_int32), ("t_submit", C.c_double), ("t_admit", C.c_double),
        ("t_done", C.c_double), ("footprint_bytes", C.c_uint64), ("samples", C.c_uint64),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64), ("cancelled", C.c_uint64),
        ("rounds", C.c_uint64), ("graph_replays", C.c_uint64), ("bdpt_slices", C.c_uint64), ("samples", C.c_uint64),
        ("persistent_rounds", C.c_uint64), ("bytes_in_use", C.c_uint64), ("peak_bytes_in_use", C.c_uint64), ("active", C.c_uint32),
        ("queued", C.c_uint32), ("seconds", C.c_double),
    ]


class SchedItem(C.Structure):
    _fields_ = [
        ("pixels", C.c_uint64), ("planes_left", C.c_uint32), ("admitted", C.c_uint32),
        ("footprint_bytes", C.c_uint64), ("integrator", C.c_uint32), ("rounds_waited", C.c_uint32),
    ]


REQ_STATES = {0: "queued", 1: "active", 2: "done", 3: "failed", 4: "cancelled"}


class NNTensor(C.Structure):
    _fields_ = [("data", C.c_void_p), ("stride", C.c_uint32), ("offset", C.c_uint32), ("channels", C.c_uint32),
                ("reserved", C.c_uint32)]


_lib = None

# (name, restype, argtypes) for every function include/yapt_gpu.h declares
SIGNATURES = [
    ("yg_last_error", C.c_char_p, []),
    ("yg_version", C.c_int, []),
    ("yg_create", C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    ("yg_destroy", C.c_int, [C.c_void_p]),
    ("yg_synchronize", C.c_int, [C.c_void_p]),
    ("yg_get_table", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    ("yg_host_table", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    ("yg_upload_mesh", C.c_int, [C.c_void_p, C.POINTER(MeshDesc), C.POINTER(C.c_uint32)]),
    ("yg_clear_meshes", C.c_int, [C.c_void_p]),
    ("yg_film_resolve_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("yg_set_punctual_lights", C.c_int, [C.c_void_p, C.POINTER(PunctualLight), C.c_uint32]),
    ("yg_upload_texture", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32)]),
    ("yg_clear_textures", C.c_int, [C.c_void_p]),
    ("yg_set_environment_texture", C.c_int, [C.c_void_p, C.c_uint32]),
    ("yg_set_environment_cube", C.c_int, [C.c_void_p, C.c_uint32]),
    ("yg_atrous_default_params", None, [C.POINTER(AtrousParams)]),
    ("yg_tonemap_default_params", None, [C.POINTER(TonemapParams)]),
    ("yg_tonemap", C.c_int, [C.c_void_p, C.POINTER(TonemapParams), C.c_void_p, C.POINTER(C.c_float)]),
    ("yg_atrous_denoise", C.c_int, [C.c_void_p, C.POINTER(AtrousParams), C.c_void_p, C.c_void_p]),
    ("yg_atrous_read", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("yg_atrous_run", C.c_int, [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Camera),
                                C.POINTER(AtrousParams), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("yg_nn_set_conv_impl", C.c_int, [C.c_int]),
    ("yg_nn_tc_timeouts", C.c_int, [C.POINTER(C.c_uint32)]),
    ("yg_nn_tile_error", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                   C.c_void_p, C.c_void_p, C.c_void_p]),
    ("yg_nn_tile_fallback", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("yg_bvh_check", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("yg_upload_materials", C.c_int, [C.c_void_p, C.POINTER(Material), C.c_uint32]),
    ("yg_upload_spectra", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_uint32, C.c_uint32, C.c_float, C.c_float]),
    ("yg_set_instances", C.c_int, [C.c_void_p, C.POINTER(Instance), C.c_uint32]),
    ("yg_set_camera", C.c_int, [C.c_void_p, C.POINTER(Camera)]),
    ("yg_build_scene", C.c_int, [C.c_void_p]),
    ("yg_scene_info", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                C.POINTER(C.c_uint64)]),
    ("yg_film_clear", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    ("yg_render", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p]),
    ("yg_film_read", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("yg_film_state_size", C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    ("yg_debug_bounds_errors", C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)]),
    ("yg_film_save", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("yg_film_restore", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("yg_features_read", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("yg_film_relmse", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_double, C.POINTER(C.c_double)]),
    ("yg_last_render_stats", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint32)]),
    ("yg_last_traversal_counts", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("yg_last_kernel_profile", C.c_int, [C.c_void_p, C.POINTER(KernelProfile)]),
    ("yg_render_samples_noalloc", C.c_int, [C.c_void_p, C.POINTER(RenderParams), C.c_void_p]),
    ("yg_server_create", C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.POINTER(ServerOptions), C.POINTER(C.c_void_p)]),
    ("yg_server_submit", C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    ("yg_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]),
    ("yg_server_info", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(RequestInfo)]),
    ("yg_server_result", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("yg_server_cancel", C.c_int, [C.c_void_p, C.c_uint64]),
    ("yg_server_release", C.c_int, [C.c_void_p, C.c_uint64]),
    ("yg_server_stats_get", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("yg_grid_barrier_selftest", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32),
                                           C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("yg_server_destroy", C.c_int, [C.c_void_p]),
    ("yg_nn_conv3x3", C.c_int, [C.POINTER(NNTensor), C.c_void_p, C.POINTER(C.c_float), C.POINTER(NNTensor),
                                C.POINTER(NNTensor), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("yg_nn_sum_rows", C.c_int, [C.POINTER(C.c_float), C.c_int, C.c_long, C.POINTER(C.c_float), C.c_void_p]),
    ("yg_nn_flip_weights", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("yg_nn_wgrad_workspace", C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("yg_nn_conv3x3_wgrad", C.c_int, [C.POINTER(NNTensor), C.POINTER(NNTensor), C.POINTER(C.c_float),
                                      C.POINTER(C.c_float), C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("yg_nn_avgpool", C.c_int, [C.POINTER(NNTensor), C.POINTER(NNTensor), C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("yg_nn_avgpool_bwd", C.c_int, [C.POINTER(NNTensor), C.POINTER(NNTensor), C.POINTER(NNTensor), C.POINTER(NNTensor),
                                    C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("yg_nn_upsample", C.c_int, [C.POINTER(NNTensor), C.POINTER(NNTensor), C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("yg_nn_upsample_bwd", C.c_int, [C.POINTER(NNTensor), C.POINTER(NNTensor), C.POINTER(NNTensor), C.c_int, C.c_int,
                                     C.c_int, C.c_void_p]),
    ("yg_nn_head", C.c_int, [C.POINTER(NNTensor), C.POINTER(NNTensor), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_long,
                             C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float),
                             C.POINTER(NNTensor), C.POINTER(C.c_float), C.c_int, C.c_void_p]),
    ("yg_nn_adam", C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                             C.c_void_p, C.c_long, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]),
    ("yg_nn_pack_input", C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float), C.c_float, C.c_long, C.POINTER(NNTensor), C.c_void_p]),
    ("yg_server_plan", C.c_int64, [C.POINTER(SchedItem), C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
]


class YaptError(RuntimeError):
    pass


def load():
    """Loads libyaptgpu.so; fails loudly when the native library is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise YaptError("libyaptgpu.so is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != YG_OK:
        msg = load().yg_last_error().decode(errors="replace")
        raise YaptError("yapt_gpu error %d: %s" % (rc, msg))
    return rc


def host_table(name, lambda_range=(380, 700)):
    """Host-generated table (no GPU needed): same values a context uploads."""
    import numpy as np
    lib = load()
    which = TABLES[name]
    n = C.c_size_t()
    check(lib.yg_host_table(DATA_DIR.encode(), which, int(lambda_range[0]), int(lambda_range[1]), None, 0, C.byref(n)))
    out = np.zeros(n.value, dtype=np.uint32 if name == "sobol" else np.float32)
    check(lib.yg_host_table(DATA_DIR.encode(), which, int(lambda_range[0]), int(lambda_range[1]),
                            out.ctypes.data_as(C.c_void_p), out.size, C.byref(n)))
    return out
