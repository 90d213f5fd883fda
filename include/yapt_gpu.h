/*
 * yapt_gpu.h -- C ABI of the GB300 spectral path-tracing integrators.
 *
 * This is the drop-in boundary that replaces YAPT's integrator plug-in
 * (PathIntegratorSubStage, Source/Renderer/inc/Renderer/Shared/RenderPipeline/
 * PathTracer/PathIntegratorSubStage.h:20-72) and the scene ingest it is fed
 * through (Renderer::createMesh/createMaterial/createRenderObject,
 * Source/Renderer/inc/Renderer/Renderer.h:52-63). Everything is plain C: opaque
 * handles, pointers and sizes; no C++ or framework types cross it.
 *
 * Conventions
 *  - Every function returns YG_OK (0) or a negative YG_ERR_* code and never aborts
 *    the process. yg_last_error() returns a message for the calling thread.
 *  - Host pointers are read during the call only (the library copies them).
 *  - Matrices are row-major float[12] (3x4: rotation/scale columns 0..2,
 *    translation column 3) or float[16] (4x4).
 *  - One context owns its device memory and one CUDA stream on one GPU.
 */
#ifndef YAPT_GPU_H
#define YAPT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YG_API __attribute__((visibility("default")))

enum
{
    YG_OK = 0,
    YG_ERR_INVALID_ARGUMENT = -1,
    YG_ERR_CUDA = -2,
    YG_ERR_OUT_OF_MEMORY = -3,
    YG_ERR_NOT_READY = -4, /* e.g. render before yg_build_scene */
    YG_ERR_IO = -5,
    YG_ERR_DEVICE_TIMEOUT = -6, /* a bounded device-side wait ran out */
    YG_ERR_ADMISSION = -7       /* serving: request does not fit the memory budget */
};

/* Integrators: YAPT's RenderPipeline options BPT / BPT_WITH_NEE / BDPT
 * (Source/Renderer/inc/Renderer/Shared/RendererVarsList.h:24). */
enum
{
    YG_INTEGRATOR_UNI = 0,
    YG_INTEGRATOR_NEE = 1,
    YG_INTEGRATOR_BDPT = 2
};

/* Material mask bits (materialsCommon.hlsl:7-9) */
#define YG_MATERIAL_TWO_SIDED (1u << 0)
#define YG_MATERIAL_DISPERSION (1u << 1)
#define YG_MATERIAL_ALPHA_BLEND (1u << 2)

/* Principled material: the field set of YAPT's MaterialParameters
 * (Source/Renderer/inc/Renderer/Shared/MaterialInternal.h:39-115), plus the
 * spectral extension: *_spectrum >= 0 selects a tabulated curve uploaded with
 * yg_upload_spectra() instead of the RGB -> spectrum conversion. */
typedef struct yg_material
{
    float albedo[3];
    float transparency;
    float specular[3];
    float metalness;
    float absorption[3];
    float dielectric_ior;
    float emissive[3];
    float roughness;
    float anisotropy;
    float anisotropy_rotation;
    uint32_t material_mask;
    float thin_film_thickness_nm;
    float cauchy[2]; /* A, B [um^2] */
    float sheen_amount;
    float emission_focus;
    float sheen_tint[3];
    float sheen_roughness;
    float specular_amount;
    float clear_coat_amount;
    float clear_coat_ior;
    float clear_coat_roughness;
    float subsurface_radius[3];
    float subsurface_amount;
    float subsurface_radius_scale;
    float alpha_cutoff;
    int32_t albedo_spectrum;   /* -1: RGB albedo */
    int32_t specular_spectrum; /* -1: RGB specular */
    int32_t emission_spectrum; /* -1: RGB emission (times D65, as in the reference) */
    int32_t reserved;
    /* Textures (MaterialEntryGPU *TexIndexAndScale, materialsCommon.hlsl:354-397): texture id
     * + 1 from yg_upload_texture, 0 for none. Albedo multiplies the RGB albedo (alpha sets the
     * transparency of alpha-blended materials), normal is a tangent-space normal map, ORM holds
     * occlusion, roughness and metalness factors (glTF), emissive multiplies the RGB emission.
     * Each texture's uv is multiplied by its scale. */
    uint32_t albedo_texture;
    uint32_t normal_texture;
    uint32_t orm_texture;
    uint32_t emissive_texture;
    float albedo_uv_scale[2];
    float normal_uv_scale[2];
    float orm_uv_scale[2];
    float emissive_uv_scale[2];
} yg_material;

/* Mesh upload (BindlessMeshManager + Mesh.setVertexBuffer/setIndexBuffer/setSubmesh). */
typedef struct yg_mesh_desc
{
    const float* positions; /* vertex_count x 3 */
    const float* normals;   /* vertex_count x 3, required */
    const float* tangents;  /* vertex_count x 4 (xyz * w), or NULL */
    const float* uvs;       /* vertex_count x 2, or NULL */
    uint32_t vertex_count;
    const void* indices;
    uint32_t index_count;
    uint32_t index_bits;            /* 16 or 32 */
    const uint32_t* submesh_ranges; /* submesh_count x (first index, index count) */
    uint32_t submesh_count;
} yg_mesh_desc;

/* One (render object, submesh) instance, as in YAPT's TLAS instance list
 * (RaytraceCommonResources.cpp:216-279). world_to_obj must be the inverse of
 * obj_to_world; both are given so that every consumer uses the same floats. */
typedef struct yg_instance
{
    float obj_to_world[12];
    float world_to_obj[12];
    uint32_t mesh;
    uint32_t submesh;
    uint32_t material;
    uint32_t reserved;
} yg_instance;

/* Camera constants (RaytraceConstantData, raytraceCommonResources.hlsl:8-31). */
typedef struct yg_camera
{
    float uv_to_view[16];
    float view_to_uv[16];
    float world_to_view[16];
    float view_to_world[16];
    float aperture_radius;
    float focus_distance;
    float view_forward_z_sign;
    float reserved;
} yg_camera;

#define YG_FLAG_DISABLE_TEXEL_JITTER (1u << 1)
#define YG_FLAG_NO_FILM (1u << 8)      /* skip film accumulation (sample dump only) */
#define YG_FLAG_FEATURES (1u << 9)     /* accumulate first-hit albedo/normal/depth */
#define YG_FLAG_COUNT_TRAVERSAL (1u << 10) /* count BVH nodes visited / triangles tested (slower) */
#define YG_FLAG_MEGAKERNEL (1u << 11)      /* one-thread-per-path kernel instead of the wavefront */
#define YG_FLAG_TIME_KERNELS (1u << 12)    /* time each wavefront kernel kind with CUDA events */
#define YG_FLAG_ATROUS_FEATURES (1u << 13) /* gather the a-trous denoiser's feature moments and odd-sample film */

/* Punctual lights (PunctualLightParameters; LightEntryGPU in materialsCommonResources.hlsl):
 * point and spot lights emit RGB intensity from a position (spot: within the cone of
 * direction, full inside cos_inner, smoothstep to zero at cos_outer); a directional light
 * delivers RGB irradiance travelling along direction. They have no geometry: BSDF
 * sampling never hits them, so they are sampled explicitly by every integrator (uni: the
 * punctual lights only; NEE: all lights). */
#define YG_LIGHT_POINT 1
#define YG_LIGHT_SPOT 2
#define YG_LIGHT_DIRECTIONAL 3
typedef struct yg_punctual_light
{
    uint32_t type;       /* YG_LIGHT_* */
    float position[3];   /* world space (point, spot) */
    float direction[3];  /* world space, direction of emission (spot axis, directional); normalised on upload */
    float intensity[3];  /* RGB */
    float cos_inner;     /* spot: cosine of the inner (full intensity) angle */
    float cos_outer;     /* spot: cosine of the outer (zero intensity) angle */
    float reserved[2];
} yg_punctual_light;

typedef struct yg_render_params
{
    uint32_t integrator; /* YG_INTEGRATOR_* */
    uint32_t width;
    uint32_t height;
    uint32_t spp_start; /* Sobol sample index of the first sample */
    uint32_t spp_count;
    uint32_t max_depth;                /* maxRayDepth (reference: 32) */
    uint32_t regularize_after_vertices; /* Regularize.AfterVertices (reference default 8) */
    uint32_t regularize_enable;         /* 1: reference behaviour; 0: no roughness widening */
    float env_intensity_scale;          /* Env.IntensityScale (reference default 1) */
    uint32_t seed;                      /* 0: reference scramble seeds */
    uint32_t flags;
    uint32_t crop_x, crop_y, crop_w, crop_h; /* render only this pixel rectangle (w=h=0: all) */
    float lambda_min, lambda_max;            /* spectral range; reference: 380..700 nm */
    uint32_t bdpt_light_paths;               /* BDPT: light subpaths per frame (0: ceil(W/8)*ceil(H/8) of the crop) */
    uint32_t bdpt_light_vertices;            /* BDPT: vertices per light subpath, light included (0: 16, max 16;
                                                maxVerticesPerLightPath, BidirectionalPathIntegratorSubStage.cpp:480-488) */
    uint32_t reserved[2];
} yg_render_params;

/* Per-sample record written by yg_render when sample_dump != NULL:
 * hero wavelength, radiance at the 4 hero wavelengths, XYZ. */
typedef struct yg_sample_record
{
    float lambda_hero;
    float radiance[4];
    float xyz[3];
} yg_sample_record;

typedef struct yg_context yg_context;

/* Tables produced by the library that any reproducing host code must share. */
enum
{
    YG_TABLE_SOBOL_MATRICES = 0,     /* uint32[256 x 32] */
    YG_TABLE_LUT_SS_NOFRESNEL = 1,   /* 32 x 32          (MultipleScatterLUT.cpp:76-136) */
    YG_TABLE_LUT_SS_AVG_NOFRESNEL = 2, /* 32 */
    YG_TABLE_LUT_SSMS = 3,           /* 16 x 16 x 16 */
    YG_TABLE_LUT_SSMS_AVG = 4,       /* 16 x 16 */
    YG_TABLE_LUT_TRANSLUCENT_DENSER = 5,  /* 16^3 */
    YG_TABLE_LUT_TRANSLUCENT_LIGHTER = 6, /* 16^3 */
    YG_TABLE_LUT_TRANSLUCENT_AVG_DENSER = 7,  /* 16^2 */
    YG_TABLE_LUT_TRANSLUCENT_AVG_LIGHTER = 8, /* 16^2 */
    YG_TABLE_LUT_SHEEN = 9,          /* 16 x 16 */
    YG_TABLE_CIE_1NM = 10,           /* 471 x 4: xbar ybar zbar d65, 360..830 nm */
    YG_TABLE_RGB_TO_SPD = 11,        /* 64^3 x 3 sigmoid-polynomial coefficients (sRGB) */
    YG_TABLE_COUNT = 12
};

/* -- lifetime -------------------------------------------------------------- */
YG_API const char* yg_last_error(void);
YG_API int yg_version(void);
/* data_dir: folder holding the shipped data tables (CIE, Joe-Kuo). device: CUDA ordinal. */
YG_API int yg_create(const char* data_dir, int device, yg_context** out);
YG_API int yg_destroy(yg_context* ctx);
YG_API int yg_synchronize(yg_context* ctx);

/* -- tables ----------------------------------------------------------------- */
/* Copies table `which` (YG_TABLE_*) into out (float or uint32 elements). *count
 * receives the element count; call with out == NULL to query it. */
YG_API int yg_get_table(yg_context* ctx, int which, void* out, size_t capacity, size_t* count);

/* Same tables generated on the host alone (no CUDA device or context needed):
 * YG_TABLE_SOBOL_MATRICES, YG_TABLE_LUT_*, YG_TABLE_CIE_1NM, and YG_TABLE_RGB_TO_SPD
 * for the spectral range lambda_min..lambda_max (whole nm). */
YG_API int yg_host_table(const char* data_dir, int which, int lambda_min, int lambda_max, void* out, size_t capacity,
                         size_t* count);

/* -- scene ingest ----------------------------------------------------------- */
YG_API int yg_upload_mesh(yg_context* ctx, const yg_mesh_desc* desc, uint32_t* mesh_id);
/* Drops every uploaded mesh (mesh ids restart at 0), as when the last reference to a
 * Mesh is released (MeshManager, Source/Renderer/src/Shared/MeshManager.cpp). The scene
 * must be rebuilt (yg_set_instances + yg_build_scene) before the next render. */
YG_API int yg_clear_meshes(yg_context* ctx);
YG_API int yg_upload_materials(yg_context* ctx, const yg_material* materials, uint32_t count);
/* n_curves curves of n_points values on a uniform grid lambda_min..lambda_max. */
YG_API int yg_upload_spectra(yg_context* ctx, const float* values, uint32_t n_curves, uint32_t n_points,
                             float lambda_min, float lambda_max);
YG_API int yg_set_instances(yg_context* ctx, const yg_instance* instances, uint32_t count);
/* 2D textures (g_textures2D): decoded at upload to linear float RGBA and sampled bilinearly with
 * wrapping at mip 0. RGBA8_UNORM: v / 255; RGBA8_SRGB: the sRGB transfer function on RGB (alpha
 * linear); RGBA32_FLOAT as given. The id (0, 1, ...) is in upload order; materials refer to id + 1.
 * yg_clear_textures drops them all (the materials' references must be updated too). */
#define YG_TEXTURE_RGBA8_UNORM 0
#define YG_TEXTURE_RGBA8_SRGB 1
#define YG_TEXTURE_RGBA32_FLOAT 2
YG_API int yg_upload_texture(yg_context* ctx, uint32_t width, uint32_t height, uint32_t format, const void* data,
                             uint32_t* texture_id);
YG_API int yg_clear_textures(yg_context* ctx);
/* The environment (RVARNAME_SKYBOX with a longitude-latitude map): texture id + 1, or 0 for the
 * reference's analytic |dir| sky. Scaled by env_intensity_scale of each request. */
YG_API int yg_set_environment_texture(yg_context* ctx, uint32_t texture);
/* A cube-map environment (RVARNAME_SKYBOX holding a TEXTURE_CUBEMAP; envType
 * ENVIRONMENT_TYPE_CUBE, RaytraceCommonResources.cpp:292-296 and getSkyBoxColor,
 * materialsCommonResources.hlsl:196-199): texture id + 1 of an uploaded texture whose six square
 * faces are stacked top to bottom in layer order +X, -X, +Y, -Y, +Z, -Z (height = 6 x width).
 * yg_set_environment_texture switches back to a longitude-latitude map or the analytic sky. */
YG_API int yg_set_environment_cube(yg_context* ctx, uint32_t texture);
/* The tonemap stage (TonemapStage.cpp; knobs Tonemap.* of RendererVarsList.h:50-57): the film
 * mean or the last a-trous output in linear sRGB, a 128-bucket EV histogram from EV -12, auto
 * exposure (key 0.18 over the mean luminance, exposure compensation in EV, approached with
 * 1 - exp(-dt * speed) each frame from the first frame's value) or a manual exposure, the ACES
 * fitted operator when enabled, and the sRGB transfer function to RGBA8. rgba8: HOST buffer of
 * W*H*4 bytes; exposure (may be NULL) receives the exposure used. Synchronous. */
typedef struct yg_tonemap_params
{
    uint32_t enable;             /* Tonemap.Enable: the ACES fitted operator */
    uint32_t auto_exposure;      /* Tonemap.UseAutoExposure */
    float manual_exposure;       /* Tonemap.ManualExposure */
    float exposure_compensation; /* Tonemap.ExposureCompensation (EV) */
    float eye_adaptation_speed;  /* Tonemap.EyeAdaptationSpeed */
    float delta_time;            /* seconds since the previous frame */
    uint32_t reset;              /* first frame: the exposure starts at its parameter value */
    uint32_t source;             /* 0: the film mean, 1: the last yg_atrous_denoise output */
} yg_tonemap_params;
YG_API void yg_tonemap_default_params(yg_tonemap_params* params);
YG_API int yg_tonemap(yg_context* ctx, const yg_tonemap_params* params, uint8_t* rgba8, float* exposure);
/* Replaces the punctual lights (count 0 removes them). The light tables are rebuilt at once
 * when the scene is built, else by yg_build_scene. */
YG_API int yg_set_punctual_lights(yg_context* ctx, const yg_punctual_light* lights, uint32_t count);
YG_API int yg_set_camera(yg_context* ctx, const yg_camera* camera);
/* Builds the acceleration structure and the light tables (alias tables over mesh
 * lights, RaytraceCommonResources.cpp:325-547) for the current meshes/instances/materials. */
YG_API int yg_build_scene(yg_context* ctx);
/* Diagnostic of the device-built wide BVH: walks the tree on the host and counts the child
 * slots whose dequantised box (evaluated in double) does not contain the triangles under
 * the slot; *violations must be 0. Also returns the node count and the depth in wide levels. */
YG_API int yg_bvh_check(yg_context* ctx, uint64_t* n_nodes, uint64_t* depth, uint64_t* violations);
/* Scene statistics: triangles, BVH nodes, lights, device bytes. */
YG_API int yg_scene_info(yg_context* ctx, uint64_t* n_triangles, uint64_t* n_nodes, uint64_t* n_lights,
                         uint64_t* device_bytes);

/* -- rendering -------------------------------------------------------------- */
/* Clears the film to width x height (Kahan FP32 XYZ sums + sample counts). */
YG_API int yg_film_clear(yg_context* ctx, uint32_t width, uint32_t height);
/* Renders params->spp_count samples per pixel starting at Sobol index spp_start and
 * accumulates them into the film in sample order. If sample_dump is non-NULL it
 * receives crop_w*crop_h*spp_count yg_sample_record (host memory), ordered
 * [spp][row][column] of the crop. Asynchronous unless sample_dump is given. */
YG_API int yg_render(yg_context* ctx, const yg_render_params* params, yg_sample_record* sample_dump);
/* Film readback: mean XYZ per pixel (width*height*3) and per-pixel sample counts
 * (width*height, may be NULL). Synchronises the context stream. */
YG_API int yg_film_read(yg_context* ctx, float* xyz_mean, float* counts);
/* Film checkpoints: the compensated XYZ sums and counts, the feature accumulators and the
 * a-trous moments of the context's film, so that a preempted render can resume. Renders after a
 * restore continue the accumulation exactly as if it had not stopped (same film, bit for bit).
 * yg_film_state_size gives the bytes; yg_film_save copies the state to host memory;
 * yg_film_restore makes it the context's film (YG_ERR_INVALID_ARGUMENT for a buffer that is not
 * a saved state of this format). */
YG_API int yg_film_state_size(yg_context* ctx, size_t* bytes);
/* Debug build (compiled with -DYG_DEBUG_BOUNDS): out-of-range node, triangle and queue indices
 * the kernels refused (counted and skipped instead of read) since the scene was built;
 * YG_ERR_NOT_READY in a normal build. */
YG_API int yg_debug_bounds_errors(yg_context* ctx, uint32_t* count);
YG_API int yg_film_save(yg_context* ctx, void* host, size_t bytes);
YG_API int yg_film_restore(yg_context* ctx, const void* host, size_t bytes);
/* The same means written to DEVICE buffers (any may be NULL: xyz_mean and albedo/normal
 * W*H*3 floats, depth W*H); the call returns when they are written. Features need a render
 * with YG_FLAG_FEATURES since the last yg_film_clear. */
YG_API int yg_film_resolve_device(yg_context* ctx, float* xyz_mean, float* albedo, float* normal, float* depth);
/* First-hit feature means (YG_FLAG_FEATURES): albedo RGB, normal xyz, depth per pixel. */

/* The reference's edge-stopping a-trous denoiser (CombineSamplesSubStage.cpp:305-313,
 * 689-698 running prefilterFeatures.comp and denoise.comp; knobs RendererVarsList.h:25-32),
 * kept as the baseline the learned denoiser is measured against. Defaults are the
 * reference's: depth sigma scale 0.02, normal sigma 0.06, material sigma 0.05, colour sigma
 * 3, feature variance scale 1, prefilter on, 5 passes. */
typedef struct yg_atrous_params
{
    float depth_sigma_scale;      /* Denoise.DepthSigmaScale */
    float normal_sigma;           /* Denoise.NormalSigma */
    float material_sigma;         /* Denoise.MaterialDifferenceSigma */
    float color_sigma;            /* Denoise.ColorDifferenceSigma */
    float feature_variance_scale; /* Denoise.FeatureVarianceScale */
    uint32_t prefilter;           /* Denoise.FeaturePrefilter: 0 off, 1 on */
    uint32_t passes;              /* a-trous passes, steps 1, 2, 4, ... (reference: 5) */
    uint32_t reserved;
} yg_atrous_params;
YG_API void yg_atrous_default_params(yg_atrous_params* params);
/* Denoises the context's film. Every film render since the last yg_film_clear must have
 * carried YG_FLAG_ATROUS_FEATURES (else YG_ERR_NOT_READY). out_xyzw: DEVICE buffer of
 * W*H*4 floats (XYZ, 1) and out_variance DEVICE W*H floats; either may be NULL, and the
 * result then stays in the context for yg_atrous_read. Returns when the output is written. */
YG_API int yg_atrous_denoise(yg_context* ctx, const yg_atrous_params* params, float* out_xyzw, float* out_variance);
/* Host copies of the context's a-trous state (any pointer may be NULL): the last
 * yg_atrous_denoise output kept in the context (W*H*4, W*H), the filter's inputs -- the film's
 * XYZ sums and counts (W*H float4), the odd-sample XYZ sums and counts (W*H float4), the
 * gathered feature-moment sums (4 planes of W*H float4: albedo.rgb, |albedo|^2; normal.xyz,
 * hits; roughness, metalness, transparency, anisotropy; IOR/2, |material|^2 + (IOR/2)^2,
 * depth, depth^2) -- and the packed prefiltered features (2 planes of W*H uint4, the
 * reference's two RGBA32_UINT feature textures). Synchronous. */
YG_API int yg_atrous_read(yg_context* ctx, float* xyzw, float* variance, float* film_sum, float* odd_sum, float* moments,
                          uint32_t* features);
/* The same filter on caller data, all HOST buffers of W*H pixels row major (copied to the
 * device and back inside the call): film_sum XYZ sums and sample count (float4), odd_sum
 * the odd-indexed samples' XYZ sums and count (float4), moments as for yg_atrous_read;
 * outputs out_xyzw (W*H*4), out_variance (W*H) and, if not NULL, features_out (2*W*H uint4). */
YG_API int yg_atrous_run(uint32_t width, uint32_t height, const float* film_sum, const float* odd_sum,
                         const float* moments, const yg_camera* camera, const yg_atrous_params* params,
                         float* out_xyzw, float* out_variance, uint32_t* features_out);
YG_API int yg_features_read(yg_context* ctx, float* albedo, float* normal, float* depth);
/* relMSE of the film mean against a reference image (host, width*height*3 floats),
 * reduced in FP64 on the device: mean over pixels and channels of
 * (x - r)^2 / (r^2 + eps). */
YG_API int yg_film_relmse(yg_context* ctx, const float* reference_xyz, double eps, double* relmse);

/* Render without allocating: no counterpart in the reference. For callers that cannot
 * allocate device memory while rendering -- a serving process whose admission controller
 * reserves the device budget up front, or a host application that must not trigger
 * cudaMalloc's implicit device synchronisation mid-frame. Same samples as yg_render (uni or
 * NEE; the film, sample dump and features are not touched). The scene must already be built
 * (yg_build_scene) and the spectral range must be the one of the context's last yg_render
 * (380..700 nm on a new context). Writes crop_w * crop_h * spp_count float4 (X, Y, Z, 1)
 * to device_sample_xyz (device memory, 16-byte aligned), ordered [spp][row][column];
 * asynchronous on the context stream (ready after yg_synchronize).
 * Scratch: a file-scope device array of about 7 MB that every GPU loading the library holds
 * until exit; at most 256 sample indices per call (spp_count > 256 is rejected) and waves of
 * 16384 paths. The first call on a device sets the array up: it looks up the array's device
 * address and copies the constant Sobol generator matrices into it (a synchronous copy); make
 * that first call before any stream capture. Later calls only launch kernels. All calls share
 * the one array: calls whose work overlaps on the GPU (other contexts or threads, other
 * streams) race on it. A material that refers to a texture that is no longer resident (after
 * yg_clear_textures) is rejected, as by yg_render. */
YG_API int yg_render_samples_noalloc(yg_context* ctx, const yg_render_params* params, float* device_sample_xyz);

/* Device timing of the most recent yg_render: kernel milliseconds, rays traced. */
YG_API int yg_last_render_stats(yg_context* ctx, float* kernel_ms, uint64_t* rays, uint32_t* launches);
/* Traversal work of the most recent render made with YG_FLAG_COUNT_TRAVERSAL. */
YG_API int yg_last_traversal_counts(yg_context* ctx, uint64_t* nodes_visited, uint64_t* triangles_tested);

/* Per-kernel device time of the most recent wavefront render made with YG_FLAG_TIME_KERNELS
 * (CUDA events on the context stream around every launch of a kind), and with
 * YG_FLAG_COUNT_TRAVERSAL the traversal work split between closest-hit and shadow rays.
 * A BDPT render times its camera-side kernels by the same kinds (trace: camera rays; regroup:
 * class keys and regroup; shade: camera vertices; shadow: visibility rays and accumulation)
 * plus its connection kernel, and counts its connection records. A render times at most 16,384
 * launches (BDPT: 8,192); launches beyond that are not timed. */
#define YG_KERNEL_TRACE 0   /* closest-hit traversal of the path queue */
#define YG_KERNEL_REGROUP 1 /* shading-class keys and the regrouping scatter */
#define YG_KERNEL_SHADE 2   /* surface interaction, BSDF sampling, light sampling */
#define YG_KERNEL_SHADOW 3  /* shadow-ray traversal */
#define YG_KERNEL_CONNECT 4 /* BDPT: camera-vertex x light-vertex connections (connect_ms) */
typedef struct yg_kernel_profile
{
    float ms[4];          /* summed device milliseconds per YG_KERNEL_* kind */
    uint32_t launches[4]; /* timed launches per kind */
    uint64_t closest_rays, closest_nodes, closest_triangles;
    uint64_t shadow_rays, shadow_nodes, shadow_triangles; /* BDPT: shadow_rays = connection records */
    float connect_ms;                 /* BDPT: the connection kernel's device time */
    uint32_t connect_launches;
    uint32_t connection_record_bytes; /* bytes the connection kernel moves per record */
    uint32_t reserved;
} yg_kernel_profile;
YG_API int yg_last_kernel_profile(yg_context* ctx, yg_kernel_profile* out);

/* -- serving loop ----------------------------------------------------------------
 * No counterpart in the reference, which renders one interactive view at a time through
 * PathTraceStage::update (PathTraceStage.cpp:90-140); this is the request loop of the
 * serving configuration. A server keeps the scenes of several contexts resident on their
 * device and renders many requests at once: requests wait in arrival order until their
 * film fits the memory budget and a slot is free, then every round merges the paths of
 * all admitted uni/NEE requests (any scene, size, spp, depth) into one wavefront, replayed
 * as a captured CUDA graph, while BDPT requests advance on a second stream. A request's
 * result is the same film as yg_render of the same parameters on its context. While a
 * server exists its contexts must not be rendered with directly. */
typedef struct yg_server yg_server;

typedef struct yg_server_options
{
    uint64_t memory_budget_bytes; /* device bytes for request films and BDPT state (0: 8 GiB) */
    uint32_t max_active;          /* requests rendered concurrently (0: 64, at most 256) */
    uint32_t wave_capacity;       /* paths per merged round (0: 2^21; at least one plane of the largest image) */
    uint32_t round_samples;       /* samples planned per round when several requests share it (0: 2^19) */
    uint32_t max_depth;           /* largest uni/NEE max_depth accepted (0: 16) */
    float lambda_min, lambda_max; /* spectral range of every request (0, 0: 380..700) */
    uint32_t use_graphs;          /* 1: replay the merged round as a captured CUDA graph; 0: plain launches */
    uint32_t persistent;          /* 1: run the merged round as one persistent cooperative kernel whose
                                     stages meet at bounded grid barriers (captured as a graph when
                                     use_graphs is set and the driver captures cooperative launches) */
    uint32_t barrier_polls;       /* polls of ~128 ns a block waits at a barrier before the round fails
                                     with YG_ERR_DEVICE_TIMEOUT (0: 2^24) */
    uint32_t reserved[3];
} yg_server_options;

typedef struct yg_request
{
    uint32_t scene;          /* index into the contexts given to yg_server_create */
    uint32_t reserved;
    yg_render_params params; /* flags may hold YG_FLAG_DISABLE_TEXEL_JITTER only */
} yg_request;

enum
{
    YG_REQ_QUEUED = 0,
    YG_REQ_ACTIVE = 1,
    YG_REQ_DONE = 2,
    YG_REQ_FAILED = 3,
    YG_REQ_CANCELLED = 4
};

typedef struct yg_request_info
{
    int32_t state;  /* YG_REQ_* */
    int32_t error;  /* YG_ERR_* of a failed request */
    double t_submit, t_admit, t_done; /* seconds since yg_server_create (-1: not yet) */
    uint64_t footprint_bytes;
    uint64_t samples;
} yg_request_info;

typedef struct yg_server_stats
{
    uint64_t submitted, completed, failed, cancelled;
    uint64_t rounds, graph_replays, bdpt_slices, samples;
    uint64_t persistent_rounds;   /* merged rounds run as one persistent kernel */
    uint64_t bytes_in_use, peak_bytes_in_use;
    uint32_t active, queued;
    double seconds;
} yg_server_stats;

YG_API int yg_server_create(yg_context* const* scenes, uint32_t n_scenes, const yg_server_options* options,
                            yg_server** out);
/* Validates and queues a request (YG_ERR_ADMISSION if it could never fit the budget). */
YG_API int yg_server_submit(yg_server* server, const yg_request* request, uint64_t* id);
/* Waits until the request is done, failed or cancelled (YG_ERR_NOT_READY after timeout_s). */
YG_API int yg_server_wait(yg_server* server, uint64_t id, double timeout_s, yg_request_info* info);
YG_API int yg_server_info(yg_server* server, uint64_t id, yg_request_info* info);
/* Mean XYZ per pixel (width x height x 3, zero outside the crop) of a finished request. */
YG_API int yg_server_result(yg_server* server, uint64_t id, float* xyz_mean, float* counts);
YG_API int yg_server_cancel(yg_server* server, uint64_t id);
/* Forgets a finished, failed or cancelled request and its result. */
YG_API int yg_server_release(yg_server* server, uint64_t id);
YG_API int yg_server_stats_get(yg_server* server, yg_server_stats* stats);
/* Cancels what is queued, finishes nothing further, waits for the device and frees it all. */
YG_API int yg_server_destroy(yg_server* server);
/* Self-check of the bounded grid barrier the persistent merged round uses: one cooperative
 * kernel on the context's stream whose blocks pass the barrier three times while `missing`
 * blocks never arrive (0: all arrive). *blocks: the grid; *passes: barriers passed summed over
 * blocks (3 x blocks when all arrive); *timed_out: 1 when a wait ran out of `poll_limit`
 * polls, after which every block returned and the context stays usable. */
YG_API int yg_grid_barrier_selftest(yg_context* ctx, uint32_t missing, uint32_t poll_limit, uint32_t* blocks,
                                    uint32_t* passes, uint32_t* timed_out);

/* One scheduling decision of the serving loop on host data only (no device work), so the
 * policy can be checked without a GPU. items[i]: pixels, planes still to render, film
 * footprint, whether admitted already, integrator. Admits queued items in order while the
 * budget and slots allow (out admit[i] = 1), then plans one merged round for the admitted
 * uni/NEE items, fewest remaining samples first (out planes[i]). Returns the planned samples. */
typedef struct yg_sched_item
{
    uint64_t pixels;
    uint32_t planes_left;
    uint32_t admitted;
    uint64_t footprint_bytes;
    uint32_t integrator;
    uint32_t rounds_waited; /* rounds passed over; from 8 on an item is planned first */
} yg_sched_item;
YG_API int64_t yg_server_plan(const yg_sched_item* items, uint32_t n, uint64_t budget_bytes, uint64_t bytes_in_use,
                              uint32_t max_active, uint32_t wave_capacity, uint32_t round_samples, uint32_t* admit,
                              uint32_t* planes);

/* -- denoiser network operators ----------------------------------------------------
 * No counterpart in the reference (its denoiser is the a-trous filter of
 * postprocess/denoise.comp). Building blocks of the learned U-Net denoiser: BF16 tensor-core
 * 3x3 convolutions with FP32 accumulation (forward, data gradient through flipped weights,
 * weight gradient), 2x2 average pooling, 2x upsampling, the 1x1 RGB head with its relMSE
 * loss, Adam and input packing. All pointers are device memory; `stream` is a cudaStream_t
 * (NULL: the default stream). Tensors are NHWC BF16 views: element (pixel q, channel c) at
 * data[q * stride + offset + c]; channels, stride and offset are multiples of 16, 8 and 8.
 * Convolution weights are BF16 [cout][3][3][cin]; the returned status reports a launch
 * error only (kernels run asynchronously). */
typedef struct yg_nn_tensor
{
    void* data;
    uint32_t stride;
    uint32_t offset;
    uint32_t channels;
    uint32_t reserved;
} yg_nn_tensor;

/* The tensor-core path of yg_nn_conv3x3: YG_NN_CONV_TCGEN05 (tcgen05.mma with the accumulator in
 * tensor memory) or YG_NN_CONV_MMA_SYNC (warp-level mma.sync). Process-wide. */
#define YG_NN_CONV_MMA_SYNC 0
#define YG_NN_CONV_TCGEN05 1
#define YG_NN_CONV_TCGEN05_TMA 2 /* tcgen05 with the operands loaded by TMA (cp.async.bulk.tensor) */
YG_API int yg_nn_set_conv_impl(int impl);
/* Bounded waits of the tcgen05 convolution that ran out since load (0 on a healthy device). */
YG_API int yg_nn_tc_timeouts(uint32_t* count);
/* y = relu?(conv3x3(x, w) + bias), times (mask > 0) where mask is given, added to y when
 * accumulate; y->channels must be a multiple of 32. Zero padding, stride 1. */
YG_API int yg_nn_conv3x3(const yg_nn_tensor* x, const void* weights, const float* bias, const yg_nn_tensor* y,
                         const yg_nn_tensor* mask, int relu, int accumulate, int n, int h, int w, void* stream);
/* out[i] = sum over r of in[r * n + i], rows summed in order (deterministic). */
YG_API int yg_nn_sum_rows(const float* in, int rows, long n, float* out, void* stream);
/* wt[ci][8 - tap][co] = w[co][tap][ci]: yg_nn_conv3x3(dy, wt) is then the data gradient. */
YG_API int yg_nn_flip_weights(const void* w, int cout, int cin, void* wt, void* stream);
/* FP32 bytes of the split-K workspace yg_nn_conv3x3_wgrad needs. */
YG_API size_t yg_nn_wgrad_workspace(int cin, int cout, int n, int h, int w);
/* dw[co][tap][ci] = sum over pixels of dy[q][co] * x[q + tap][ci] (FP32), db[co] = sum dy. */
YG_API int yg_nn_conv3x3_wgrad(const yg_nn_tensor* x, const yg_nn_tensor* dy, float* dw, float* db, void* workspace,
                               int n, int h, int w, void* stream);
YG_API int yg_nn_avgpool(const yg_nn_tensor* in, const yg_nn_tensor* out, int n, int h, int w, void* stream);
/* din = dout / 4 over each 2x2 window (+ add), times (mask > 0); h, w are the input's size. */
YG_API int yg_nn_avgpool_bwd(const yg_nn_tensor* dout, const yg_nn_tensor* add, const yg_nn_tensor* mask,
                             const yg_nn_tensor* din, int n, int h, int w, void* stream);
/* nearest 2x upsampling of an h x w input. */
YG_API int yg_nn_upsample(const yg_nn_tensor* in, const yg_nn_tensor* out, int n, int h, int w, void* stream);
YG_API int yg_nn_upsample_bwd(const yg_nn_tensor* dout, const yg_nn_tensor* mask, const yg_nn_tensor* din, int n, int h,
                              int w, void* stream);
/* out = expm1(w x + b + skip[0..2]) per pixel (w: 3 x 32 FP32; skip, when given: the input's
 * log1p radiance channels, so the network predicts a log-space correction); with target: per-block sums of
 * (out - t)^2 / (t^2 + eps) in loss_partial[blocks]; with din: the loss gradient wrt x (mean
 * over pixels and channels, through the features' ReLU) and per-block partial gradients of w
 * and b in gw_partial[blocks][99]. */
YG_API int yg_nn_head(const yg_nn_tensor* in, const yg_nn_tensor* skip, const float* w, const float* b, long pixels, float* out,
                      const float* target, float eps, float* loss_partial, const yg_nn_tensor* din, float* gw_partial, int blocks,
                      void* stream);
/* One Adam step on FP32 parameters (step counts from 1); writes the BF16 copy when given. */
YG_API int yg_nn_adam(float* params, const float* grads, float* m, float* v, void* params_bf16, long n, float lr, float beta1,
                      float beta2, float eps, int step, void* stream);
/* 16-channel network input: log1p(linear sRGB of the mean XYZ), albedo, normal, depth / depth_scale, zeros. */
YG_API int yg_nn_pack_input(const float* xyz, const float* albedo, const float* normal, const float* depth, float depth_scale,
                            long pixels, const yg_nn_tensor* out, void* stream);
/* Per-tile error estimate of a denoised image `out` (height x width x 3, FP32) from the denoised
 * images a and b of two independent half renders: the tile mean of ((a-b)^2/4)/(out^2+eps) into
 * tile_err, and tile_flags = err > threshold (tiles of `tile` pixels, row-major). */
YG_API int yg_nn_tile_error(const float* a, const float* b, const float* out, int height, int width, int tile, float eps,
                            float threshold, float* tile_err, uint32_t* tile_flags, void* stream);
/* Replaces the flagged tiles of out by the linear sRGB of film_xyz (the plain film mean). */
YG_API int yg_nn_tile_fallback(float* out, const float* film_xyz, const uint32_t* tile_flags, int height, int width, int tile,
                               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* YAPT_GPU_H */
