/*
 * oracle.h -- CPU oracle for the spectral path-tracing integrators.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain scalar C++ restatement of YAPT's
 * integrator shaders (uni / NEE), written from the HLSL sources and templated on
 * the scalar type: float (per-sample parity with the GPU) and double (the
 * reference images that relMSE is judged against). It is used by tests/, by
 * smoke() and by bench.py's CPU baseline, never by the product path.
 *
 * Parity status: the reference's hot path is HLSL for DX12/Vulkan ray tracing and
 * cannot run as a renderer here, and its tests hold no golden vectors for this path
 * beyond the Sobol generator matrices of SobolMatrices.h. The shader math itself is
 * pinned: oracle/ref_build.py compiles the reference's own .hlsl files as C++ (through
 * oracle/hlsl_shim.h) into oracle/_ref/refcheck, which compares this oracle with them
 * function by function on seeded inputs -- sampler and Owen scrambling bit for bit; the
 * spectral conversions, ToXYZ, Russian roulette, GGX, Fresnel, sheen, every lobe, the
 * multiple-scattering compensation (both models), layer probabilities, layer sampling and
 * the layered evaluateSurface within 1e-4 (tests/test_reference_pin.py). Traversal, the
 * bounce loop, NEE and the BDPT connection logic remain restatements checked against the
 * device and against each other (uni/NEE/BDPT agreement), not against reference code.
 */
#ifndef YAPT_ORACLE_H
#define YAPT_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/yapt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_instance
{
    float o2w[12];
    float w2o[12];
    uint32_t first_index; /* into indices */
    uint32_t prim_count;
    uint32_t vertex_base;
    uint32_t material;
    uint32_t has_tangents;
    uint32_t has_uvs;
    uint32_t reserved[2];
} oracle_instance;

typedef struct oracle_texture
{
    const void* data; /* width*height RGBA texels in the yg_upload_texture format */
    uint32_t width, height, format, reserved;
} oracle_texture;

typedef struct oracle_scene
{
    const float* positions; /* 3 per vertex, object space */
    const float* normals;
    const float* tangents; /* 4 per vertex (may be NULL when no instance uses tangents) */
    const uint32_t* indices;
    const oracle_instance* instances;
    uint32_t n_instances;
    const yg_material* materials;
    uint32_t n_materials;
    const float* spectra; /* n_curves x spec_points */
    uint32_t spec_points;
    float spec_lmin, spec_lmax;
    const yg_camera* camera;
    /* tables shared with the GPU path (yg_get_table) */
    const float* luts[9];     /* YG_TABLE_LUT_* in order */
    const float* rgb_to_spd;  /* 64^3 x 3 or NULL */
    const char* data_dir;     /* CIE + Joe-Kuo data files */
    const yg_punctual_light* punctual; /* may be NULL when n_punctual is 0 */
    uint32_t n_punctual;
    const float* uvs;                  /* 2 per vertex (may be NULL when no instance has uvs) */
    const oracle_texture* textures;    /* materials refer to id + 1 */
    uint32_t n_textures;
    uint32_t env_texture;              /* id + 1 of the environment texture, 0: |dir| */
    uint32_t env_cube;                 /* 1: env_texture is a cube map (six faces stacked), 0: longitude-latitude */
} oracle_scene;

typedef struct oracle_stats
{
    uint64_t rays;
    double seconds;
} oracle_stats;

/* Renders the crop/spp range of params with `threads` threads. precision: 32 or 64.
 * records (optional): crop_w*crop_h*spp_count x 8 floats [spp][row][col]: hero lambda,
 * L[4], XYZ. film_xyz (optional): crop_w*crop_h*3 doubles, mean XYZ over the samples. */
int oracle_render(const oracle_scene* scene, const yg_render_params* params, int precision, int threads,
                  float* records, double* film_xyz, oracle_stats* stats);

/* The uni/NEE render of every stride-th pixel of the crop in x and y (pixel (cx + i*stride,
 * cy + j*stride) with its own sample indices and seeds); film_xyz (optional) holds the mean XYZ
 * of the ceil(crop_w/stride) x ceil(crop_h/stride) rendered pixels. A bounded sample of a large
 * request for timing. */
int oracle_render_strided(const oracle_scene* scene, const yg_render_params* params, uint32_t stride, int precision,
                          int threads, double* film_xyz, oracle_stats* stats);

/* 1 when rendering params on the scene converts RGB colours to spectra (so the scene must
 * carry rgb_to_spd), 0 when not, -1 on a null argument. */
int oracle_needs_rgb_table(const oracle_scene* scene, const yg_render_params* params);

/* Sobol generator matrices derived here from the Joe-Kuo file (256 x 32 uint32). */
int oracle_sobol_matrices(const char* data_dir, uint32_t* out);

/* The a-trous denoiser (the reference's baseline denoiser), FP32 in the device order.
 * oracle_atrous_moments adds the first-camera-vertex feature moments of every sample of the
 * request onto `moments` (4 planes of width*height float4, layout of yg_atrous_read).
 * oracle_atrous runs the prefilter and the passes on the same inputs as yg_atrous_run. */
int oracle_atrous_moments(const oracle_scene* scene, const yg_render_params* params, int threads, float* moments);
int oracle_atrous(uint32_t width, uint32_t height, const float* film_sum, const float* odd_sum, const float* moments,
                  const yg_camera* camera, const yg_atrous_params* params, int threads, float* out_xyzw,
                  float* out_variance, uint32_t* features);

/* The precomputed tables the integrators read (YG_TABLE_SOBOL_MATRICES, YG_TABLE_LUT_*,
 * YG_TABLE_RGB_TO_SPD for [lmin, lmax]), generated on the host without a GPU. The oracle and
 * the device load the same tables by design: they are inputs of the integrator math, built by
 * the shared generator (yapt_gb300/csrc/yg_tables.cpp, linked into this library) and checked
 * on their own (brute-force integration of the LUTs, the reference's Sobol matrices). Same
 * calling convention as yg_host_table: *count receives the element count; out may be NULL. */
int oracle_host_table(const char* data_dir, int which, int lmin, int lmax, void* out, size_t capacity, size_t* count);

#ifdef __cplusplus
}
#endif
#endif
