// Device-resident scene layout shared by the host runtime and the CUDA kernels.
//
// HBM layout (one context, all arrays 16-byte aligned, read-only during a render):
//   tris      float4[3 * T]  world-space triangles in BVH leaf order:
//                            (v0.xyz, instance) (e1.xyz, primitive) (e2.xyz, 0)
//   nodes     float4[4 * N]  binary BVH, two child boxes per node (64 B)
//   instances GpuInstance[I] per (render object, submesh): transforms, mesh refs
//   materials GpuMaterial[M] principled parameters after the reference's clamps
//   vertex pools (object space): positions/normals float[3V], tangents float4[V],
//   uvs float2[V], indices uint32 (local to the mesh, offset by vertex_base)
//   LUTs / CIE / Sobol tables (a few hundred KB, L2 resident)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace yg
{

constexpr int kSobolDims = 256;       // NUMBER_OF_RANDOM_SAMPLE_DIMENSIONS (raytraceCommon.hlsl:12)
constexpr int kMaxVolumes = 4;        // RAY_MAX_VOLUMES_ENTERED (raytraceCommon.hlsl:19)
constexpr float kRayMinT = 5e-4f;     // DEFAULT_RAY_MIN_T (raytraceCommon.hlsl:24)
constexpr int kLutSS = 32;            // SS_ALBEDO_LUT_DIM
constexpr int kLutSSMS = 16;          // SSMS_ALBEDO_LUT_DIM
constexpr int kLutTrans = 16;         // SS_ALBEDO_TRANSLUCENT_LUT_DIM
constexpr int kLutSheen = 16;         // SS_ALBEDO_SHEEN_LUT_DIM
constexpr int kRgbLutRes = 64;        // SRGB_TO_SPD_RES (spectralConstants.h:27)

// MaterialEntryGPU (materialsCommonResources.hlsl:10-38) after the clamps of
// BindlessMaterialManager.cpp:73-98, plus spectral curve references.
struct alignas(16) GpuMaterial
{
    float4 specAmount_ccAmount_ccIOR_ccRough;
    float4 albedo_transparency;
    float4 specular_metalness;
    float4 absorption_ior;
    float4 emissive_roughness;
    float anisotropy, anisotropyRotation;
    uint32_t mask;
    float thinFilmNM;
    float cauchyA, cauchyB, sheenAmount, emissionFocus;
    float4 sheenColor_roughness;
    float4 subsurfaceRadius_amount;
    int albedoSpectrum, specularSpectrum, emissionSpectrum, pad;
    int4 textures;            // albedo, normal, ORM, emissive texture index (-1: none)
    float4 albedoNormalScale; // uv scales of the albedo (xy) and normal (zw) textures
    float4 ormEmissiveScale;  // uv scales of the ORM (xy) and emissive (zw) textures
};

constexpr uint32_t kMaterialTextured = 1u << 8; // GpuMaterial::mask: some texture slot is bound

// A 2D texture, decoded to linear float RGBA at upload, sampled bilinearly with wrapping
// (the reference's LINEAR_REPEAT colour sampler at mip 0)
struct alignas(16) GpuTexture
{
    const float4* texels; // row major, width x height
    uint32_t width, height;
};

// Per (render object, submesh) instance: RenderObjectTransformDataGPU + MeshEntryGPU refs.
struct alignas(16) GpuInstance
{
    float4 o2w[3];
    float4 w2o[3];
    uint32_t firstIndex;  // into the index pool
    uint32_t primCount;   // triangles of the submesh
    uint32_t vertexBase;  // added to the mesh-local indices
    uint32_t material;
    float lightPdf;       // g_instanceLightSelectionPDFs entry (0: not a light)
    uint32_t hasTangents;
    uint32_t hasUVs;
    uint32_t alphaSource; // id + 1 of the instance's GpuAlphaSource, 0: opaque
};

// The cutout of an alpha-tested instance (alphaTestPasses, hitShadersCommon.hlsl:162-183): a
// material with an alpha cutoff above 0 and an albedo texture, on a mesh with texture
// coordinates. Traversal rejects a candidate hit whose albedo alpha at the hit's uv (times
// the albedo uv scale) is below the cutoff. Used by the scene build only, which copies it into
// the per-triangle cutout records behind the triangles.
struct alignas(16) GpuAlphaSource
{
    const float4* texels;
    uint32_t size;   // width | height << 16 (textures are at most 32768 texels wide)
    float cutoff;
    float su, sv;    // albedo uv scale
    uint32_t pad[2];
};

// LightEntryGPU (materialsCommonResources.hlsl:51-71): the mesh lights first, then the
// punctual lights, which also carry a second alias table over the punctual lights alone
// (used when they are the only explicitly sampled lights, i.e. without NEE).
constexpr uint32_t kLightMesh = 0, kLightPoint = 1, kLightSpot = 2, kLightDirectional = 3;
constexpr uint32_t kPunctualShadow = 0xffffffffu; // shadow-ray target of a punctual light: nothing may be hit
struct alignas(16) GpuLight
{
    uint32_t instance; // mesh lights
    float selectionPdf;
    float aliasThreshold;
    uint32_t aliasIndex;
    uint32_t type;     // kLight*
    float punctualSelectionPdf;
    float punctualAliasThreshold;
    uint32_t punctualAliasIndex;
    float4 positionCosInner;  // punctual: world position, cos of the spot's inner angle
    float4 directionCosOuter; // punctual: world direction of emission, cos of the outer angle
    float4 intensity;         // punctual: RGB intensity (irradiance for directional lights)
};

struct alignas(16) GpuCamera
{
    float uvToView[16];
    float viewToUV[16];
    float worldToView[16];
    float viewToWorld[16];
    float apertureRadius, focusDistance, forwardZSign, pad;
};

// All read-only tables and scene arrays a render kernel needs.
struct SceneView
{
    const float4* tris;
    const float4* nodes;
    const GpuInstance* instances;
    const GpuMaterial* materials;
    const GpuLight* lights;
    const float* positions;
    const float* normals;
    const float4* tangents;
    const float2* uvs;
    const uint32_t* indices;
    const float* spectra;  // n_curves x specPoints
    const float* lutSS, *lutSSAvg, *lutSSMS, *lutSSMSAvg;
    const float* lutTransDenser, *lutTransLighter, *lutTransAvgDenser, *lutTransAvgLighter;
    const float* lutSheen;
    const float4* cie;     // (xbar, ybar, zbar, d65) per 1 nm over [lambdaMin, lambdaMax]
    const float* rgbToSpd; // 64^3 x 3, may be null
    const uint32_t* sobol; // [spp_count][kSobolDims] points of this launch
    const uint32_t* instPrimStart; // first primitive of each instance in the scene's primitive order
    const uint32_t* triOfPrim;     // position in `tris` of each primitive (0xffffffff: none)
    uint32_t nNodes, nTris;        // wide nodes and triangles (bounds of the debug build's checks)
    unsigned int* boundsErrors;    // debug build (YG_DEBUG_BOUNDS): out-of-range accesses refused
    GpuCamera cam;
    const GpuTexture* textures;
    int envTexture;        // environment texture, -1: the analytic sky
    uint32_t envCube;      // 1: envTexture is a cube map (six square faces stacked), 0: longitude-latitude
    uint32_t nLights;      // mesh and punctual
    uint32_t nPunctual;    // the last nPunctual entries of lights
    uint32_t nInstances;
    uint32_t specPoints;
    float specLmin, specLmax;
    uint32_t cieN;
    float lambdaMin, lambdaMax;
    float cieYSumInv;      // CIE_Y_SUM_INV for the range
    float d65SumInv;       // CIE_D65_SUM_INV for the range
    uint32_t rootIsLeaf;
};

struct LaunchParams
{
    uint32_t integrator;
    uint32_t width, height;
    uint32_t cropX, cropY, cropW, cropH;
    uint32_t sppStart, sppCount;
    uint32_t maxDepth;
    uint32_t regularizeAfter;
    uint32_t regularizeEnable;
    float envScale;
    uint32_t seed;
    uint32_t flags;
    uint64_t nSamples;      // cropW * cropH * sppCount
    float4* sampleXYZ;      // [sppCount][cropH*cropW] (xyz, 1) per sample
    float* dump;            // optional per-sample records (8 floats) or null
    float4* featAlbedo;     // optional per-sample first-hit features or null
    float4* featNormalDepth;
    unsigned long long* rayCounter; // optional
    unsigned long long* traversalCounter; // optional [nodes, triangles]; selects the counting kernel
};

} // namespace yg
