// Kernel launchers shared between the CUDA translation units and the C-ABI runtime.
#pragma once
#include "yg_types.h"

#include <string>
#include <vector>

namespace yg
{
int launchPathKernel(const SceneView& S, const LaunchParams& P, int smCount, cudaStream_t stream);
// Wavefront integrator over P.nSamples samples in waves of `capacity` paths; `arena`
// holds capacity * wavefrontBytesPerSlot() bytes plus 64 KB. Returns the launch count.
size_t wavefrontBytesPerSlot();
// Device-built 8-wide BVH (yg_bvh_build.cu). Input: the instances, object-space vertex and
// index pools already on the device, and the first primitive of every instance (host,
// nInstances + 1 prefix sums of primCount). Output: leaf-ordered world-space triangles (3
// float4 each: v0 + instance, e1 + primitive, e2) and 80-byte wide nodes (5 float4, layout
// in yg_trace.cuh), both allocated with cudaMalloc and owned by the caller.
constexpr int kMaxLeafTris = 3;   // triangles per wide-node leaf slot
constexpr int kWideMaxDepth = 30; // wide levels (the traversal stack holds one entry per level)
struct WideBvhInput
{
    const GpuInstance* instances;
    uint32_t nInstances;
    std::vector<uint32_t> instPrimStart;
    const float* positions;
    const uint32_t* indices;
    uint32_t nPrims;
    const float2* uvs;              // texture coordinates of the vertices (alpha-tested meshes)
    const GpuAlphaSource* alpha;    // indexed by GpuInstance::alphaSource - 1; null: no cutouts
};
struct WideBvhOutput
{
    float4* tris;
    float4* nodes;
    uint32_t nNodes;
    uint32_t depth;
    float lo[3], hi[3]; // world bounds of all triangles
};
int buildWideBvh(const WideBvhInput& in, WideBvhOutput& out, cudaStream_t stream, std::string& error);
// out[primStart[instance] + primitive] = position of that triangle in tris (nTris triangles of
// 48 bytes in leaf order), 0xffffffff where none; returns a cudaError_t
int indexTrianglesByPrim(const float4* tris, uint32_t nTris, const uint32_t* primStart, uint32_t* out, cudaStream_t stream);

// Kernel kinds of the timer (the C-ABI's YG_KERNEL_* values).
constexpr uint8_t kKernelTrace = 0, kKernelRegroup = 1, kKernelShade = 2, kKernelShadow = 3, kKernelConnect = 4;
// Optional CUDA-event timing of launches by kind: events[2k], events[2k+1] bracket the k-th
// timed launch, whose kind is kinds[k]. Timing stops when the events run out.
struct KernelTimer
{
    cudaEvent_t* events;
    uint8_t* kinds;
    uint32_t capacity; // launches
    uint32_t used;
    void begin(cudaStream_t s)
    {
        if (used < capacity) cudaEventRecord(events[2 * used], s);
    }
    void end(uint8_t kind, cudaStream_t s)
    {
        if (used < capacity)
        {
            cudaEventRecord(events[2 * used + 1], s);
            kinds[used++] = kind;
        }
    }
};
// Traversal counters (LaunchParams::traversalCounter): [0] nodes and [1] triangles of
// closest-hit rays, [2] nodes and [3] triangles of shadow rays, [4] closest-hit rays,
// [5] shadow rays (the path kernel counts all rays' work in [0] and [1]).
constexpr int kTraversalCounters = 6;
int launchWavefront(const SceneView& S, const LaunchParams& P, void* arena, uint32_t capacity, int smCount,
                    cudaStream_t stream, KernelTimer* timer = nullptr);
int launchFilm(float4* sum, float4* comp, const float4* samples, uint32_t width, uint32_t cx, uint32_t cy, uint32_t cw,
               uint32_t ch, uint32_t nspp, int smCount, cudaStream_t stream);
int launchFeatures(float4* accA, float4* accN, const float4* fa, const float4* fn, uint32_t width, uint32_t cx, uint32_t cy,
                   uint32_t cw, uint32_t ch, uint32_t nspp, int smCount, cudaStream_t stream);
int launchSobolPoints(const uint32_t* matrices, uint32_t start, uint32_t count, uint32_t* out, int smCount, cudaStream_t stream);
int launchFilmResolve(const float4* sum, const float4* accA, const float4* accN, uint64_t n, float* xyz, float* albedo,
                      float* normal, float* depth, int smCount, cudaStream_t stream);
int launchRelmse(const float4* sum, const float* ref, uint32_t npix, double eps, double* out, int smCount,
                 cudaStream_t stream);
// Edge-stopping a-trous denoiser (the reference's denoiser, kept as a baseline).
struct AtrousSettings
{
    float depthSigmaScale, normalSigma, materialSigma, colorSigma, featureVarianceScale;
    uint32_t prefilter, passes;
};
struct AtrousBuffers
{
    uint32_t width, height;
    float invW, invH;
    float uvToView[16], viewToWorld[16]; // row-major camera matrices
    const float4* film;    // [pixel] XYZ sums and sample count
    const float4* odd;     // [pixel] XYZ sums and count of the odd-indexed samples
    const float4* moments; // [4][pixel] feature moment sums
    uint4* feat0;          // [pixel] packed prefiltered features, two halves
    uint4* feat1;
    float4* colour[2];     // ping-pong colour planes; [0] receives the merged input colour
    float* variance[2];
};
int launchAtrousGather(const SceneView& S, const LaunchParams& P, float4* moments, float4* odd, const float4* samples,
                       uint32_t nspp, int smCount, cudaStream_t stream);
int launchAtrous(const AtrousBuffers& B, const AtrousSettings& A, float4* outColour, float* outVar, cudaStream_t stream);
// The tonemap stage's display path: histogram auto-exposure and the ACES fitted curve to RGBA8.
struct DisplayArgs
{
    uint32_t width, height;
    const float4* film;   // film sums and counts (used when atrous is null)
    const float4* atrous; // the a-trous filter's XYZ output, or null
    uint32_t* histogram;  // 128 buckets
    float* exposure;      // persistent device state
    float* stats;         // [0] mean luminance of the frame
    uint32_t* out;        // RGBA8, one word a pixel
    uint32_t tonemap, autoExposure, init;
    float exposureParam;  // the manual exposure, or the compensation (EV) with auto exposure
    float deltaTime, adaptSpeed;
};
int launchDisplay(const DisplayArgs& A, int smCount, cudaStream_t stream);
// Merged wavefront of several requests (serving). All tables live in device memory and are
// read by the kernels, so a captured launch sequence can be replayed round after round.
struct MultiTables
{
    const SceneView* views;      // [request slot] scene arrays, Sobol points of the round
    const LaunchParams* params;  // [request slot] image, depth, integrator, sample buffer of the round
    const uint32_t* segReq;      // [segment] request slot
    const uint32_t* segStart;    // [segment + 1] first wave slot (prefix sums of plane counts x pixels)
    const uint32_t* segPixStart; // [segment + 1] first pixel of the film pass (prefix sums of pixels)
    const uint32_t* nSeg;        // segments in this round
    float4* const* filmSum;      // [request slot] Kahan film sums and compensations
    float4* const* filmComp;
    uint32_t* req;               // [wave slot] request slot (set by the launcher)
    uint32_t* local;             // [wave slot] sample index within the request's round
};
size_t multiWaveBytes(uint32_t capacity);
int launchWavefrontMulti(const MultiTables& M, void* arena, uint32_t capacity, uint32_t maxDepth,
                         unsigned long long* rayCounter, int smCount, cudaStream_t stream);
// The same round as one persistent cooperative kernel with bounded grid barriers (`barrier`:
// 16 bytes of device memory; its third word is nonzero after a barrier ran out of `pollLimit`
// polls). Returns the launch count, or minus the CUDA error of the launch.
struct GridBarrier;
int launchWavefrontMultiPersistent(const MultiTables& M, void* arena, uint32_t capacity, uint32_t maxDepth,
                                   unsigned long long* rayCounter, int smCount, cudaStream_t stream, GridBarrier* barrier,
                                   uint32_t pollLimit);
// Cooperative probe of the grid barrier: `missing` blocks never arrive. *passes counts the
// barriers each block passed; the barrier's error word tells whether the wait ran out.
int gridBarrierCheck(GridBarrier* barrier, uint32_t* passes, uint32_t missing, uint32_t pollLimit, int smCount,
                     cudaStream_t stream, uint32_t* blocks);
// Bidirectional integrator over P.sppCount sample indices. `arena` holds
// bdptArenaBytes(P.sppCount, lightPaths, maxLightVerts, cropW*cropH) bytes; `perm` is a
// permutation of the crop's pixel indices (camera groups take 64 consecutive entries).
constexpr uint32_t kBdptMaxLightVertices = 16; // MAX_LIGHT_PATH_VERTICES_HARD_LIMIT
size_t bdptArenaBytes(uint32_t frames, uint32_t lightPaths, uint32_t maxLightVerts, uint64_t cropPixels);
// With a timer: wbTrace as trace, the class keys and regroup as regroup, wbShade as shade,
// wbConnect as connect, wbVisibility and wbAccumulate as shadow. With P.traversalCounter, the
// connection records are counted as shadow rays.
int launchBdpt(const SceneView& S, const LaunchParams& P, void* arena, const uint32_t* perm, uint32_t lightPaths,
               uint32_t maxLightVerts, float3 worldCenter, float worldRadiusSqr, int smCount, cudaStream_t stream,
               KernelTimer* timer = nullptr);
// bytes one connection record moves in wbConnect: its (slot, light vertex) pair, the camera
// vertex's surface, context and state, the prepared light vertex, and the record written
uint32_t bdptConnectionRecordBytes();
} // namespace yg
