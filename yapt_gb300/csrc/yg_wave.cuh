// Device helpers and the structure-of-arrays path state shared by the wavefront kernels
// (single request: yg_integrator.cu; merged requests of the serving loop: yg_serve_kernels.cu).
#pragma once
#include "yg_path.cuh"
#include "yg_kernels.h"

namespace yg
{

__device__ __forceinline__ uint32_t warpAppend(uint32_t* counter, bool pred)
{
    // one atomic per warp; returns this lane's slot (valid only where pred)
    // called by all 32 lanes of a warp (the callers iterate a warp-uniform trip count)
    uint32_t mask = __ballot_sync(0xffffffffu, pred);
    uint32_t lane = threadIdx.x & 31;
    uint32_t leader = mask ? (uint32_t)(__ffs(mask) - 1) : 0u;
    uint32_t base = 0;
    if (mask && lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void countRays(unsigned long long* ctr, uint32_t n)
{
    if (!ctr) return;
    for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(ctr, (unsigned long long)n);
}

__device__ __forceinline__ void countTraversal(unsigned long long* ctr, const TraversalCount& tc)
{
    if (!ctr) return;
    unsigned long long n = tc.nodes, t = tc.tris;
    for (int o = 16; o > 0; o >>= 1)
    {
        n += __shfl_down_sync(0xffffffffu, n, o);
        t += __shfl_down_sync(0xffffffffu, t, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicAdd(ctr, n);
        atomicAdd(ctr + 1, t);
    }
}

YG_DEV void pixelOf(const LaunchParams& P, uint64_t idx, uint32_t& sl, uint32_t& cx, uint32_t& cy)
{
    const uint64_t npix = (uint64_t)P.cropW * P.cropH;
    sl = (uint32_t)(idx / npix);
    uint32_t pl = (uint32_t)(idx - (uint64_t)sl * npix);
    cx = P.cropX + pl % P.cropW;
    cy = P.cropY + pl / P.cropW;
}

// The sample a wave slot renders (the wave holds samples base .. base + n - 1). Within every
// band of four full rows of a sample plane that lies wholly in the wave, 32 consecutive slots
// cover an 8x4 pixel tile, so the primary rays of a warp (and their shadow rays) start close
// together and point nearly the same way; elsewhere slots follow scanline order. A bijection
// on the wave: the film still receives every sample at its own index.
YG_DEV uint64_t sampleOfSlot(const LaunchParams& P, uint64_t base, uint32_t n, uint32_t s)
{
    const uint64_t idx = base + s;
    const uint32_t W = P.cropW;
    if ((W & 7u) != 0u) return idx;
    const uint64_t npix = (uint64_t)W * P.cropH;
    const uint64_t sl = idx / npix;
    const uint64_t pl = idx - sl * npix;
    const uint64_t band = 4ull * W;
    const uint64_t b0 = (pl / band) * band; // the band's first pixel
    if (b0 + band > npix) return idx;      // the partial band at the bottom of the plane
    const uint64_t g0 = sl * npix + b0;     // its first sample
    if (g0 < base || g0 + band > base + n) return idx;
    const uint32_t local = (uint32_t)(pl - b0);
    const uint32_t x = (local >> 5) * 8u + (local & 7u), y = (local >> 3) & 3u;
    return g0 + (uint64_t)y * W + x;
}

// Resident 128-thread blocks per SM the shading kernels ask for (__launch_bounds__ minimum): 8
// (64 registers, the rest spilled to L1-resident local memory) measured faster than 4, 6, 12 or
// 16 on the NEE workload; more warps hide the instruction-fetch and memory latency.
#ifndef YG_SHADE_MIN_BLOCKS
#define YG_SHADE_MIN_BLOCKS 8
#endif

YG_DEV Luts lutsOf(const SceneView& S)
{
    return Luts{S.lutSS, S.lutSSAvg, S.lutSSMS, S.lutSSMSAvg, S.lutTransDenser, S.lutTransLighter,
                S.lutTransAvgDenser, S.lutTransAvgLighter, S.lutSheen};
}

YG_DEV void writeSample(const SceneView& S, const LaunchParams& P, uint64_t idx, const Spectral& sp, float4 total,
                        const FirstHit& fh)
{
    float3 X = toXYZ(S, sp, total);
    P.sampleXYZ[idx] = mk4(X.x, X.y, X.z, 1.0f);
    if (P.dump)
    {
        float* d = P.dump + idx * 8;
        d[0] = sp.hero;
        d[1] = total.x; d[2] = total.y; d[3] = total.z; d[4] = total.w;
        d[5] = X.x; d[6] = X.y; d[7] = X.z;
    }
    if (P.featAlbedo)
    {
        P.featAlbedo[idx] = mk4(fh.albedo.x, fh.albedo.y, fh.albedo.z, 0.0f);
        P.featNormalDepth[idx] = mk4(fh.normal.x, fh.normal.y, fh.normal.z, fh.depth);
    }
}

// ------------------------------------------------------------------ wavefront
// Path state of one wave, structure of arrays (index = slot = sample index - wave base).
struct WaveState
{
    float4* thr;      // throughput
    float4* tot;      // accumulated radiance
    float4* orgPdf;   // ray origin, pdfThisRay
    float4* dirHero;  // ray direction, hero wavelength
    uint4* misc;      // flags | pathLength << 8 | nVol << 16, dimension cursor, scramble seed, Sobol row
    float4* volIOR;   // volume stack (RAY_MAX_VOLUMES_ENTERED = 4)
    uint4* volMat;
    float4* volAbs;   // [4][capacity]
    float4* fhAlb;    // first-hit features of the wave
    float4* fhNrm;
    uint32_t capacity;
};
struct RayQueue
{
    float4* o; // origin, slot
    float4* d; // direction
    uint32_t* count;
};
struct HitQueue
{
    float4* a;    // t, b1, b2, instance
    uint32_t* b;  // prim | front << 31, or 0xffffffff for a miss
};
struct ShadowQueue
{
    float4* o;        // origin, slot
    float4* d;        // direction, tmax
    uint2* target;    // light instance, primitive
    float4* contrib;
    uint32_t* count;
};

YG_DEV void loadPath(const WaveState& W, uint32_t s, PathState& ps, RandomSampler& rs, Spectral& sp, const SceneView& S)
{
    float4 t = W.thr[s], a = W.tot[s], o = W.orgPdf[s], d = W.dirHero[s];
    uint4 m = W.misc[s];
    ps.throughput = t;
    ps.total = a;
    ps.origin = mk3(o.x, o.y, o.z);
    ps.pdfThisRay = o.w;
    ps.dir = mk3(d.x, d.y, d.z);
    ps.flags = m.x & 0xffu;
    ps.pathLength = (m.x >> 8) & 0xffu;
    ps.nVol = (m.x >> 16) & 0xffu;
    rs.dim = m.y;
    rs.seed = m.z;
    rs.point = S.sobol + (size_t)m.w * kSobolDims;
    spectralOf(S, d.w, sp);
    if (ps.nVol)
    {
        float4 vi = W.volIOR[s];
        uint4 vm = W.volMat[s];
        ps.volIOR[0] = vi.x; ps.volIOR[1] = vi.y; ps.volIOR[2] = vi.z; ps.volIOR[3] = vi.w;
        ps.volMat[0] = vm.x; ps.volMat[1] = vm.y; ps.volMat[2] = vm.z; ps.volMat[3] = vm.w;
        for (int k = 0; k < kMaxVolumes; ++k) ps.volAbs[k] = W.volAbs[(size_t)k * W.capacity + s];
    }
}

YG_DEV void storePath(const WaveState& W, uint32_t s, const PathState& ps, const RandomSampler& rs, float hero,
                      uint32_t row, bool volumesTouched)
{
    W.thr[s] = ps.throughput;
    W.tot[s] = ps.total;
    W.orgPdf[s] = mk4(ps.origin.x, ps.origin.y, ps.origin.z, ps.pdfThisRay);
    W.dirHero[s] = mk4(ps.dir.x, ps.dir.y, ps.dir.z, hero);
    W.misc[s] = make_uint4(ps.flags | (ps.pathLength << 8) | (ps.nVol << 16), rs.dim, rs.seed, row);
    if (volumesTouched)
    {
        W.volIOR[s] = mk4(ps.volIOR[0], ps.volIOR[1], ps.volIOR[2], ps.volIOR[3]);
        W.volMat[s] = make_uint4(ps.volMat[0], ps.volMat[1], ps.volMat[2], ps.volMat[3]);
        for (int k = 0; k < kMaxVolumes; ++k) W.volAbs[(size_t)k * W.capacity + s] = ps.volAbs[k];
    }
}

// Shading coherence: before each shade pass the hit queue is regrouped by the kind of work the
// hit needs (miss, emitter, opaque dielectric base, conductor, transparent dielectric), so that
// a warp runs one branch of the layered BSDF instead of all of them. A path's result does not
// depend on its queue position.
constexpr int kShadeClasses = 5;
YG_DEV uint32_t shadeClass(const SceneView& S, float4 ha, uint32_t hb)
{
    if (hb == 0xffffffffu) return 0;
    const GpuMaterial& M = S.materials[S.instances[__float_as_uint(ha.w)].material];
    float4 e = M.emissive_roughness;
    if (e.x + e.y + e.z > 0.0f) return 1;
    if (M.albedo_transparency.w > 0.0f) return 4;
    if (M.specular_metalness.w > 0.0f) return 3;
    return 2;
}

// shading-class key of every queued hit and the class counts
template <int CLASSES>
__global__ void __launch_bounds__(256) wfClassify(const SceneView S, RayQueue Q, HitQueue H, uint8_t* keys, uint32_t* counts)
{
    const uint32_t n = *Q.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t r = 0; r < rounds; ++r)
    {
        uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + r * stride;
        bool active = i < n;
        uint32_t key = active ? shadeClass(S, H.a[i], H.b[i]) : 0xffu;
        if (active) keys[i] = (uint8_t)key;
        for (uint32_t c = 0; c < (uint32_t)CLASSES; ++c)
        {
            uint32_t m = __ballot_sync(0xffffffffu, key == c);
            if (lane == 0 && m) atomicAdd(&counts[c], (uint32_t)__popc(m));
        }
    }
}

template <int CLASSES>
__device__ __forceinline__ void regroupBody(RayQueue Q, HitQueue H, const uint8_t* keys, const uint32_t* counts,
                                            uint32_t* cursors, RayQueue Qs, HitQueue Hs)
{
    const uint32_t n = *Q.count;
    uint32_t base[CLASSES];
    uint32_t acc = 0;
    for (int c = 0; c < CLASSES; ++c)
    {
        base[c] = acc;
        acc += counts[c];
    }
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t r = 0; r < rounds; ++r)
    {
        uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + r * stride;
        bool active = i < n;
        uint32_t key = active ? keys[i] : 0xffu;
        uint32_t pos = 0;
        for (uint32_t c = 0; c < (uint32_t)CLASSES; ++c)
        {
            uint32_t m = __ballot_sync(0xffffffffu, key == c);
            if (!m) continue;
            uint32_t leader = (uint32_t)(__ffs(m) - 1);
            uint32_t b0 = 0;
            if (lane == leader) b0 = atomicAdd(&cursors[c], (uint32_t)__popc(m));
            b0 = __shfl_sync(0xffffffffu, b0, leader);
            if (key == c) pos = base[c] + b0 + __popc(m & ((1u << lane) - 1u));
        }
        if (active)
        {
            Qs.o[pos] = Q.o[i];
            Qs.d[pos] = Q.d[i];
            Hs.a[pos] = H.a[i];
            Hs.b[pos] = H.b[i];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *Qs.count = n;
}
template <int CLASSES>
__global__ void __launch_bounds__(256) wfRegroup(RayQueue Q, HitQueue H, const uint8_t* keys, const uint32_t* counts,
                                                 uint32_t* cursors, RayQueue Qs, HitQueue Hs)
{
    regroupBody<CLASSES>(Q, H, keys, counts, cursors, Qs, Hs);
}

// A barrier over every block of a cooperative launch, with a bounded wait: generation counting
// in device memory; the last block to arrive starts the next generation. A block that waits
// longer than `limit` polls records the time-out in `error` and every block returns false, so
// a kernel never hangs on a block that does not arrive. `expected` is normally gridDim.x.
struct GridBarrier
{
    unsigned int count, gen, error, expected;
};
__device__ __forceinline__ bool gridSync(GridBarrier* b, uint32_t limit)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        ok = 1;
        volatile unsigned int* vgen = &b->gen;
        volatile unsigned int* verr = &b->error;
        const unsigned int g = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(&b->count, 1u) + 1u;
        if (arrived == b->expected)
        {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        }
        else
        {
            uint32_t polls = 0;
            while (*vgen == g)
            {
                if (*verr != 0u || ++polls > limit)
                {
                    atomicExch(&b->error, 1u);
                    break;
                }
                __nanosleep(128);
            }
        }
        __threadfence();
        if (*verr != 0u) ok = 0;
    }
    __syncthreads();
    return ok != 0;
}

} // namespace yg
