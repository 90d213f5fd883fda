// Unidirectional and NEE spectral path integrators on the GPU, in two forms that
// produce bit-identical samples:
//  * wavefront (default): generate -> closest-hit traversal -> shade (emitter MIS,
//    NEE request, BSDF sample, Russian roulette) -> shadow traversal -> next bounce,
//    with path state in HBM (SoA) and ray queues compacted by warp-aggregated appends.
//    The traversal kernels carry no shading state, so they run at high occupancy.
//  * megakernel: one thread traces one path to the end (kept as a cross-check).
// Samples of a launch are written to a [sample][pixel] buffer and folded into the
// film in sample order, so the film does not depend on thread scheduling.
#include "yg_wave.cuh"
#include "yg_nvtx.h"

#include <algorithm>

namespace yg
{

// ------------------------------------------------------------------ megakernel
template <bool NEE, bool COUNT>
__global__ void __launch_bounds__(128) pathKernel(const __grid_constant__ SceneView S, const __grid_constant__ LaunchParams P)
{
    Luts Lt = lutsOf(S);
    TraversalCount tc{0, 0};
    uint32_t rays = 0;
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < P.nSamples;
         idx += (uint64_t)gridDim.x * blockDim.x)
    {
        uint32_t sl, cx, cy;
        pixelOf(P, idx, sl, cx, cy);
        uint32_t seed = (cy * P.width + cx) ^ (P.seed * 0x9E3779B9u);
        RandomSampler rs{S.sobol + (size_t)sl * kSobolDims, 2u, seed};
        Spectral sp;
        PathState ps;
        beginPath(S, P, cx, cy, rs, sp, ps);
        FirstHit fh{mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f), 0.0f};
        bool alive = true;
        for (uint32_t bounce = 0; bounce < P.maxDepth && alive; ++bounce)
        {
            Hit hit;
            rays++;
            bool found = traceClosest<COUNT>(S, ps.origin, ps.dir, kRayMinT, __int_as_float(0x7f800000), hit, &tc);
            ShadowRequest sr;
            alive = shadeSegment<NEE>(S, P, Lt, sp, found, hit, ps, rs, sr, P.featAlbedo ? &fh : nullptr);
            if (sr.valid)
            {
                rays++;
                if (traceShadow<COUNT>(S, sr.origin, sr.dir, kRayMinT, sr.tmax, sr.instance, sr.prim, &tc))
                    ps.total = ps.total + sr.contrib;
            }
        }
        writeSample(S, P, idx, sp, ps.total, fh);
    }
    countRays(P.rayCounter, rays);
    if (COUNT) countTraversal(P.traversalCounter, tc);
}

// ------------------------------------------------------------------ wavefront
// The path state travels with its ray. A PathQueue holds the live paths of a wave in queue
// order (structure of arrays): the regroup before shading moves each path's whole record with
// its hit, so the shading kernel reads and writes contiguous records instead of gathering the
// state of scattered slots. What stays per slot (sample): the volume stack (touched only inside
// media), the first-hit features and the final radiance of paths that ended.
struct PathQueue
{
    float4* thr;     // throughput
    float4* tot;     // accumulated radiance
    float4* orgPdf;  // ray origin, pdf of the ray
    float4* dirHero; // ray direction, hero wavelength
    uint4* misc;     // flags | pathLength << 8 | nVol << 16, dimension cursor, scramble seed, Sobol row
    uint32_t* slot;  // the sample's slot in the wave
    uint32_t* count;
};
struct SlotState
{
    float4* finalTot; // radiance of the ended path (x, y, z, w lanes); finalHero its hero wavelength
    float* finalHero;
    float4* volIOR;   // volume stack (RAY_MAX_VOLUMES_ENTERED = 4)
    uint4* volMat;
    float4* volAbs;   // [4][capacity]
    float4* fhAlb;    // first-hit features
    float4* fhNrm;
    uint32_t capacity;
};
// shadow-queue target of a path that ended at this vertex: its slot, flagged
constexpr uint32_t kShadowToSlot = 0x80000000u;

YG_DEV void loadQueued(const PathQueue& Q, uint32_t i, const SlotState& W, uint32_t slot, PathState& ps,
                       RandomSampler& rs, Spectral& sp, const SceneView& S)
{
    float4 t = Q.thr[i], a = Q.tot[i], o = Q.orgPdf[i], d = Q.dirHero[i];
    uint4 m = Q.misc[i];
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
        float4 vi = W.volIOR[slot];
        uint4 vm = W.volMat[slot];
        ps.volIOR[0] = vi.x; ps.volIOR[1] = vi.y; ps.volIOR[2] = vi.z; ps.volIOR[3] = vi.w;
        ps.volMat[0] = vm.x; ps.volMat[1] = vm.y; ps.volMat[2] = vm.z; ps.volMat[3] = vm.w;
        for (int k = 0; k < kMaxVolumes; ++k) ps.volAbs[k] = W.volAbs[(size_t)k * W.capacity + slot];
    }
}

YG_DEV void storeQueued(const PathQueue& Q, uint32_t k, uint32_t slot, const PathState& ps, const RandomSampler& rs,
                        float hero, uint32_t row)
{
    Q.thr[k] = ps.throughput;
    Q.tot[k] = ps.total;
    Q.orgPdf[k] = mk4(ps.origin.x, ps.origin.y, ps.origin.z, ps.pdfThisRay);
    Q.dirHero[k] = mk4(ps.dir.x, ps.dir.y, ps.dir.z, hero);
    Q.misc[k] = make_uint4(ps.flags | (ps.pathLength << 8) | (ps.nVol << 16), rs.dim, rs.seed, row);
    Q.slot[k] = slot;
}

YG_DEV void storeVolumes(const SlotState& W, uint32_t slot, const PathState& ps)
{
    W.volIOR[slot] = mk4(ps.volIOR[0], ps.volIOR[1], ps.volIOR[2], ps.volIOR[3]);
    W.volMat[slot] = make_uint4(ps.volMat[0], ps.volMat[1], ps.volMat[2], ps.volMat[3]);
    for (int k = 0; k < kMaxVolumes; ++k) W.volAbs[(size_t)k * W.capacity + slot] = ps.volAbs[k];
}

__global__ void __launch_bounds__(256) wfGenerate(const __grid_constant__ SceneView S, const __grid_constant__ LaunchParams P, SlotState W, PathQueue Q,
                                                  uint64_t base, uint32_t n)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        uint64_t idx = sampleOfSlot(P, base, n, s);
        uint32_t sl, cx, cy;
        pixelOf(P, idx, sl, cx, cy);
        uint32_t seed = (cy * P.width + cx) ^ (P.seed * 0x9E3779B9u);
        RandomSampler rs{S.sobol + (size_t)sl * kSobolDims, 2u, seed};
        Spectral sp;
        PathState ps;
        beginPath(S, P, cx, cy, rs, sp, ps);
        storeQueued(Q, s, s, ps, rs, sp.hero, sl);
        if (P.featAlbedo)
        {
            W.fhAlb[s] = splat4(0.0f);
            W.fhNrm[s] = splat4(0.0f);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *Q.count = n;
}

// Closest hits of the queued paths, each with its shading-class key for the regroup (the class
// counts are summed per group of lanes that finish together, one atomic per class and group).
template <bool COUNT>
__global__ void __launch_bounds__(128, YG_TRACE_MIN_BLOCKS) wfTrace(const __grid_constant__ SceneView S, PathQueue Q, HitQueue H, uint8_t* keys,
                                               uint32_t* classCounts, unsigned long long* rayCtr, unsigned long long* travCtr)
{
    const uint32_t n = *Q.count;
    TraversalCount tc{0, 0};
    uint32_t rays = 0;
    traceGrid<COUNT>(
        n,
        [&](TraceState& t, uint32_t i) {
            const float4 o = Q.orgPdf[i], d = Q.dirHero[i];
            traceBegin(t, S, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), kRayMinT, __int_as_float(0x7f800000));
        },
        [&](const TraceState& t, uint32_t i) {
            const float4 a = mk4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.instance));
            const uint32_t b = t.found ? (t.h.prim | (t.h.front ? 0x80000000u : 0u)) : 0xffffffffu;
            H.a[i] = a;
            H.b[i] = b;
            const uint32_t key = shadeClass(S, a, b);
            keys[i] = (uint8_t)key;
            const uint32_t group = __activemask();
            const uint32_t leader = (uint32_t)(__ffs(group) - 1);
            for (uint32_t c = 0; c < (uint32_t)kShadeClasses; ++c)
            {
                const uint32_t m = __ballot_sync(group, key == c);
                if ((threadIdx.x & 31u) == leader && m) atomicAdd(&classCounts[c], (uint32_t)__popc(m));
            }
        },
        tc, rays);
    countRays(rayCtr, rays);
    if (COUNT)
    {
        countTraversal(travCtr, tc);
        countRays(travCtr + 4, rays);
    }
}

// Moves every queued path (record and hit) to its class range: warp-aggregated cursors per class.
__global__ void __launch_bounds__(256) wfRegroupQ(PathQueue A, HitQueue H, const uint8_t* keys, const uint32_t* counts,
                                                  uint32_t* cursors, PathQueue B, HitQueue HB)
{
    const uint32_t n = *A.count;
    uint32_t base[kShadeClasses];
    uint32_t acc = 0;
    for (int c = 0; c < kShadeClasses; ++c)
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
        for (uint32_t c = 0; c < (uint32_t)kShadeClasses; ++c)
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
            B.thr[pos] = A.thr[i];
            B.tot[pos] = A.tot[i];
            B.orgPdf[pos] = A.orgPdf[i];
            B.dirHero[pos] = A.dirHero[i];
            B.misc[pos] = A.misc[i];
            B.slot[pos] = A.slot[i];
            HB.a[pos] = H.a[i];
            HB.b[pos] = H.b[i];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *B.count = n;
}

// Shades the regrouped hits of shading classes [classLo, classHi): a contiguous range of the
// regrouped queue, located from the class counts. The host launches one class group at a time,
// so that the warps resident on an SM run one kind of surface and share its instructions.
// Continuing paths are appended to Qout (record by record), ended ones leave their radiance in
// their slot.
template <bool NEE>
__global__ void __launch_bounds__(128, YG_SHADE_MIN_BLOCKS) wfShade(const __grid_constant__ SceneView S, const __grid_constant__ LaunchParams P, SlotState W,
                                                                   PathQueue Qin, HitQueue H, PathQueue Qout, ShadowQueue SQ,
                                                                   const uint32_t* classCounts, uint32_t classLo,
                                                                   uint32_t classHi)
{
    Luts Lt = lutsOf(S);
    uint32_t begin = 0, n = 0;
    for (uint32_t c = 0; c < classHi; ++c)
    {
        if (c < classLo) begin += classCounts[c];
        else n += classCounts[c];
    }
    // uniform trip count per warp so that the warp-wide appends see every lane
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r)
    {
        uint32_t j = first + r * stride;
        bool active = j < n;
        uint32_t i = begin + j;
        bool alive = false;
        ShadowRequest sr;
        sr.valid = false;
        uint32_t slot = 0;
        PathState ps;
        RandomSampler rs;
        Spectral sp;
        if (active)
        {
            slot = Qin.slot[i];
            loadQueued(Qin, i, W, slot, ps, rs, sp, S);
            uint32_t nVol0 = ps.nVol;
            float4 ha = H.a[i];
            uint32_t hb = H.b[i];
            bool found = hb != 0xffffffffu;
            Hit hit;
            hit.t = ha.x;
            hit.b1 = ha.y;
            hit.b2 = ha.z;
            hit.instance = __float_as_uint(ha.w);
            hit.prim = hb & 0x7fffffffu;
            hit.front = (hb & 0x80000000u) != 0;
            FirstHit fh{mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f), 0.0f};
            bool first = ps.pathLength == 0;
            alive = shadeSegment<NEE>(S, P, Lt, sp, found, hit, ps, rs, sr, P.featAlbedo ? &fh : nullptr);
            if (first && P.featAlbedo)
            {
                W.fhAlb[slot] = mk4(fh.albedo.x, fh.albedo.y, fh.albedo.z, 0.0f);
                W.fhNrm[slot] = mk4(fh.normal.x, fh.normal.y, fh.normal.z, fh.depth);
            }
            alive = alive && ps.pathLength < P.maxDepth;
            if (ps.nVol != 0 || nVol0 != 0) storeVolumes(W, slot, ps);
            if (!alive)
            {
                W.finalTot[slot] = ps.total;
                W.finalHero[slot] = sp.hero;
            }
        }
        uint32_t k = warpAppend(Qout.count, alive);
#ifdef YG_DEBUG_BOUNDS
        if (alive && !YG_BOUNDS(k < W.capacity, S.boundsErrors)) alive = false;
#endif
        if (alive) storeQueued(Qout, k, slot, ps, rs, sp.hero, (uint32_t)(rs.point - S.sobol) / kSobolDims);
        if (NEE || S.nPunctual > 0)
        {
            uint32_t q = warpAppend(SQ.count, sr.valid);
#ifdef YG_DEBUG_BOUNDS
            if (sr.valid && !YG_BOUNDS(q < W.capacity, S.boundsErrors)) sr.valid = false;
#endif
            if (sr.valid)
            {
                SQ.o[q] = mk4(sr.origin.x, sr.origin.y, sr.origin.z, __uint_as_float(alive ? k : (slot | kShadowToSlot)));
                SQ.d[q] = mk4(sr.dir.x, sr.dir.y, sr.dir.z, sr.tmax);
                SQ.target[q] = make_uint2(sr.instance, sr.prim);
                SQ.contrib[q] = sr.contrib;
            }
        }
    }
}

// Shadow rays: a visible light adds its contribution to the path's record in the next queue, or
// to the slot of a path that ended at this vertex.
template <bool COUNT>
__global__ void __launch_bounds__(128, YG_SHADOW_MIN_BLOCKS) wfShadow(const __grid_constant__ SceneView S, SlotState W, PathQueue Qnext, ShadowQueue SQ,
                                                unsigned long long* rayCtr, unsigned long long* travCtr)
{
    const uint32_t n = *SQ.count;
    TraversalCount tc{0, 0};
    uint32_t rays = 0;
    uint2 tg = make_uint2(0u, 0u);
    bool early = false;
    traceGridStop<COUNT>(
        n,
        [&](TraceState& t, uint32_t i) {
            const float4 o = SQ.o[i], d = SQ.d[i];
            tg = SQ.target[i];
            early = shadowBegin(t, S, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), kRayMinT, d.w, tg.x, tg.y);
        },
        [&](const TraceState& t, uint32_t i) {
            if (shadowVisible(t.found, t.h, tg.x, tg.y))
            {
                const uint32_t to = __float_as_uint(SQ.o[i].w);
                if (to & kShadowToSlot)
                {
                    const uint32_t s = to & ~kShadowToSlot;
                    W.finalTot[s] = W.finalTot[s] + SQ.contrib[i];
                }
                else
                {
                    Qnext.tot[to] = Qnext.tot[to] + SQ.contrib[i];
                }
            }
        },
        [&](const TraceState& t) { return shadowStopped(t, early, tg.x, tg.y); }, tc, rays);
    countRays(rayCtr, rays);
    if (COUNT)
    {
        countTraversal(travCtr + 2, tc);
        countRays(travCtr + 5, rays);
    }
}

__global__ void __launch_bounds__(256) wfFinalize(const __grid_constant__ SceneView S, const __grid_constant__ LaunchParams P, SlotState W, uint64_t base,
                                                  uint32_t n)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        Spectral sp;
        spectralOf(S, W.finalHero[s], sp);
        FirstHit fh{mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f), 0.0f};
        if (P.featAlbedo)
        {
            float4 a = W.fhAlb[s], nd = W.fhNrm[s];
            fh.albedo = mk3(a.x, a.y, a.z);
            fh.normal = mk3(nd.x, nd.y, nd.z);
            fh.depth = nd.w;
        }
        writeSample(S, P, sampleOfSlot(P, base, n, s), sp, W.finalTot[s], fh);
    }
}

// Film: Kahan-compensated FP32 running sums of XYZ and sample count per pixel,
// folded in sample order (one thread per pixel, samples of the launch in order).
__global__ void filmAccumulateKernel(float4* __restrict__ sum, float4* __restrict__ comp, const float4* __restrict__ samples,
                                     uint32_t width, uint32_t cropX, uint32_t cropY, uint32_t cropW, uint32_t cropH,
                                     uint32_t nspp)
{
    uint32_t npix = cropW * cropH;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x)
    {
        uint32_t x = cropX + p % cropW, y = cropY + p / cropW;
        size_t fi = (size_t)y * width + x;
        float4 s = sum[fi], c = comp[fi];
        for (uint32_t k = 0; k < nspp; ++k)
        {
            float4 v = samples[(size_t)k * npix + p];
            float4 yv = v - c;
            float4 t = s + yv;
            c = (t - s) - yv;
            s = t;
        }
        sum[fi] = s;
        comp[fi] = c;
    }
}

__global__ void featAccumulateKernel(float4* __restrict__ accA, float4* __restrict__ accN, const float4* __restrict__ fa,
                                     const float4* __restrict__ fn, uint32_t width, uint32_t cropX, uint32_t cropY,
                                     uint32_t cropW, uint32_t cropH, uint32_t nspp)
{
    uint32_t npix = cropW * cropH;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x)
    {
        uint32_t x = cropX + p % cropW, y = cropY + p / cropW;
        size_t fi = (size_t)y * width + x;
        float4 a = accA[fi], n = accN[fi];
        for (uint32_t k = 0; k < nspp; ++k)
        {
            a = a + fa[(size_t)k * npix + p];
            n = n + fn[(size_t)k * npix + p];
        }
        accA[fi] = a;
        accN[fi] = n;
    }
}

// relMSE reduction in FP64: sum over pixels/channels of (x - r)^2 / (r^2 + eps)
__global__ void relmseKernel(const float4* __restrict__ sum, const float* __restrict__ ref, uint32_t npix, double eps,
                             double* __restrict__ out)
{
    double acc = 0.0;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x)
    {
        float4 s = sum[p];
        double n = s.w > 0.0f ? (double)s.w : 1.0;
        double m[3] = {(double)s.x / n, (double)s.y / n, (double)s.z / n};
        for (int c = 0; c < 3; ++c)
        {
            double r = (double)ref[3 * (size_t)p + c];
            double d = m[c] - r;
            acc += d * d / (r * r + eps);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (uint32_t w = 0; w < (blockDim.x + 31) / 32; ++w) t += red[w];
        atomicAdd(out, t);
    }
}

// Sobol points of sample indices [start, start + count), kSobolDims each: the XOR of the
// generator-matrix columns of the set bits of the index (sobolUint, RandUtility.inl:34-46)
__global__ void sobolPointsKernel(const uint32_t* __restrict__ matrices, uint32_t start, uint32_t count,
                                  uint32_t* __restrict__ out)
{
    const uint64_t total = (uint64_t)count * kSobolDims;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t dim = (uint32_t)(i % kSobolDims);
        uint32_t index = start + (uint32_t)(i / kSobolDims);
        const uint32_t* m = matrices + dim * 32;
        uint32_t v = 0;
        for (int b = 0; index != 0; index >>= 1, ++b)
            if (index & 1u) v ^= m[b];
        out[i] = v;
    }
}

int launchSobolPoints(const uint32_t* matrices, uint32_t start, uint32_t count, uint32_t* out, int smCount, cudaStream_t stream)
{
    const uint64_t total = (uint64_t)count * kSobolDims;
    int blocks = (int)std::min<uint64_t>((total + 255) / 256, (uint64_t)smCount * 8);
    sobolPointsKernel<<<std::max(blocks, 1), 256, 0, stream>>>(matrices, start, count, out);
    return 1;
}

// film means on the device: XYZ (and first-hit features) divided by the sample count
__global__ void filmResolveKernel(const float4* __restrict__ sum, const float4* __restrict__ accA,
                                  const float4* __restrict__ accN, uint64_t n, float* __restrict__ xyz,
                                  float* __restrict__ albedo, float* __restrict__ normal, float* __restrict__ depth)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const float4 s = sum[i];
        const float c = s.w > 0.0f ? 1.0f / s.w : 0.0f;
        if (xyz)
        {
            xyz[3 * i] = s.x * c;
            xyz[3 * i + 1] = s.y * c;
            xyz[3 * i + 2] = s.z * c;
        }
        if (albedo)
        {
            const float4 a = accA[i];
            albedo[3 * i] = a.x * c;
            albedo[3 * i + 1] = a.y * c;
            albedo[3 * i + 2] = a.z * c;
        }
        if (normal || depth)
        {
            const float4 nd = accN[i];
            if (normal)
            {
                normal[3 * i] = nd.x * c;
                normal[3 * i + 1] = nd.y * c;
                normal[3 * i + 2] = nd.z * c;
            }
            if (depth) depth[i] = nd.w * c;
        }
    }
}

// ---------------------------------------------------------------- launchers
int launchFilmResolve(const float4* sum, const float4* accA, const float4* accN, uint64_t n, float* xyz, float* albedo,
                      float* normal, float* depth, int smCount, cudaStream_t stream)
{
    int blocks = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)smCount * 8);
    filmResolveKernel<<<std::max(blocks, 1), 256, 0, stream>>>(sum, accA, accN, n, xyz, albedo, normal, depth);
    return 1;
}

int launchPathKernel(const SceneView& S, const LaunchParams& P, int smCount, cudaStream_t stream)
{
    const int threads = 128;
    uint64_t blocksNeeded = (P.nSamples + threads - 1) / threads;
    uint64_t maxBlocks = (uint64_t)smCount * 16;
    int blocks = (int)(blocksNeeded < maxBlocks ? blocksNeeded : maxBlocks);
    if (blocks < 1) blocks = 1;
    bool count = P.traversalCounter != nullptr;
    if (P.integrator == 1)
    {
        if (count) pathKernel<true, true><<<blocks, threads, 0, stream>>>(S, P);
        else pathKernel<true, false><<<blocks, threads, 0, stream>>>(S, P);
    }
    else
    {
        if (count) pathKernel<false, true><<<blocks, threads, 0, stream>>>(S, P);
        else pathKernel<false, false><<<blocks, threads, 0, stream>>>(S, P);
    }
    return 1;
}

size_t wavefrontBytesPerSlot()
{
    // two path queues (5 x 16 + 4 each), per slot the final radiance (16 + 4), the volume stack
    // (16 + 16 + 64) and the features (32); hits and regrouped hits (20 + 20), the shadow queue
    // (56) and the class keys (1)
    return 2 * (5 * 16 + 4) + 16 + 4 + 16 + 16 + 64 + 32 + 2 * 20 + 56 + 1;
}

// Shading launches per bounce, by class ranges of the regrouped queue: misses and emitters
// (short), opaque dielectric bases, conductors, transparent dielectrics.
#ifndef YG_SHADE_ONE_LAUNCH
constexpr uint32_t kShadeGroups[][2] = {{0, 2}, {2, 3}, {3, 4}, {4, kShadeClasses}};
#else
constexpr uint32_t kShadeGroups[][2] = {{0, kShadeClasses}};
#endif

int launchWavefront(const SceneView& S, const LaunchParams& P, void* arena, uint32_t capacity, int smCount,
                    cudaStream_t stream, KernelTimer* T)
{
    char* p = static_cast<char*>(arena);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    size_t C = capacity;
    uint32_t* counters = (uint32_t*)take(256);
    auto queue = [&](uint32_t* count) {
        PathQueue q;
        q.thr = (float4*)take(C * 16);
        q.tot = (float4*)take(C * 16);
        q.orgPdf = (float4*)take(C * 16);
        q.dirHero = (float4*)take(C * 16);
        q.misc = (uint4*)take(C * 16);
        q.slot = (uint32_t*)take(C * 4);
        q.count = count;
        return q;
    };
    PathQueue QA = queue(counters + 0), QB = queue(counters + 1);
    SlotState W;
    W.capacity = capacity;
    W.finalTot = (float4*)take(C * 16);
    W.finalHero = (float*)take(C * 4);
    W.volIOR = (float4*)take(C * 16);
    W.volMat = (uint4*)take(C * 16);
    W.volAbs = (float4*)take(C * 64);
    W.fhAlb = (float4*)take(C * 16);
    W.fhNrm = (float4*)take(C * 16);
    HitQueue H{(float4*)take(C * 16), (uint32_t*)take(C * 4)};
    HitQueue HS{(float4*)take(C * 16), (uint32_t*)take(C * 4)};
    ShadowQueue SQ{(float4*)take(C * 16), (float4*)take(C * 16), (uint2*)take(C * 8), (float4*)take(C * 16),
                   counters + 2};
    uint8_t* keys = (uint8_t*)take(C);
    uint32_t* classCounts = counters + 8; // [kShadeClasses] counts, then [kShadeClasses] cursors
    bool count = P.traversalCounter != nullptr;
    int launches = 0;
    const int traceBlocks = smCount * 16, shadeBlocks = smCount * 8;
    for (uint64_t base = 0; base < P.nSamples; base += C)
    {
        uint32_t n = (uint32_t)((P.nSamples - base) < C ? (P.nSamples - base) : C);
        int gblocks = (int)((n + 255) / 256);
        if (gblocks > smCount * 8) gblocks = smCount * 8;
        NvtxRange waveRange("wave");
        wfGenerate<<<gblocks, 256, 0, stream>>>(S, P, W, QA, base, n);
        ++launches;
        // QA: the live paths in trace order; QB: the same paths regrouped by shading class.
        // Shading reads QB and appends the continuing paths to QA again.
        for (uint32_t b = 0; b < P.maxDepth; ++b)
        {
            cudaMemsetAsync(classCounts, 0, 2 * kShadeClasses * 4, stream);
            if (T) T->begin(stream);
            if (count) wfTrace<true><<<traceBlocks, 128, 0, stream>>>(S, QA, H, keys, classCounts, P.rayCounter, P.traversalCounter);
            else wfTrace<false><<<traceBlocks, 128, 0, stream>>>(S, QA, H, keys, classCounts, P.rayCounter, nullptr);
            if (T) T->end(kKernelTrace, stream);
            if (T) T->begin(stream);
            wfRegroupQ<<<smCount * 4, 256, 0, stream>>>(QA, H, keys, classCounts, classCounts + kShadeClasses, QB, HS);
            if (T) T->end(kKernelRegroup, stream);
            cudaMemsetAsync(QA.count, 0, 4, stream);
            cudaMemsetAsync(SQ.count, 0, 4, stream);
            if (T) T->begin(stream);
            for (const auto& g : kShadeGroups)
            {
                if (P.integrator == 1)
                    wfShade<true><<<shadeBlocks, 128, 0, stream>>>(S, P, W, QB, HS, QA, SQ, classCounts, g[0], g[1]);
                else
                    wfShade<false><<<shadeBlocks, 128, 0, stream>>>(S, P, W, QB, HS, QA, SQ, classCounts, g[0], g[1]);
                ++launches;
            }
            if (T) T->end(kKernelShade, stream);
            launches += 2;
            if (P.integrator == 1 || S.nPunctual > 0)
            {
                if (T) T->begin(stream);
                if (count) wfShadow<true><<<traceBlocks, 128, 0, stream>>>(S, W, QA, SQ, P.rayCounter, P.traversalCounter);
                else wfShadow<false><<<traceBlocks, 128, 0, stream>>>(S, W, QA, SQ, P.rayCounter, nullptr);
                if (T) T->end(kKernelShadow, stream);
                ++launches;
            }
        }
        wfFinalize<<<gblocks, 256, 0, stream>>>(S, P, W, base, n);
        ++launches;
    }
    return launches;
}

int launchFilm(float4* sum, float4* comp, const float4* samples, uint32_t width, uint32_t cx, uint32_t cy, uint32_t cw,
               uint32_t ch, uint32_t nspp, int smCount, cudaStream_t stream)
{
    uint32_t npix = cw * ch;
    int threads = 256;
    int blocks = (int)((npix + threads - 1) / threads);
    if (blocks > smCount * 8) blocks = smCount * 8;
    if (blocks < 1) blocks = 1;
    filmAccumulateKernel<<<blocks, threads, 0, stream>>>(sum, comp, samples, width, cx, cy, cw, ch, nspp);
    return 1;
}

int launchFeatures(float4* accA, float4* accN, const float4* fa, const float4* fn, uint32_t width, uint32_t cx, uint32_t cy,
                   uint32_t cw, uint32_t ch, uint32_t nspp, int smCount, cudaStream_t stream)
{
    uint32_t npix = cw * ch;
    int threads = 256;
    int blocks = (int)((npix + threads - 1) / threads);
    if (blocks > smCount * 8) blocks = smCount * 8;
    if (blocks < 1) blocks = 1;
    featAccumulateKernel<<<blocks, threads, 0, stream>>>(accA, accN, fa, fn, width, cx, cy, cw, ch, nspp);
    return 1;
}

int launchRelmse(const float4* sum, const float* ref, uint32_t npix, double eps, double* out, int smCount, cudaStream_t stream)
{
    int threads = 256;
    int blocks = (int)((npix + threads - 1) / threads);
    if (blocks > smCount * 4) blocks = smCount * 4;
    if (blocks < 1) blocks = 1;
    relmseKernel<<<blocks, threads, 0, stream>>>(sum, ref, npix, eps, out);
    return 1;
}

} // namespace yg
