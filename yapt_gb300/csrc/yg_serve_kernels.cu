// Serving-loop kernels: the merged wavefront that carries the paths of several render
// requests (different scenes, image sizes, sample counts, depths; uni and NEE) in one set of
// queues, with a per-segment Kahan film pass.
#include <algorithm>

#include "yg_wave.cuh"

namespace yg
{

// ---------------------------------------------------------------- merged wavefront (serving)
// One wave holds the paths of several requests (each a segment of consecutive wave slots:
// whole sample planes of one request), possibly of different scenes, sizes, depths and of
// both unidirectional integrators. Every per-round quantity is read from device tables, so
// one captured launch sequence serves every round. A path computes exactly what it computes
// in a request of its own.

YG_DEV uint32_t segmentOf(const MultiTables& M, uint32_t nSeg, uint32_t s)
{
    uint32_t lo = 0, hi = nSeg; // segStart[lo] <= s < segStart[hi]
    while (hi - lo > 1)
    {
        uint32_t mid = (lo + hi) >> 1;
        if (M.segStart[mid] <= s) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void generateBody(const MultiTables& M, const WaveState& W, const RayQueue& Q)
{
    const uint32_t nSeg = *M.nSeg;
    const uint32_t total = M.segStart[nSeg];
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < total; s += gridDim.x * blockDim.x)
    {
        uint32_t k = segmentOf(M, nSeg, s);
        uint32_t req = M.segReq[k];
        uint32_t local = s - M.segStart[k];
        const SceneView& S = M.views[req];
        const LaunchParams& P = M.params[req];
        uint32_t sl, cx, cy;
        pixelOf(P, local, sl, cx, cy);
        uint32_t seed = (cy * P.width + cx) ^ (P.seed * 0x9E3779B9u);
        RandomSampler rs{S.sobol + (size_t)sl * kSobolDims, 2u, seed};
        Spectral sp;
        PathState ps;
        beginPath(S, P, cx, cy, rs, sp, ps);
        storePath(W, s, ps, rs, sp.hero, sl, false);
        M.req[s] = req;
        M.local[s] = local;
        Q.o[s] = mk4(ps.origin.x, ps.origin.y, ps.origin.z, __uint_as_float(s));
        Q.d[s] = mk4(ps.dir.x, ps.dir.y, ps.dir.z, 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *Q.count = total;
}
__global__ void __launch_bounds__(256) wfmGenerate(MultiTables M, WaveState W, RayQueue Q) { generateBody(M, W, Q); }

__device__ __forceinline__ void traceBody(const MultiTables& M, const RayQueue& Q, const HitQueue& H,
                                          unsigned long long* rayCtr)
{
    const uint32_t n = *Q.count;
    uint32_t rays = 0;
    TraversalCount tc{0, 0};
    traceGrid<false>(
        n,
        [&](TraceState& t, uint32_t i) {
            const float4 o = Q.o[i], d = Q.d[i];
            const SceneView& S = M.views[M.req[__float_as_uint(o.w)]];
            traceBegin(t, S, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), kRayMinT, __int_as_float(0x7f800000));
        },
        [&](const TraceState& t, uint32_t i) {
            H.a[i] = mk4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.instance));
            H.b[i] = t.found ? (t.h.prim | (t.h.front ? 0x80000000u : 0u)) : 0xffffffffu;
        },
        tc, rays);
    countRays(rayCtr, rays);
}
__global__ void __launch_bounds__(128) wfmTrace(MultiTables M, RayQueue Q, HitQueue H, unsigned long long* rayCtr)
{
    traceBody(M, Q, H, rayCtr);
}

__device__ __forceinline__ void classifyBody(const MultiTables& M, const RayQueue& Q, const HitQueue& H, uint8_t* keys,
                                             uint32_t* counts)
{
    const uint32_t n = *Q.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t r = 0; r < rounds; ++r)
    {
        uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + r * stride;
        bool active = i < n;
        uint32_t key = 0xffu;
        if (active)
        {
            const SceneView& S = M.views[M.req[__float_as_uint(Q.o[i].w)]];
            key = shadeClass(S, H.a[i], H.b[i]);
            keys[i] = (uint8_t)key;
        }
        for (uint32_t c = 0; c < (uint32_t)kShadeClasses; ++c)
        {
            uint32_t m = __ballot_sync(0xffffffffu, key == c);
            if (lane == 0 && m) atomicAdd(&counts[c], (uint32_t)__popc(m));
        }
    }
}

__global__ void __launch_bounds__(256) wfmClassify(MultiTables M, RayQueue Q, HitQueue H, uint8_t* keys, uint32_t* counts)
{
    classifyBody(M, Q, H, keys, counts);
}

__device__ __forceinline__ void shadeBody(const MultiTables& M, const WaveState& W, const RayQueue& Qin, const HitQueue& H,
                                          const RayQueue& Qout, const ShadowQueue& SQ)
{
    const uint32_t n = *Qin.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r)
    {
        uint32_t i = first + r * stride;
        bool active = i < n;
        bool alive = false;
        ShadowRequest sr;
        sr.valid = false;
        uint32_t slot = 0;
        PathState ps;
        if (active)
        {
            slot = __float_as_uint(Qin.o[i].w);
            const uint32_t req = M.req[slot];
            const SceneView& S = M.views[req];
            const LaunchParams& P = M.params[req];
            const Luts Lt = lutsOf(S);
            RandomSampler rs;
            Spectral sp;
            loadPath(W, slot, ps, rs, sp, S);
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
            if (P.integrator == 1) alive = shadeSegment<true>(S, P, Lt, sp, found, hit, ps, rs, sr, nullptr);
            else alive = shadeSegment<false>(S, P, Lt, sp, found, hit, ps, rs, sr, nullptr);
            alive = alive && ps.pathLength < P.maxDepth;
            storePath(W, slot, ps, rs, sp.hero, (uint32_t)(rs.point - S.sobol) / kSobolDims, ps.nVol != 0 || nVol0 != 0);
        }
        uint32_t k = warpAppend(Qout.count, alive);
        if (alive)
        {
            Qout.o[k] = mk4(ps.origin.x, ps.origin.y, ps.origin.z, __uint_as_float(slot));
            Qout.d[k] = mk4(ps.dir.x, ps.dir.y, ps.dir.z, 0.0f);
        }
        uint32_t j = warpAppend(SQ.count, sr.valid);
        if (sr.valid)
        {
            SQ.o[j] = mk4(sr.origin.x, sr.origin.y, sr.origin.z, __uint_as_float(slot));
            SQ.d[j] = mk4(sr.dir.x, sr.dir.y, sr.dir.z, sr.tmax);
            SQ.target[j] = make_uint2(sr.instance, sr.prim);
            SQ.contrib[j] = sr.contrib;
        }
    }
}
__global__ void __launch_bounds__(128, YG_SHADE_MIN_BLOCKS) wfmShade(MultiTables M, WaveState W, RayQueue Qin, HitQueue H, RayQueue Qout,
                                                ShadowQueue SQ)
{
    shadeBody(M, W, Qin, H, Qout, SQ);
}

__device__ __forceinline__ void shadowBody(const MultiTables& M, const WaveState& W, const ShadowQueue& SQ,
                                           unsigned long long* rayCtr)
{
    const uint32_t n = *SQ.count;
    uint32_t rays = 0;
    TraversalCount tc{0, 0};
    uint2 tg = make_uint2(0u, 0u);
    bool early = false;
    traceGridStop<false>(
        n,
        [&](TraceState& t, uint32_t i) {
            const float4 o = SQ.o[i], d = SQ.d[i];
            const SceneView& S = M.views[M.req[__float_as_uint(o.w)]];
            tg = SQ.target[i];
            early = shadowBegin(t, S, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), kRayMinT, d.w, tg.x, tg.y);
        },
        [&](const TraceState& t, uint32_t i) {
            if (shadowVisible(t.found, t.h, tg.x, tg.y))
            {
                const uint32_t s = __float_as_uint(SQ.o[i].w);
                W.tot[s] = W.tot[s] + SQ.contrib[i];
            }
        },
        [&](const TraceState& t) { return shadowStopped(t, early, tg.x, tg.y); }, tc, rays);
    countRays(rayCtr, rays);
}

__global__ void __launch_bounds__(128) wfmShadow(MultiTables M, WaveState W, ShadowQueue SQ, unsigned long long* rayCtr)
{
    shadowBody(M, W, SQ, rayCtr);
}

__device__ __forceinline__ void finalizeBody(const MultiTables& M, const WaveState& W)
{
    const uint32_t total = M.segStart[*M.nSeg];
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < total; s += gridDim.x * blockDim.x)
    {
        const uint32_t req = M.req[s];
        const SceneView& S = M.views[req];
        const LaunchParams& P = M.params[req];
        Spectral sp;
        spectralOf(S, W.dirHero[s].w, sp);
        FirstHit fh{mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f), 0.0f};
        writeSample(S, P, M.local[s], sp, W.tot[s], fh);
    }
}

__global__ void __launch_bounds__(256) wfmFinalize(MultiTables M, WaveState W) { finalizeBody(M, W); }

// Kahan film of every segment: the request's pixels, its planes of this round in order
__device__ __forceinline__ void filmBody(const MultiTables& M)
{
    const uint32_t nSeg = *M.nSeg;
    const uint32_t totalPix = M.segPixStart[nSeg];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < totalPix; q += gridDim.x * blockDim.x)
    {
        uint32_t lo = 0, hi = nSeg;
        while (hi - lo > 1)
        {
            uint32_t mid = (lo + hi) >> 1;
            if (M.segPixStart[mid] <= q) lo = mid;
            else hi = mid;
        }
        const uint32_t req = M.segReq[lo];
        const LaunchParams& P = M.params[req];
        const uint32_t npix = P.cropW * P.cropH;
        const uint32_t p = q - M.segPixStart[lo];
        const uint32_t nspp = (M.segStart[lo + 1] - M.segStart[lo]) / npix;
        const uint32_t x = P.cropX + p % P.cropW, y = P.cropY + p / P.cropW;
        const size_t fi = (size_t)y * P.width + x;
        float4* sum = M.filmSum[req];
        float4* comp = M.filmComp[req];
        float4 sacc = sum[fi], c = comp[fi];
        for (uint32_t k = 0; k < nspp; ++k)
        {
            float4 v = P.sampleXYZ[(size_t)k * npix + p];
            float4 yv = v - c;
            float4 t = sacc + yv;
            c = (t - sacc) - yv;
            sacc = t;
        }
        sum[fi] = sacc;
        comp[fi] = c;
    }
}
__global__ void __launch_bounds__(256) wfmFilm(MultiTables M) { filmBody(M); }

// The queues of a merged round, carved from the round's arena
struct RoundQueues
{
    WaveState W;
    RayQueue QA, QB, QS;
    HitQueue H, HS;
    ShadowQueue SQ;
    uint8_t* keys;
    uint32_t* classCounts;
};

// One merged round as one persistent cooperative kernel: every stage of the multi-kernel round
// (generate; per bounce trace, classify, regroup, shade, shadow; finalize; film), each a
// grid-stride loop over the stage's queue, separated by grid barriers instead of launches. The
// paths compute what they compute in the multi-kernel round. A barrier that does not complete
// within `pollLimit` polls stops every block (the round reports the time-out through the
// barrier's error word) instead of hanging.
__global__ void __launch_bounds__(128, 4) wfmRound(MultiTables M, RoundQueues R, uint32_t maxDepth, GridBarrier* bar,
                                                   uint32_t pollLimit, unsigned long long* rayCtr)
{
    generateBody(M, R.W, R.QA);
    if (!gridSync(bar, pollLimit)) return;
    RayQueue cur = R.QA, nxt = R.QB;
    for (uint32_t b = 0; b < maxDepth; ++b)
    {
        // the same count in every block (written before the last barrier): no path left
        if (*(volatile uint32_t*)cur.count == 0) break;
        // nothing reads these counters between here and the next barrier
        if (blockIdx.x == 0 && threadIdx.x == 0)
        {
            *nxt.count = 0;
            *R.SQ.count = 0;
            for (int c = 0; c < 2 * kShadeClasses; ++c) R.classCounts[c] = 0;
        }
        traceBody(M, cur, R.H, rayCtr);
        if (!gridSync(bar, pollLimit)) return;
        classifyBody(M, cur, R.H, R.keys, R.classCounts);
        if (!gridSync(bar, pollLimit)) return;
        regroupBody<kShadeClasses>(cur, R.H, R.keys, R.classCounts, R.classCounts + kShadeClasses, R.QS, R.HS);
        if (!gridSync(bar, pollLimit)) return;
        shadeBody(M, R.W, R.QS, R.HS, nxt, R.SQ);
        if (!gridSync(bar, pollLimit)) return;
        shadowBody(M, R.W, R.SQ, rayCtr);
        if (!gridSync(bar, pollLimit)) return;
        RayQueue t = cur;
        cur = nxt;
        nxt = t;
    }
    finalizeBody(M, R.W);
    if (!gridSync(bar, pollLimit)) return;
    filmBody(M);
}

__global__ void gridBarrierInit(GridBarrier* bar, uint32_t expected)
{
    bar->count = 0;
    bar->gen = 0;
    bar->error = 0;
    bar->expected = expected;
}

// Every block passes the barrier three times; with `missing` blocks that never arrive the first
// barrier runs out of polls and every block returns.
__global__ void __launch_bounds__(128) gridBarrierProbe(GridBarrier* bar, uint32_t pollLimit, uint32_t* passes)
{
    for (int k = 0; k < 3; ++k)
    {
        if (!gridSync(bar, pollLimit)) return;
        if (threadIdx.x == 0) atomicAdd(passes, 1u);
    }
}

int gridBarrierCheck(GridBarrier* bar, uint32_t* passes, uint32_t missing, uint32_t pollLimit, int smCount,
                     cudaStream_t stream, uint32_t* blocks)
{
    int perSm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, gridBarrierProbe, 128, 0);
    if (e != cudaSuccess) return (int)e;
    const uint32_t grid = (uint32_t)std::max(1, std::min(perSm, 2) * smCount);
    *blocks = grid;
    gridBarrierInit<<<1, 1, 0, stream>>>(bar, grid + missing);
    void* args[] = {&bar, &pollLimit, &passes};
    return (int)cudaLaunchCooperativeKernel((const void*)gridBarrierProbe, dim3(grid), dim3(128), args, 0, stream);
}

size_t multiWaveBytes(uint32_t capacity)
{
    return (size_t)capacity * (wavefrontBytesPerSlot() + 8) + (64u << 10);
}

static RoundQueues carveRound(MultiTables& M, void* arena, uint32_t capacity)
{
    char* p = static_cast<char*>(arena);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    const size_t C = capacity;
    RoundQueues R;
    WaveState& W = R.W;
    W.capacity = capacity;
    W.thr = (float4*)take(C * 16);
    W.tot = (float4*)take(C * 16);
    W.orgPdf = (float4*)take(C * 16);
    W.dirHero = (float4*)take(C * 16);
    W.misc = (uint4*)take(C * 16);
    W.volIOR = (float4*)take(C * 16);
    W.volMat = (uint4*)take(C * 16);
    W.volAbs = (float4*)take(C * 64);
    W.fhAlb = (float4*)take(C * 16);
    W.fhNrm = (float4*)take(C * 16);
    M.req = (uint32_t*)take(C * 4);
    M.local = (uint32_t*)take(C * 4);
    uint32_t* counters = (uint32_t*)take(256);
    R.QA = RayQueue{(float4*)take(C * 16), (float4*)take(C * 16), counters + 0};
    R.QB = RayQueue{(float4*)take(C * 16), (float4*)take(C * 16), counters + 1};
    R.H = HitQueue{(float4*)take(C * 16), (uint32_t*)take(C * 4)};
    R.SQ = ShadowQueue{(float4*)take(C * 16), (float4*)take(C * 16), (uint2*)take(C * 8), (float4*)take(C * 16),
                       counters + 2};
    R.QS = RayQueue{(float4*)take(C * 16), (float4*)take(C * 16), counters + 3};
    R.HS = HitQueue{(float4*)take(C * 16), (uint32_t*)take(C * 4)};
    R.keys = (uint8_t*)take(C);
    R.classCounts = counters + 8;
    return R;
}

int launchWavefrontMulti(const MultiTables& M0, void* arena, uint32_t capacity, uint32_t maxDepth,
                         unsigned long long* rayCounter, int smCount, cudaStream_t stream)
{
    MultiTables M = M0;
    RoundQueues R = carveRound(M, arena, capacity);
    WaveState& W = R.W;
    RayQueue& QA = R.QA;
    RayQueue& QB = R.QB;
    RayQueue& QS = R.QS;
    HitQueue& H = R.H;
    HitQueue& HS = R.HS;
    ShadowQueue& SQ = R.SQ;
    uint8_t* keys = R.keys;
    uint32_t* classCounts = R.classCounts;
    const size_t C = capacity;
    const int traceBlocks = smCount * 16, shadeBlocks = smCount * 8;
    int gblocks = (int)std::min<uint64_t>((C + 255) / 256, (uint64_t)smCount * 8);
    int launches = 0;
    wfmGenerate<<<gblocks, 256, 0, stream>>>(M, W, QA);
    ++launches;
    RayQueue* cur = &QA;
    RayQueue* nxt = &QB;
    for (uint32_t b = 0; b < maxDepth; ++b)
    {
        wfmTrace<<<traceBlocks, 128, 0, stream>>>(M, *cur, H, rayCounter);
        cudaMemsetAsync(nxt->count, 0, 4, stream);
        cudaMemsetAsync(SQ.count, 0, 4, stream);
        cudaMemsetAsync(classCounts, 0, 2 * kShadeClasses * 4, stream);
        wfmClassify<<<smCount * 4, 256, 0, stream>>>(M, *cur, H, keys, classCounts);
        wfRegroup<kShadeClasses><<<smCount * 4, 256, 0, stream>>>(*cur, H, keys, classCounts, classCounts + kShadeClasses, QS, HS);
        wfmShade<<<shadeBlocks, 128, 0, stream>>>(M, W, QS, HS, *nxt, SQ);
        wfmShadow<<<traceBlocks, 128, 0, stream>>>(M, W, SQ, rayCounter);
        launches += 5;
        RayQueue* t = cur;
        cur = nxt;
        nxt = t;
    }
    wfmFinalize<<<gblocks, 256, 0, stream>>>(M, W);
    wfmFilm<<<gblocks, 256, 0, stream>>>(M);
    launches += 2;
    return launches;
}

int launchWavefrontMultiPersistent(const MultiTables& M0, void* arena, uint32_t capacity, uint32_t maxDepth,
                                   unsigned long long* rayCounter, int smCount, cudaStream_t stream, GridBarrier* barrier,
                                   uint32_t pollLimit)
{
    MultiTables M = M0;
    RoundQueues R = carveRound(M, arena, capacity);
    int perSm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, wfmRound, 128, 0);
    if (e != cudaSuccess) return -(int)e;
    if (perSm < 1) return -(int)cudaErrorCooperativeLaunchTooLarge;
    const uint32_t grid = (uint32_t)(perSm * smCount);
    gridBarrierInit<<<1, 1, 0, stream>>>(barrier, grid);
    void* args[] = {&M, &R, &maxDepth, &barrier, &pollLimit, &rayCounter};
    e = cudaLaunchCooperativeKernel((const void*)wfmRound, dim3(grid), dim3(128), args, 0, stream);
    if (e != cudaSuccess) return -(int)e;
    return 2;
}

} // namespace yg
