// Device-built 8-wide compressed BVH (replaces YAPT's DXR BLAS/TLAS builds,
// AccelerationStructureHelper.cpp:96-213). Every (instance, submesh) is flattened into one
// world-space triangle set, so a ray needs one traversal and closest-hit keys stay
// (instance, primitive).
//
// Pipeline, all on the device:
//  1. world-space triangles and their bounds (one thread per primitive);
//  2. 63-bit Morton codes of the bound centres, stable LSD radix sort (4-bit digits);
//  3. binary tree by locally-ordered clustering (PLOC, Meister and Bittner 2018): every
//     cluster finds the neighbour within a window of the Morton order whose union box has
//     the smallest surface area, mutual nearest pairs merge, the survivors are compacted,
//     until one cluster is left;
//  4. bottom-up surface-area-heuristic pass (one thread per leaf walks up; the second
//     thread to reach a node continues, the first stops) deciding which subtrees of at
//     most kMaxLeafTris triangles become leaves;
//  5. top-down collapse into 8-wide nodes, level by level: a wide node takes the children
//     of its binary node and repeatedly opens the largest internal child until it has 8;
//     children are placed in slots by octant so that the slot order XOR the ray's
//     direction octant approximates near-to-far; child boxes are quantised to 8 bits
//     relative to the node box with one quantum of outward padding.
// Node layout (80 B) and traversal: yg_trace.cuh. Deterministic: every allocation order
// comes from prefix sums, never from atomics.
#include "yg_kernels.h"
#include "yg_vec.cuh"

#include <cstring>
#include <string>
#include <vector>

namespace yg
{
namespace
{

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kSortThreads = 256;
constexpr int kSortBatches = 8;
constexpr int kSortTile = kSortThreads * kSortBatches;
#ifndef YG_BVH_PLOC_RADIUS
#define YG_BVH_PLOC_RADIUS 32
#endif
#ifndef YG_BVH_COST_TRI
#define YG_BVH_COST_TRI 3.0f
#endif
constexpr int kPlocRadius = YG_BVH_PLOC_RADIUS;
constexpr int kPlocThreads = 256;
constexpr float kCostNode = 1.0f;            // SAH cost of a wide-node visit relative to
constexpr float kCostTri = YG_BVH_COST_TRI;  // one triangle test
constexpr int kMaxPlocIterations = 4096;

__device__ __forceinline__ uint32_t orderedBits(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fromOrdered(uint32_t b)
{
    return __uint_as_float((b & 0x80000000u) ? (b & 0x7fffffffu) : ~b);
}

__device__ __forceinline__ float halfArea(float4 lo, float4 hi)
{
    float dx = fmaxf(hi.x - lo.x, 0.f), dy = fmaxf(hi.y - lo.y, 0.f), dz = fmaxf(hi.z - lo.z, 0.f);
    return dx * dy + dy * dz + dz * dx;
}

// ------------------------------------------------------------------ 1. triangles
__global__ void worldTriangles(const GpuInstance* __restrict__ inst, const uint32_t* __restrict__ instStart,
                               uint32_t nInst, const float* __restrict__ pos, const uint32_t* __restrict__ idx,
                               uint32_t nPrims, float4* __restrict__ tris, float4* __restrict__ lo,
                               float4* __restrict__ hi, uint32_t* __restrict__ bounds, const float2* __restrict__ uvs,
                               const GpuAlphaSource* __restrict__ alpha, float4* __restrict__ cutouts)
{
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    float blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (g < nPrims)
    {
        // instance of primitive g: last instance whose first primitive is <= g
        uint32_t a = 0, b = nInst;
        while (b - a > 1)
        {
            uint32_t m = (a + b) >> 1;
            if (instStart[m] <= g) a = m;
            else b = m;
        }
        const GpuInstance& I = inst[a];
        uint32_t p = g - instStart[a];
        float3 w[3];
        uint32_t vi[3];
        for (int k = 0; k < 3; ++k)
        {
            vi[k] = idx[I.firstIndex + 3 * p + k] + I.vertexBase;
            w[k] = xformPoint(I.o2w, mk3(pos[3 * vi[k]], pos[3 * vi[k] + 1], pos[3 * vi[k] + 2]));
        }
        // the cutout record of an alpha-tested triangle, behind the reordered triangles; the
        // triangle refers to it by its float4 offset from the start of the triangle array
        uint32_t cut = 0;
        if (cutouts && I.alphaSource)
        {
            const GpuAlphaSource A = alpha[I.alphaSource - 1];
            const float2 t0 = uvs[vi[0]], t1 = uvs[vi[1]], t2 = uvs[vi[2]];
            const uint64_t tp = reinterpret_cast<uint64_t>(A.texels);
            float4* r = cutouts + 3 * (size_t)g;
            r[0] = make_float4(t0.x, t0.y, t1.x, t1.y);
            r[1] = make_float4(t2.x, t2.y, A.su, A.sv);
            r[2] = make_float4(__uint_as_float((uint32_t)tp), __uint_as_float((uint32_t)(tp >> 32)), __uint_as_float(A.size),
                               A.cutoff);
            cut = 3 * nPrims + 3 * g;
        }
        float3 e1 = mk3(w[1].x - w[0].x, w[1].y - w[0].y, w[1].z - w[0].z);
        float3 e2 = mk3(w[2].x - w[0].x, w[2].y - w[0].y, w[2].z - w[0].z);
        tris[3 * (size_t)g] = make_float4(w[0].x, w[0].y, w[0].z, __uint_as_float(a));
        tris[3 * (size_t)g + 1] = make_float4(e1.x, e1.y, e1.z, __uint_as_float(p));
        tris[3 * (size_t)g + 2] = make_float4(e2.x, e2.y, e2.z, __uint_as_float(cut));
        for (int k = 0; k < 3; ++k)
        {
            const float c[3] = {w[k].x, w[k].y, w[k].z};
            for (int ax = 0; ax < 3; ++ax)
            {
                blo[ax] = fminf(blo[ax], c[ax]);
                bhi[ax] = fmaxf(bhi[ax], c[ax]);
            }
        }
        // a triangle with a non-finite vertex is never hit; give it a point box at the origin
        bool finite = true;
        for (int ax = 0; ax < 3; ++ax) finite = finite && isfinite(blo[ax]) && isfinite(bhi[ax]);
        if (!finite)
            for (int ax = 0; ax < 3; ++ax) blo[ax] = bhi[ax] = 0.0f;
        lo[g] = make_float4(blo[0], blo[1], blo[2], 0.f);
        hi[g] = make_float4(bhi[0], bhi[1], bhi[2], 0.f);
    }
    // world bounds [0..2] min, [3..5] max, and bound-centre bounds [6..8] min, [9..11] max
    __shared__ uint32_t red[12];
    if (threadIdx.x < 12) red[threadIdx.x] = threadIdx.x % 6 < 3 ? 0xffffffffu : 0u;
    __syncthreads();
    if (g < nPrims)
        for (int ax = 0; ax < 3; ++ax)
        {
            float c = (blo[ax] + bhi[ax]) * 0.5f;
            atomicMin(&red[ax], orderedBits(blo[ax]));
            atomicMax(&red[3 + ax], orderedBits(bhi[ax]));
            atomicMin(&red[6 + ax], orderedBits(c));
            atomicMax(&red[9 + ax], orderedBits(c));
        }
    __syncthreads();
    if (threadIdx.x < 12)
    {
        if (threadIdx.x % 6 < 3) atomicMin(&bounds[threadIdx.x], red[threadIdx.x]);
        else atomicMax(&bounds[threadIdx.x], red[threadIdx.x]);
    }
}

__device__ __forceinline__ uint64_t spread21(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void mortonCodes(const float4* __restrict__ lo, const float4* __restrict__ hi, const uint32_t* bounds,
                            uint32_t n, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float cl[3], ch[3];
    for (int ax = 0; ax < 3; ++ax)
    {
        cl[ax] = fromOrdered(bounds[6 + ax]);
        ch[ax] = fromOrdered(bounds[9 + ax]);
    }
    float4 a = lo[i], b = hi[i];
    const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
    uint64_t code = 0;
    for (int ax = 0; ax < 3; ++ax)
    {
        float ext = ch[ax] - cl[ax];
        float t = ext > 0.f ? (c[ax] - cl[ax]) / ext : 0.f;
        uint32_t q = (uint32_t)fminf(fmaxf(t * 2097152.0f, 0.0f), 2097151.0f);
        code |= spread21(q) << ax;
    }
    keys[i] = code;
    vals[i] = i;
}

// ------------------------------------------------------------------ exclusive scan (uint64)
__device__ __forceinline__ uint64_t warpInclusive(uint64_t v)
{
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// exclusive scan of each tile of kScanTile items; tile totals to sums
__global__ void __launch_bounds__(kScanThreads) scanTiles(const uint64_t* __restrict__ in, uint64_t* __restrict__ out,
                                                           uint64_t* __restrict__ sums, uint32_t n)
{
    __shared__ uint64_t warpTot[kScanThreads / 32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint64_t v[kScanItems];
    uint64_t local = 0;
    for (int k = 0; k < kScanItems; ++k)
    {
        v[k] = base + k < n ? in[base + k] : 0;
        local += v[k];
    }
    uint64_t inc = warpInclusive(local);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) warpTot[warp] = inc;
    __syncthreads();
    uint64_t warpOff = 0;
    for (int w = 0; w < warp; ++w) warpOff += warpTot[w];
    uint64_t run = warpOff + inc - local;
    for (int k = 0; k < kScanItems; ++k)
    {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = warpOff + inc;
}

__global__ void scanAddOffsets(uint64_t* __restrict__ out, const uint64_t* __restrict__ offs, uint32_t n)
{
    size_t i = (size_t)blockIdx.x * kScanTile + threadIdx.x;
    for (int k = 0; k < kScanItems; ++k, i += kScanThreads)
        if (i < n) out[i] += offs[blockIdx.x];
}

// ------------------------------------------------------------------ stable radix sort
// digit histograms per tile, digit-major: hist[d * tiles + tile]
__global__ void __launch_bounds__(kSortThreads) sortHistogram(const uint64_t* __restrict__ keys, uint32_t n, int shift,
                                                               uint64_t* __restrict__ hist, uint32_t tiles)
{
    __shared__ uint32_t h[16];
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
    for (int j = 0; j < kSortBatches; ++j)
    {
        size_t i = base + (size_t)j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 15u], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 16) hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) sortScatter(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                                             uint32_t n, int shift, const uint64_t* __restrict__ offs,
                                                             uint32_t tiles, uint64_t* __restrict__ keysOut,
                                                             uint32_t* __restrict__ valsOut)
{
    constexpr int W = kSortThreads / 32;
    __shared__ uint32_t cnt[W][16];
    __shared__ uint32_t running[16];
    __shared__ uint32_t tileBase[16];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 16)
    {
        running[threadIdx.x] = 0;
        tileBase[threadIdx.x] = (uint32_t)offs[(size_t)threadIdx.x * tiles + blockIdx.x];
    }
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
    const uint32_t below = (1u << lane) - 1u;
    for (int j = 0; j < kSortBatches; ++j)
    {
        size_t i = base + (size_t)j * kSortThreads + threadIdx.x;
        bool valid = i < n;
        uint64_t k = valid ? keys[i] : 0;
        uint32_t v = valid ? vals[i] : 0;
        uint32_t d = valid ? (uint32_t)((k >> shift) & 15u) : 16u;
        uint32_t myRank = 0;
        for (uint32_t dv = 0; dv < 16; ++dv)
        {
            uint32_t m = __ballot_sync(0xffffffffu, d == dv);
            if (d == dv) myRank = __popc(m & below);
            if (lane == (int)dv) cnt[warp][dv] = __popc(m);
        }
        __syncthreads();
        if (valid)
        {
            uint32_t r = running[d] + myRank;
            for (int w = 0; w < warp; ++w) r += cnt[w][d];
            keysOut[tileBase[d] + r] = k;
            valsOut[tileBase[d] + r] = v;
        }
        __syncthreads();
        if (threadIdx.x < 16)
        {
            uint32_t t = 0;
            for (int w = 0; w < W; ++w) t += cnt[w][threadIdx.x];
            running[threadIdx.x] += t;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ PLOC
struct Clusters
{
    float4* lo; // .w: node id (int bits)
    float4* hi;
};

__global__ void initLeaves(const uint32_t* __restrict__ order, const float4* __restrict__ plo, const float4* __restrict__ phi,
                           uint32_t n, Clusters C, float4* __restrict__ nlo, float4* __restrict__ nhi)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = order[i];
    float4 a = plo[p], b = phi[p];
    // leaf node i of the binary tree: children (-1, primitive)
    nlo[i] = make_float4(a.x, a.y, a.z, __int_as_float(-1));
    nhi[i] = make_float4(b.x, b.y, b.z, __int_as_float((int)p));
    C.lo[i] = make_float4(a.x, a.y, a.z, __int_as_float((int)i));
    C.hi[i] = make_float4(b.x, b.y, b.z, 0.f);
}

__global__ void __launch_bounds__(kPlocThreads) plocNearest(Clusters C, uint32_t n, int32_t* __restrict__ nn)
{
    __shared__ float4 slo[kPlocThreads + 2 * kPlocRadius], shi[kPlocThreads + 2 * kPlocRadius];
    const int first = (int)(blockIdx.x * kPlocThreads) - kPlocRadius;
    for (int t = threadIdx.x; t < kPlocThreads + 2 * kPlocRadius; t += kPlocThreads)
    {
        int j = first + t;
        if (j >= 0 && j < (int)n)
        {
            slo[t] = C.lo[j];
            shi[t] = C.hi[j];
        }
    }
    __syncthreads();
    const int i = (int)(blockIdx.x * kPlocThreads + threadIdx.x);
    if (i >= (int)n) return;
    const float4 a = slo[threadIdx.x + kPlocRadius], b = shi[threadIdx.x + kPlocRadius];
    float best = INFINITY;
    int bestJ = -1;
    const int j0 = max(0, i - kPlocRadius), j1 = min((int)n - 1, i + kPlocRadius);
    for (int j = j0; j <= j1; ++j)
    {
        if (j == i) continue;
        const float4 c = slo[j - first], d = shi[j - first];
        float4 ul = make_float4(fminf(a.x, c.x), fminf(a.y, c.y), fminf(a.z, c.z), 0.f);
        float4 uh = make_float4(fmaxf(b.x, d.x), fmaxf(b.y, d.y), fmaxf(b.z, d.z), 0.f);
        float s = halfArea(ul, uh);
        if (s < best)
        {
            best = s;
            bestJ = j;
        }
    }
    nn[i] = bestJ;
}

// low 32 bits: the cluster survives; high 32 bits: it becomes a new node
__global__ void plocFlags(const int32_t* __restrict__ nn, uint32_t n, uint64_t* __restrict__ flags)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = nn[i];
    bool mutual = j >= 0 && nn[j] == (int)i;
    bool keep = !mutual || (int)i < j;
    bool merge = mutual && (int)i < j;
    flags[i] = (keep ? 1ull : 0ull) | ((merge ? 1ull : 0ull) << 32);
}

__global__ void plocCompact(Clusters C, const int32_t* __restrict__ nn, const uint64_t* __restrict__ flags,
                            const uint64_t* __restrict__ scan, uint32_t n, uint32_t nodeBase, Clusters out,
                            float4* __restrict__ nlo, float4* __restrict__ nhi, int32_t* __restrict__ parent)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t f = flags[i];
    if (!(f & 0xffffffffull)) return;
    uint32_t dst = (uint32_t)(scan[i] & 0xffffffffull);
    float4 a = C.lo[i], b = C.hi[i];
    if (f >> 32)
    {
        int j = nn[i];
        float4 c = C.lo[j], d = C.hi[j];
        uint32_t node = nodeBase + (uint32_t)(scan[i] >> 32);
        int ca = __float_as_int(a.w), cb = __float_as_int(c.w);
        float4 ul = make_float4(fminf(a.x, c.x), fminf(a.y, c.y), fminf(a.z, c.z), __int_as_float(ca));
        float4 uh = make_float4(fmaxf(b.x, d.x), fmaxf(b.y, d.y), fmaxf(b.z, d.z), __int_as_float(cb));
        nlo[node] = ul;
        nhi[node] = uh;
        parent[ca] = (int)node;
        parent[cb] = (int)node;
        out.lo[dst] = make_float4(ul.x, ul.y, ul.z, __int_as_float((int)node));
        out.hi[dst] = make_float4(uh.x, uh.y, uh.z, 0.f);
    }
    else
    {
        out.lo[dst] = a;
        out.hi[dst] = b;
    }
}

// ------------------------------------------------------------------ 4. bottom-up SAH
struct TreeCost
{
    uint32_t* count;   // primitives under the node
    float* cost;       // SAH cost (area units)
    uint8_t* leaf;     // node becomes one wide-node leaf slot
    uint32_t* visits;  // arrival counters
};

__global__ void bottomUp(const float4* __restrict__ nlo, const float4* __restrict__ nhi, const int32_t* __restrict__ parent,
                         uint32_t nLeaves, TreeCost T)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nLeaves) return;
    int node = (int)i;
    {
        float a = halfArea(nlo[node], nhi[node]);
        T.count[node] = 1;
        T.cost[node] = a * kCostTri;
        T.leaf[node] = 1;
    }
    while (true)
    {
        int p = parent[node];
        if (p < 0) return;
        __threadfence();
        if (atomicAdd(&T.visits[p], 1u) == 0) return; // the sibling subtree is not finished
        int l = __float_as_int(nlo[p].w), r = __float_as_int(nhi[p].w);
        uint32_t cl = __ldcg(T.count + l), cr = __ldcg(T.count + r);
        float kl = __ldcg(T.cost + l), kr = __ldcg(T.cost + r);
        float a = halfArea(nlo[p], nhi[p]);
        uint32_t c = cl + cr;
        float split = a * kCostNode + kl + kr;
        float asLeaf = a * kCostTri * (float)c;
        bool leaf = c <= (uint32_t)kMaxLeafTris && asLeaf <= split;
        T.count[p] = c;
        T.cost[p] = leaf ? asLeaf : split;
        T.leaf[p] = leaf ? 1 : 0;
        node = p;
    }
}

// ------------------------------------------------------------------ 5. collapse to 8-wide
struct Plan
{
    int32_t child[8]; // binary nodes of the wide node's children (-1: none)
};

__device__ __forceinline__ bool isOpenable(const TreeCost& T, const float4* nlo, int b)
{
    return !T.leaf[b] && __float_as_int(nlo[b].w) >= 0;
}

__global__ void collapsePlan(const int32_t* __restrict__ items, uint32_t nItems, const float4* __restrict__ nlo,
                             const float4* __restrict__ nhi, TreeCost T, Plan* __restrict__ plans,
                             uint64_t* __restrict__ counts)
{
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nItems) return;
    int b = items[w];
    int ch[8];
    int k = 0;
    if (T.leaf[b] || __float_as_int(nlo[b].w) < 0)
    {
        ch[k++] = b; // a wide node holding one leaf (a tree of at most kMaxLeafTris triangles)
    }
    else
    {
        ch[k++] = __float_as_int(nlo[b].w);
        ch[k++] = __float_as_int(nhi[b].w);
        while (k < 8)
        {
            int best = -1;
            float bestA = -1.f;
            for (int c = 0; c < k; ++c)
                if (isOpenable(T, nlo, ch[c]))
                {
                    float a = halfArea(nlo[ch[c]], nhi[ch[c]]);
                    if (a > bestA)
                    {
                        bestA = a;
                        best = c;
                    }
                }
            if (best < 0) break;
            int o = ch[best];
            ch[best] = __float_as_int(nlo[o].w);
            ch[k++] = __float_as_int(nhi[o].w);
        }
    }
    uint32_t nInternal = 0, nTris = 0;
    Plan P;
    for (int c = 0; c < 8; ++c)
    {
        P.child[c] = c < k ? ch[c] : -1;
        if (c < k)
        {
            if (T.leaf[ch[c]] || __float_as_int(nlo[ch[c]].w) < 0) nTris += T.count[ch[c]];
            else ++nInternal;
        }
    }
    plans[w] = P;
    counts[w] = (uint64_t)nInternal | ((uint64_t)nTris << 32);
}

__device__ __forceinline__ uint32_t quantExp(float ext)
{
    // smallest power of two 2^e with 2^e >= ext / 250 (biased by 127), clamped to normal floats
    float x = __fdiv_ru(ext, 250.0f);
    uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xffu);
    if (b & 0x7fffffu) ++e;
    return (uint32_t)min(max(e, 1), 253);
}

__global__ void collapseEmit(const int32_t* __restrict__ items, const uint32_t* __restrict__ itemWide, uint32_t nItems,
                             const Plan* __restrict__ plans, const uint64_t* __restrict__ scan, uint32_t wideNext,
                             uint32_t triNext, const float4* __restrict__ nlo, const float4* __restrict__ nhi, TreeCost T,
                             const float4* __restrict__ trisIn, float4* __restrict__ trisOut, float4* __restrict__ wide,
                             int32_t* __restrict__ nextItems, uint32_t* __restrict__ nextWide)
{
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nItems) return;
    const int b = items[w];
    const Plan P = plans[w];
    const uint32_t childBase = wideNext + (uint32_t)(scan[w] & 0xffffffffull);
    const uint32_t triBase = triNext + (uint32_t)(scan[w] >> 32);
    const uint32_t nextBase = (uint32_t)(scan[w] & 0xffffffffull);
    // node box and quantisation grid
    const float4 L = nlo[b], H = nhi[b];
    const float lo[3] = {L.x, L.y, L.z}, hi[3] = {H.x, H.y, H.z};
    float p[3], scale[3], inv[3];
    uint32_t e[3];
    for (int a = 0; a < 3; ++a)
    {
        float ext = __fsub_ru(hi[a], lo[a]);
        float mag = fmaxf(fabsf(lo[a]), fabsf(hi[a]));
        ext = fmaxf(fmaxf(ext, mag * 9.5367431640625e-7f), 1e-30f); // flat boxes get a thickness
        e[a] = quantExp(ext);
        scale[a] = __uint_as_float(e[a] << 23);
        inv[a] = __uint_as_float((254u - e[a]) << 23); // exact 1 / scale
        p[a] = __fsub_rd(lo[a], scale[a]);
    }
    // slot assignment: child centre direction against the octant of each slot, greedy
    const float pc[3] = {(lo[0] + hi[0]) * 0.5f, (lo[1] + hi[1]) * 0.5f, (lo[2] + hi[2]) * 0.5f};
    int slotOf[8];
    int childInSlot[8];
    for (int s = 0; s < 8; ++s) childInSlot[s] = -1;
    for (int c = 0; c < 8; ++c) slotOf[c] = -1;
    for (int round = 0; round < 8; ++round)
    {
        float best = -INFINITY;
        int bc = -1, bs = -1;
        for (int c = 0; c < 8; ++c)
        {
            if (P.child[c] < 0 || slotOf[c] >= 0) continue;
            float4 cl = nlo[P.child[c]], chh = nhi[P.child[c]];
            float d[3] = {(cl.x + chh.x) * 0.5f - pc[0], (cl.y + chh.y) * 0.5f - pc[1], (cl.z + chh.z) * 0.5f - pc[2]};
            for (int s = 0; s < 8; ++s)
            {
                if (childInSlot[s] >= 0) continue;
                float score = ((s & 1) ? d[0] : -d[0]) + ((s & 2) ? d[1] : -d[1]) + ((s & 4) ? d[2] : -d[2]);
                if (score > best)
                {
                    best = score;
                    bc = c;
                    bs = s;
                }
            }
        }
        if (bc < 0) break;
        slotOf[bc] = bs;
        childInSlot[bs] = bc;
    }
    uint32_t imask = 0, meta[8], qlo[3][8], qhi[3][8];
    uint32_t internalRank = 0, triOff = 0;
    for (int s = 0; s < 8; ++s)
    {
        meta[s] = 0;
        for (int a = 0; a < 3; ++a)
        {
            qlo[a][s] = 255;
            qhi[a][s] = 0;
        }
        int c = childInSlot[s];
        if (c < 0) continue;
        int cb = P.child[c];
        float4 cl = nlo[cb], chh = nhi[cb];
        const float clo[3] = {cl.x, cl.y, cl.z}, chi[3] = {chh.x, chh.y, chh.z};
        for (int a = 0; a < 3; ++a)
        {
            int ql = (int)floorf(__fmul_rd(__fsub_rd(clo[a], p[a]), inv[a])) - 1;
            int qh = (int)ceilf(__fmul_ru(__fsub_ru(chi[a], p[a]), inv[a])) + 1;
            qlo[a][s] = (uint32_t)min(max(ql, 0), 255);
            qhi[a][s] = (uint32_t)min(max(qh, 0), 255);
        }
        const bool leaf = T.leaf[cb] || __float_as_int(cl.w) < 0;
        if (!leaf)
        {
            imask |= 1u << s;
            meta[s] = 1;
            nextItems[nextBase + internalRank] = cb;
            nextWide[nextBase + internalRank] = childBase + internalRank;
            ++internalRank;
        }
        else
        {
            // the leaf's primitives, left to right
            int stack[8];
            int sp = 0;
            stack[sp++] = cb;
            uint32_t cnt = 0;
            while (sp > 0)
            {
                int x = stack[--sp];
                int l = __float_as_int(nlo[x].w);
                if (l < 0)
                {
                    uint32_t prim = (uint32_t)__float_as_int(nhi[x].w);
                    size_t dst = 3 * (size_t)(triBase + triOff + cnt);
                    trisOut[dst] = trisIn[3 * (size_t)prim];
                    trisOut[dst + 1] = trisIn[3 * (size_t)prim + 1];
                    trisOut[dst + 2] = trisIn[3 * (size_t)prim + 2];
                    ++cnt;
                }
                else if (sp + 2 <= 8)
                {
                    stack[sp++] = __float_as_int(nhi[x].w);
                    stack[sp++] = l;
                }
            }
            meta[s] = (cnt << 5) | triOff;
            triOff += cnt;
        }
    }
    auto pack4 = [](const uint32_t* v) { return v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24); };
    float4* o = wide + 5 * (size_t)itemWide[w];
    o[0] = make_float4(p[0], p[1], p[2], __uint_as_float(e[0] | (e[1] << 8) | (e[2] << 16) | (imask << 24)));
    o[1] = make_float4(__uint_as_float(childBase), __uint_as_float(triBase), __uint_as_float(pack4(meta)),
                       __uint_as_float(pack4(meta + 4)));
    o[2] = make_float4(__uint_as_float(pack4(qlo[0])), __uint_as_float(pack4(qlo[0] + 4)), __uint_as_float(pack4(qlo[1])),
                       __uint_as_float(pack4(qlo[1] + 4)));
    o[3] = make_float4(__uint_as_float(pack4(qlo[2])), __uint_as_float(pack4(qlo[2] + 4)), __uint_as_float(pack4(qhi[0])),
                       __uint_as_float(pack4(qhi[0] + 4)));
    o[4] = make_float4(__uint_as_float(pack4(qhi[1])), __uint_as_float(pack4(qhi[1] + 4)), __uint_as_float(pack4(qhi[2])),
                       __uint_as_float(pack4(qhi[2] + 4)));
}

// ------------------------------------------------------------------ host helpers
struct Pool
{
    std::vector<void*> ptrs;
    ~Pool()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    T* get(size_t count, cudaError_t& err)
    {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

unsigned blocksFor(size_t n, unsigned threads)
{
    return (unsigned)std::max<size_t>(1, (n + threads - 1) / threads);
}

// exclusive scan of n values in place (tile sums scanned recursively)
cudaError_t exclusiveScan(uint64_t* data, uint32_t n, Pool& pool, cudaStream_t s)
{
    cudaError_t err = cudaSuccess;
    if (n == 0) return err;
    uint32_t tiles = (n + kScanTile - 1) / kScanTile;
    uint64_t* sums = pool.get<uint64_t>(tiles, err);
    if (err != cudaSuccess) return err;
    scanTiles<<<tiles, kScanThreads, 0, s>>>(data, data, sums, n);
    if (tiles > 1)
    {
        if ((err = exclusiveScan(sums, tiles, pool, s)) != cudaSuccess) return err;
        scanAddOffsets<<<tiles, kScanThreads, 0, s>>>(data, sums, n);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t readBack(T& v, const T* d, cudaStream_t s)
{
    cudaError_t e = cudaMemcpyAsync(&v, d, sizeof(T), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

} // namespace

namespace
{
__global__ void triangleSlots(const float4* __restrict__ tris, uint32_t n, const uint32_t* __restrict__ primStart,
                              uint32_t* __restrict__ out)
{
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    {
        const uint32_t inst = __float_as_uint(tris[3 * (size_t)j].w), prim = __float_as_uint(tris[3 * (size_t)j + 1].w);
        out[primStart[inst] + prim] = j;
    }
}
} // namespace

int indexTrianglesByPrim(const float4* tris, uint32_t nTris, const uint32_t* primStart, uint32_t* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0xff, 4 * (size_t)std::max<uint32_t>(nTris, 1), s);
    if (e != cudaSuccess || nTris == 0) return (int)e;
    triangleSlots<<<(int)std::min<uint32_t>((nTris + 255) / 256, 4096), 256, 0, s>>>(tris, nTris, primStart, out);
    return (int)cudaGetLastError();
}

int buildWideBvh(const WideBvhInput& in, WideBvhOutput& out, cudaStream_t s, std::string& err)
{
    Pool pool;
    cudaError_t ce = cudaSuccess;
    auto cuda = [&](const char* what) {
        if (ce == cudaSuccess) ce = cudaGetLastError();
        if (ce != cudaSuccess) err = std::string(what) + ": " + cudaGetErrorString(ce);
        return ce == cudaSuccess;
    };
    const uint32_t N = in.nPrims;
    out.tris = nullptr;
    out.nodes = nullptr;
    out.nNodes = 0;
    out.depth = 0;
    // 1. triangles, bounds
    float4* trisIn = pool.get<float4>(3 * (size_t)N, ce);
    float4* plo = pool.get<float4>(N, ce);
    float4* phi = pool.get<float4>(N, ce);
    uint32_t* bounds = pool.get<uint32_t>(12, ce);
    uint32_t* instStart = pool.get<uint32_t>(in.instPrimStart.size(), ce);
    if (!cuda("bvh: allocation")) return -1;
    uint32_t init[12];
    for (int k = 0; k < 12; ++k) init[k] = k % 6 < 3 ? 0xffffffffu : 0u;
    cudaMemcpyAsync(bounds, init, sizeof(init), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(instStart, in.instPrimStart.data(), in.instPrimStart.size() * 4, cudaMemcpyHostToDevice, s);
    // the output triangles, with room for one cutout record per triangle when some instance
    // is alpha-tested (record offsets are 32-bit)
    const bool cutouts = in.alpha != nullptr && N > 0;
    if (cutouts && 6ull * N > 0xffffffffull) return err = "bvh: too many triangles for cutout records", -1;
    float4* trisOut = pool.get<float4>(3 * (size_t)std::max<uint32_t>(N, 1) * (cutouts ? 2 : 1), ce);
    if (!cuda("bvh: allocation")) return -1;
    if (N)
        worldTriangles<<<blocksFor(N, 256), 256, 0, s>>>(in.instances, instStart, in.nInstances, in.positions, in.indices, N,
                                                         trisIn, plo, phi, bounds, in.uvs, in.alpha,
                                                         cutouts ? trisOut + 3 * (size_t)N : nullptr);
    uint32_t hb[12];
    cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, s);
    if (!cuda("bvh: triangles")) return -1;
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda("bvh: triangles"), -1;
    auto unorder = [](uint32_t b) {
        uint32_t u = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
        float f;
        std::memcpy(&f, &u, 4);
        return f;
    };
    for (int a = 0; a < 3; ++a)
    {
        out.lo[a] = N ? unorder(hb[a]) : 0.f;
        out.hi[a] = N ? unorder(hb[3 + a]) : 0.f;
    }
    // the wide tree: at most one wide node per primitive, plus the root
    const size_t maxWide = (size_t)N + 1;
    float4* wide = pool.get<float4>(5 * maxWide, ce);

    if (N == 0)
    {
        // an empty root: no slot is ever hit
        float4 z[5];
        std::memset(z, 0, sizeof(z));
        uint32_t q255 = 0xffffffffu;
        float f255;
        std::memcpy(&f255, &q255, 4);
        z[0].w = 0.0f;
        z[2] = make_float4(f255, f255, f255, f255);
        z[3] = make_float4(f255, f255, 0.f, 0.f);
        cudaMemcpyAsync(wide, z, sizeof(z), cudaMemcpyHostToDevice, s);
        if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda("bvh: empty scene"), -1;
        out.nNodes = 1;
        out.depth = 1;
    }
    else
    {
        // 2. Morton order
        uint64_t* keys = pool.get<uint64_t>(N, ce);
        uint64_t* keys2 = pool.get<uint64_t>(N, ce);
        uint32_t* vals = pool.get<uint32_t>(N, ce);
        uint32_t* vals2 = pool.get<uint32_t>(N, ce);
        const uint32_t tiles = (N + kSortTile - 1) / kSortTile;
        uint64_t* hist = pool.get<uint64_t>((size_t)16 * tiles, ce);
        if (!cuda("bvh: allocation")) return -1;
        mortonCodes<<<blocksFor(N, 256), 256, 0, s>>>(plo, phi, bounds, N, keys, vals);
        for (int shift = 0; shift < 64; shift += 4)
        {
            sortHistogram<<<tiles, kSortThreads, 0, s>>>(keys, N, shift, hist, tiles);
            if ((ce = exclusiveScan(hist, 16 * tiles, pool, s)) != cudaSuccess) return cuda("bvh: sort"), -1;
            sortScatter<<<tiles, kSortThreads, 0, s>>>(keys, vals, N, shift, hist, tiles, keys2, vals2);
            std::swap(keys, keys2);
            std::swap(vals, vals2);
        }
        if (!cuda("bvh: sort")) return -1;
        // 3. PLOC binary tree: leaves 0..N-1, internal nodes N..2N-2
        const size_t nBin = 2 * (size_t)N - 1;
        float4* nlo = pool.get<float4>(nBin, ce);
        float4* nhi = pool.get<float4>(nBin, ce);
        int32_t* parent = pool.get<int32_t>(nBin, ce);
        Clusters A{pool.get<float4>(N, ce), pool.get<float4>(N, ce)};
        Clusters B{pool.get<float4>(N, ce), pool.get<float4>(N, ce)};
        int32_t* nn = pool.get<int32_t>(N, ce);
        uint64_t* flags = pool.get<uint64_t>(N, ce);
        uint64_t* scan = pool.get<uint64_t>(N, ce);
        if (!cuda("bvh: allocation")) return -1;
        cudaMemsetAsync(parent, 0xff, nBin * 4, s);
        initLeaves<<<blocksFor(N, 256), 256, 0, s>>>(vals, plo, phi, N, A, nlo, nhi);
        uint32_t n = N, nodeNext = N;
        int iter = 0;
        while (n > 1)
        {
            if (++iter > kMaxPlocIterations)
            {
                err = "bvh: clustering did not converge";
                return -1;
            }
            plocNearest<<<blocksFor(n, kPlocThreads), kPlocThreads, 0, s>>>(A, n, nn);
            plocFlags<<<blocksFor(n, 256), 256, 0, s>>>(nn, n, flags);
            cudaMemcpyAsync(scan, flags, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
            if ((ce = exclusiveScan(scan, n, pool, s)) != cudaSuccess) return cuda("bvh: clustering"), -1;
            plocCompact<<<blocksFor(n, 256), 256, 0, s>>>(A, nn, flags, scan, n, nodeNext, B, nlo, nhi, parent);
            uint64_t last = 0, lastFlag = 0;
            if ((ce = readBack(last, scan + (n - 1), s)) != cudaSuccess) return cuda("bvh: clustering"), -1;
            if ((ce = readBack(lastFlag, flags + (n - 1), s)) != cudaSuccess) return cuda("bvh: clustering"), -1;
            uint64_t total = last + lastFlag;
            uint32_t kept = (uint32_t)(total & 0xffffffffull), merged = (uint32_t)(total >> 32);
            if (merged == 0)
            {
                err = "bvh: clustering made no progress";
                return -1;
            }
            n = kept;
            nodeNext += merged;
            std::swap(A, B);
        }
        if (nodeNext != nBin)
        {
            err = "bvh: clustering produced " + std::to_string(nodeNext) + " nodes for " + std::to_string(N) + " leaves";
            return -1;
        }
        float4 rootLo;
        if ((ce = readBack(rootLo, A.lo, s)) != cudaSuccess) return cuda("bvh: clustering"), -1;
        int root = 0;
        std::memcpy(&root, &rootLo.w, 4);
        // 4. leaf decisions
        TreeCost T{pool.get<uint32_t>(nBin, ce), pool.get<float>(nBin, ce), pool.get<uint8_t>(nBin, ce),
                   pool.get<uint32_t>(nBin, ce)};
        if (!cuda("bvh: allocation")) return -1;
        cudaMemsetAsync(T.visits, 0, nBin * 4, s);
        bottomUp<<<blocksFor(N, 256), 256, 0, s>>>(nlo, nhi, parent, N, T);
        if (!cuda("bvh: leaf decisions")) return -1;
        // 5. collapse, one level of wide nodes at a time
        int32_t* items = pool.get<int32_t>(maxWide, ce);
        int32_t* items2 = pool.get<int32_t>(maxWide, ce);
        uint32_t* itemWide = pool.get<uint32_t>(maxWide, ce);
        uint32_t* itemWide2 = pool.get<uint32_t>(maxWide, ce);
        Plan* plans = pool.get<Plan>(maxWide, ce);
        uint64_t* counts = pool.get<uint64_t>(maxWide, ce);
        uint64_t* cscan = pool.get<uint64_t>(maxWide, ce);
        if (!cuda("bvh: allocation")) return -1;
        const uint32_t zero = 0;
        cudaMemcpyAsync(items, &root, 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(itemWide, &zero, 4, cudaMemcpyHostToDevice, s);
        uint32_t nItems = 1, wideNext = 1, triNext = 0, depth = 0;
        while (nItems > 0)
        {
            if (++depth > (uint32_t)kWideMaxDepth)
            {
                err = "bvh: wide tree deeper than " + std::to_string(kWideMaxDepth) + " levels";
                return -1;
            }
            collapsePlan<<<blocksFor(nItems, 128), 128, 0, s>>>(items, nItems, nlo, nhi, T, plans, counts);
            cudaMemcpyAsync(cscan, counts, (size_t)nItems * 8, cudaMemcpyDeviceToDevice, s);
            if ((ce = exclusiveScan(cscan, nItems, pool, s)) != cudaSuccess) return cuda("bvh: collapse"), -1;
            uint64_t last = 0, lastCount = 0;
            if ((ce = readBack(last, cscan + (nItems - 1), s)) != cudaSuccess) return cuda("bvh: collapse"), -1;
            if ((ce = readBack(lastCount, counts + (nItems - 1), s)) != cudaSuccess) return cuda("bvh: collapse"), -1;
            uint64_t total = last + lastCount;
            uint32_t nInternal = (uint32_t)(total & 0xffffffffull), nTris = (uint32_t)(total >> 32);
            if (wideNext + nInternal > maxWide || triNext + nTris > N)
            {
                err = "bvh: collapse overflow";
                return -1;
            }
            collapseEmit<<<blocksFor(nItems, 128), 128, 0, s>>>(items, itemWide, nItems, plans, cscan, wideNext, triNext,
                                                               nlo, nhi, T, trisIn, trisOut, wide, items2, itemWide2);
            if (!cuda("bvh: collapse")) return -1;
            wideNext += nInternal;
            triNext += nTris;
            nItems = nInternal;
            std::swap(items, items2);
            std::swap(itemWide, itemWide2);
        }
        if (triNext != N)
        {
            err = "bvh: " + std::to_string(triNext) + " of " + std::to_string(N) + " triangles placed";
            return -1;
        }
        out.nNodes = wideNext;
        out.depth = depth;
    }
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda("bvh: build"), -1;
    // hand the two results to the caller (the pool frees the rest)
    for (auto& p : pool.ptrs)
        if (p == wide || p == trisOut) p = nullptr;
    out.nodes = wide;
    out.tris = trisOut;
    return 0;
}

} // namespace yg
