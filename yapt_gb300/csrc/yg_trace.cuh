// Closest-hit ray traversal of the device BVH (replaces DXR TraceRay / RayQuery,
// rayGenPrimaryRays.hlsl:62 and rayHitDefault.hlsl:83-133).
//
// Wide node (80 B, five float4 read with 128-bit read-only loads; built by yg_bvh_build.cu):
//   n0 = (p.x, p.y, p.z, e.x | e.y << 8 | e.z << 16 | imask << 24)
//   n1 = (child base, triangle base, meta[0..3], meta[4..7])        (uint32 / uint8 lanes)
//   n2 = (qlo.x[0..3], qlo.x[4..7], qlo.y[0..3], qlo.y[4..7])
//   n3 = (qlo.z[0..3], qlo.z[4..7], qhi.x[0..3], qhi.x[4..7])
//   n4 = (qhi.y[0..3], qhi.y[4..7], qhi.z[0..3], qhi.z[4..7])
// Child slot i spans p + 2^(e-127) * [qlo[i], qhi[i]] per axis (conservative: the builder
// rounds outward and pads one quantum). imask bit i: slot i is an inner node, stored at
// child base + (inner slots below i). Otherwise meta[i] = count << 5 | offset: a leaf of
// `count` triangles at triangle base + offset; meta[i] == 0: empty slot.
// Triangles (48 B): (v0.xyz, instance) (e1.xyz, primitive) (e2.xyz, cutout), world space.
// cutout = 0 for an opaque triangle; otherwise the float4 offset from the triangle array's
// start of the triangle's cutout record (three float4 behind all the triangles):
//   (uv0, uv1) (uv2, albedo uv scale) (texels pointer lo, hi, width | height << 16, cutoff)
// A candidate hit that would become the closest one is dropped when the albedo alpha at its
// uv is below the cutoff (PROCEED_ALPHA_TESTED / rayAnyHitAlphaTest.hlsl), for closest-hit
// and shadow rays alike, so the result does not depend on the order the tree is visited in.
//
// Traversal keeps one group of unvisited inner children (child base, inner mask, hit mask
// in near-to-far key order) and a stack of such groups. Children sit in slots by octant, so
// visiting keys in increasing order, slot = key XOR (ray direction sign bits), goes roughly
// near to far. The triangles of a node's leaf slots are tested when the node is opened.
//
// Intersection is Moller-Trumbore with a fixed operation order; hits count when
// tmin < t < tmax. Equal-t hits resolve to the smaller (instance, primitive) so
// the result does not depend on the tree layout. Front face = determinant > 0
// (the ray sees the side the geometric normal cross(e1, e2) points to), which is
// DXR's default clockwise-in-left-handed-space rule.
#pragma once
#include "yg_vec.cuh"
#include "yg_types.h"

namespace yg
{

struct Hit
{
    float t;
    float b1, b2;
    uint32_t instance;
    uint32_t prim;
    bool front;
};

YG_HD bool keyLess(uint32_t ia, uint32_t pa, uint32_t ib, uint32_t pb)
{
    return ia < ib || (ia == ib && pa < pb);
}

// Texture2D.SampleLevel(LINEAR_REPEAT, uv, 0): bilinear between the four nearest texel
// centres, coordinates wrapped. Done in FP32 arithmetic (not the texture unit's 8-bit
// fraction) so that a CPU restatement computes the same value.
__device__ __forceinline__ float4 bilinearWrap(const float4* __restrict__ texels, uint32_t width, uint32_t height, float2 uv)
{
    const float w = (float)width, h = (float)height;
    float u = uv.x - floorf(uv.x), v = uv.y - floorf(uv.y);
    float x = u * w - 0.5f, y = v * h - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float tx = x - fx, ty = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    const int W = (int)width, H = (int)height;
    x0 = x0 < 0 ? x0 + W : (x0 >= W ? x0 - W : x0);
    y0 = y0 < 0 ? y0 + H : (y0 >= H ? y0 - H : y0);
    const int x1 = x0 + 1 == W ? 0 : x0 + 1, y1 = y0 + 1 == H ? 0 : y0 + 1;
    const float4 c00 = __ldg(texels + (size_t)y0 * W + x0), c10 = __ldg(texels + (size_t)y0 * W + x1);
    const float4 c01 = __ldg(texels + (size_t)y1 * W + x0), c11 = __ldg(texels + (size_t)y1 * W + x1);
    const float sx = 1.0f - tx, sy = 1.0f - ty;
    return (c00 * sx + c10 * tx) * sy + (c01 * sx + c11 * tx) * ty;
}

// alphaTestPasses (hitShadersCommon.hlsl:162-183) on a triangle's cutout record, at the
// barycentrics (b1, b2) of a candidate hit. Out of line: only alpha-tested triangles pay.
static __device__ __noinline__ bool cutoutPasses(const float4* __restrict__ r, float b1, float b2)
{
    const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
    const float b0 = 1.0f - b1 - b2;
    const float u = a.x * b0 + a.z * b1 + b.x * b2, v = a.y * b0 + a.w * b1 + b.y * b2;
    const uint64_t lo = __float_as_uint(c.x), hi = __float_as_uint(c.y);
    const float4* texels = reinterpret_cast<const float4*>(lo | hi << 32);
    const uint32_t size = __float_as_uint(c.z);
    const float4 t = bilinearWrap(texels, size & 0xffffu, size >> 16, make_float2(u * b.z, v * b.w));
    return t.w >= c.w;
}

// onlyInst: with FILTER, triangles of every other instance are ignored (the subsurface probe
// rays, which look for the surface of the instance they started in)
template <bool FILTER = false>
__device__ __forceinline__ void intersectTri(const float4* __restrict__ tris, int ti, float3 o, float3 d, float tmin,
                                             Hit& h, bool& found, uint32_t onlyInst = 0)
{
    float4 a = __ldg(tris + 3 * ti);
    if (FILTER && __float_as_uint(a.w) != onlyInst) return;
    float4 b = __ldg(tris + 3 * ti + 1);
    float4 c = __ldg(tris + 3 * ti + 2);
    float3 v0 = mk3(a.x, a.y, a.z), e1 = mk3(b.x, b.y, b.z), e2 = mk3(c.x, c.y, c.z);
    float3 pvec = cross(d, e2);
    float det = dot(e1, pvec);
    if (det == 0.0f) return;
    float inv = 1.0f / det;
    float3 tvec = o - v0;
    float u = dot(tvec, pvec) * inv;
    if (u < 0.0f || u > 1.0f) return;
    float3 qvec = cross(tvec, e1);
    float v = dot(d, qvec) * inv;
    if (v < 0.0f || u + v > 1.0f) return;
    float t = dot(e2, qvec) * inv;
    if (!(t > tmin)) return;
    uint32_t inst = __float_as_uint(a.w), prim = __float_as_uint(b.w);
    if (t < h.t || (t == h.t && found && keyLess(inst, prim, h.instance, h.prim)))
    {
        const uint32_t cut = __float_as_uint(c.w);
        if (cut != 0u && !cutoutPasses(tris + cut, u, v)) return;
        h.t = t;
        h.b1 = u;
        h.b2 = v;
        h.instance = inst;
        h.prim = prim;
        h.front = det > 0.0f;
        found = true;
    }
}

// Traversal work counters (nodes visited, triangles tested), used to measure the
// algorithmic bytes of a workload; compiled in only for the counting kernel.
struct TraversalCount
{
    uint32_t nodes, tris;
};

constexpr int kTraversalStack = 32;    // one group per wide level (the builder caps the depth)
constexpr uint32_t kMaxNodeVisits = 1u << 20; // a guard only: a valid tree never reaches it

// Byte i of the 8-byte lane pair (lo4, hi4) as the float 2^23 + byte: the byte is placed
// in the low mantissa bits of 2^23 by one PRMT. The 2^23 bias is folded into the plane
// offset of the node (see traceStep).
__device__ __forceinline__ float biasedByte(uint32_t lo4, uint32_t hi4, int i)
{
    const uint32_t sel = (uint32_t)(i & 3) | 0x7650u; // byte i, then bytes 1..3 of 0x4B000000
    return __uint_as_float(__byte_perm(i < 4 ? lo4 : hi4, 0x4B000000u, sel));
}

// One ray's traversal, advanced one node at a time by traceStep so that a persistent
// kernel can hand a lane a new ray as soon as its ray is done.
// Debug build (YG_DEBUG_BOUNDS): node and triangle indices are checked against the scene's
// counts before they are read; an out-of-range index is counted in the scene's error word and
// the access skipped (the traversal ends), so a faulty tree shows as a count, never as a fault.
#ifdef YG_DEBUG_BOUNDS
#define YG_BOUNDS(ok, errors)                                                                                          \
    (((ok) ? true : ((errors) ? (atomicAdd((errors), 1u), false) : false)))
#else
#define YG_BOUNDS(ok, errors) true
#endif

struct TraceState
{
    const float4* nodes;
    const float4* tris;
#ifdef YG_DEBUG_BOUNDS
    uint32_t nNodes, nTris;
    unsigned int* errors;
#endif
    float3 o, d, inv;
    float tmin;
    uint32_t oct;
    Hit h;
    bool found;
    uint32_t gBase, gImask, gHits, visits;
    int sp;
    uint32_t onlyInst; // the instance a filtered traversal is restricted to
};
// the groups waiting below the current one (kept apart from TraceState so that the state's
// scalars stay in registers), all in local memory
struct TraceStack
{
    uint2 e[kTraversalStack];
    __device__ __forceinline__ void push(int sp, uint2 v) { e[sp] = v; }
    __device__ __forceinline__ uint2 pop(int sp) const { return e[sp]; }
};

// The same stack with its top kSharedStack entries in the block's shared memory: one slice per
// thread, laid out [entry][thread] so that a warp's entries fall in distinct banks. The wide
// tree is shallow (a few levels for 10^5-10^6 triangles), so the deeper local-memory entries are
// rarely touched and the node and triangle loads keep the L1 to themselves.
constexpr int kSharedStack = 8;
constexpr int kTraceBlock = 128; // the block size of every kernel that uses traceGrid
// resident blocks per SM the traversal kernels ask for (__launch_bounds__ minimum): 7 keeps
// them at 72 registers or fewer, the 7 blocks their plain loop had, where the refill loop
// below would otherwise take 74-78 and one block fewer; 12 or 16 blocks measured slower
#ifndef YG_TRACE_MIN_BLOCKS
#define YG_TRACE_MIN_BLOCKS 7
#endif
// the same for the NEE shadow-ray kernel
#ifndef YG_SHADOW_MIN_BLOCKS
#define YG_SHADOW_MIN_BLOCKS 7
#endif
struct SharedTraceStack
{
    uint2* sh; // this thread's slice (entry k at sh[k * kTraceBlock]), or null: local only
    uint2 e[kTraversalStack];
    __device__ __forceinline__ void push(int sp, uint2 v)
    {
        if (sh && sp < kSharedStack) sh[sp * kTraceBlock] = v;
        else e[sp] = v;
    }
    __device__ __forceinline__ uint2 pop(int sp) const
    {
        if (sh && sp < kSharedStack) return sh[sp * kTraceBlock];
        return e[sp];
    }
};

__device__ __forceinline__ void traceBegin(TraceState& t, const SceneView& S, float3 o, float3 d, float tmin, float tmax)
{
    t.nodes = S.nodes;
    t.tris = S.tris;
#ifdef YG_DEBUG_BOUNDS
    t.nNodes = S.nNodes;
    t.nTris = S.nTris;
    t.errors = S.boundsErrors;
#endif
    t.o = o;
    t.d = d;
    t.inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    t.tmin = tmin;
    t.oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    t.h.t = tmax;
    t.found = false;
    // the root as the only inner child of a virtual parent
    t.gBase = 0;
    t.gImask = 1u;
    t.gHits = 1u << t.oct;
    t.visits = 0;
    t.sp = 0;
}

// Opens the next node (testing its eight child boxes and the triangles of the leaf slots
// that are hit); returns false once nothing is left to visit.
template <bool COUNT, typename Stack, bool FILTER = false>
__device__ __forceinline__ bool traceStep(TraceState& t, Stack& st, TraversalCount* tc)
{
    if (t.gHits == 0)
    {
        if (t.sp == 0) return false;
        const uint2 e = st.pop(--t.sp);
        t.gBase = e.x;
        t.gHits = e.y & 0xffu;
        t.gImask = e.y >> 8;
    }
    const uint32_t slot = (uint32_t)(__ffs(t.gHits) - 1) ^ t.oct;
    t.gHits &= t.gHits - 1;
    const uint32_t idx = t.gBase + __popc(t.gImask & ((1u << slot) - 1u));
#ifdef YG_DEBUG_BOUNDS
    if (!YG_BOUNDS(idx < t.nNodes, t.errors))
    {
        t.gHits = 0;
        t.sp = 0;
        return false;
    }
#endif
    if (++t.visits > kMaxNodeVisits) return false;
    const float4* __restrict__ np = t.nodes + 5 * (size_t)idx;
    const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
    if (COUNT) tc->nodes++;
    const uint32_t packed = __float_as_uint(n0.w);
    const uint32_t imask = packed >> 24;
    const float3 inv = t.inv, o = t.o;
    // per axis: t(q) = q * (scale / d) + (p - o) / d, evaluated as (2^23 + q) * sx + b' with
    // b' = (p - o) / d - 2^23 * sx. Rounding b' errs by at most half a quantum (|sx| / 2),
    // within the quantum of outward padding every child box carries.
    const float sx = __uint_as_float((packed & 0xffu) << 23) * inv.x;
    const float sy = __uint_as_float(((packed >> 8) & 0xffu) << 23) * inv.y;
    const float sz = __uint_as_float(((packed >> 16) & 0xffu) << 23) * inv.z;
    const float bx = fmaf(-8388608.0f, sx, (n0.x - o.x) * inv.x);
    const float by = fmaf(-8388608.0f, sy, (n0.y - o.y) * inv.y);
    const float bz = fmaf(-8388608.0f, sz, (n0.z - o.z) * inv.z);
    const uint32_t m0 = __float_as_uint(n1.z), m1 = __float_as_uint(n1.w);
    // near and far planes per axis chosen once by the sign of the direction
    const uint32_t lx0 = __float_as_uint(n2.x), lx1 = __float_as_uint(n2.y);
    const uint32_t ly0 = __float_as_uint(n2.z), ly1 = __float_as_uint(n2.w);
    const uint32_t lz0 = __float_as_uint(n3.x), lz1 = __float_as_uint(n3.y);
    const uint32_t hx0 = __float_as_uint(n3.z), hx1 = __float_as_uint(n3.w);
    const uint32_t hy0 = __float_as_uint(n4.x), hy1 = __float_as_uint(n4.y);
    const uint32_t hz0 = __float_as_uint(n4.z), hz1 = __float_as_uint(n4.w);
    const uint32_t oct = t.oct;
    const bool nx = oct & 1u, ny = oct & 2u, nz = oct & 4u;
    const uint32_t nx0 = nx ? hx0 : lx0, nx1 = nx ? hx1 : lx1, fx0 = nx ? lx0 : hx0, fx1 = nx ? lx1 : hx1;
    const uint32_t ny0 = ny ? hy0 : ly0, ny1 = ny ? hy1 : ly1, fy0 = ny ? ly0 : hy0, fy1 = ny ? ly1 : hy1;
    const uint32_t nz0 = nz ? hz0 : lz0, nz1 = nz ? hz1 : lz1, fz0 = nz ? lz0 : hz0, fz1 = nz ? lz1 : hz1;
    const float tmin = t.tmin, tfar = t.h.t;
    uint32_t hits = 0, triHits = 0;
    // all eight slots unrolled (a loop over the occupied slots only, with runtime byte
    // selects, measured slower)
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
        const uint32_t meta = ((i < 4 ? m0 : m1) >> (8 * (i & 3))) & 0xffu;
        if (meta == 0) continue;
        const float tnx = fmaf(biasedByte(nx0, nx1, i), sx, bx), tfx = fmaf(biasedByte(fx0, fx1, i), sx, bx);
        const float tny = fmaf(biasedByte(ny0, ny1, i), sy, by), tfy = fmaf(biasedByte(fy0, fy1, i), sy, by);
        const float tnz = fmaf(biasedByte(nz0, nz1, i), sz, bz), tfz = fmaf(biasedByte(fz0, fz1, i), sz, bz);
        // NaN terms (a zero direction component) drop out of fmaxf/fminf: that axis does not cull
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
        // tfar widened by 4 ulp so grazing hits on box faces are kept
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tfar)) * 1.0000005f;
        if (!(tn <= tf)) continue;
        if (imask & (1u << i)) hits |= 1u << i;
        else triHits |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
    }
    // slot order -> key order: key = slot XOR oct swaps bits, bit pairs and nibbles
    if (oct & 1u) hits = ((hits & 0x55u) << 1) | ((hits & 0xAAu) >> 1);
    if (oct & 2u) hits = ((hits & 0x33u) << 2) | ((hits & 0xCCu) >> 2);
    if (oct & 4u) hits = ((hits & 0x0Fu) << 4) | ((hits & 0xF0u) >> 4);
    if (triHits)
    {
        const uint32_t triBase = __float_as_uint(n1.y);
        if (COUNT) tc->tris += __popc(triHits);
        while (triHits)
        {
            const uint32_t j = __ffs(triHits) - 1;
            triHits &= triHits - 1;
#ifdef YG_DEBUG_BOUNDS
            if (!YG_BOUNDS(triBase + j < t.nTris, t.errors)) continue;
#endif
            intersectTri<FILTER>(t.tris, (int)(triBase + j), t.o, t.d, t.tmin, t.h, t.found, t.onlyInst);
        }
    }
    if (hits)
    {
        // descend; the rest of the current group waits on the stack (one entry per
        // level, and the builder keeps the tree within kTraversalStack levels)
        if (t.gHits && t.sp < kTraversalStack) st.push(t.sp++, make_uint2(t.gBase, t.gHits | (t.gImask << 8)));
        t.gBase = __float_as_uint(n1.x);
        t.gImask = imask;
        t.gHits = hits;
    }
    return t.gHits != 0 || t.sp != 0;
}

// Returns true if something was hit in (tmin, tmax); h.t starts at tmax.
template <bool COUNT>
__device__ __noinline__ bool traceClosest(const SceneView& S, float3 o, float3 d, float tmin, float tmax, Hit& h,
                                          TraversalCount* tc)
{
    TraceState t;
    TraceStack st;
    traceBegin(t, S, o, d, tmin, tmax);
    while (traceStep<COUNT>(t, st, tc)) {}
    h = t.h;
    return t.found;
}

// The closest hit in (tmin, tmax) on the triangles of instance `inst` alone, as the reference's
// subsurface probe query commits only that instance's hits (subsurface.hlsl:265-274).
static __device__ __noinline__ bool traceInstanceClosest(const SceneView& S, float3 o, float3 d, float tmin, float tmax,
                                                  uint32_t inst, Hit& h)
{
    TraceState t;
    TraceStack st;
    traceBegin(t, S, o, d, tmin, tmax);
    t.onlyInst = inst;
    while (traceStep<false, TraceStack, true>(t, st, nullptr)) {}
    h = t.h;
    return t.found;
}

// Traverses rays 0..n-1 of a queue, one ray per thread at a time, in grid-stride order.
// A warp takes its rays in that order (its k-th ray is (k / 32) * 32 * warps + warp * 32 +
// k % 32), and once fewer than K of its lanes still have a ray, the idle lanes finish theirs
// (end) and take the next rays of the order together (begin): the warp no longer runs at the
// occupancy of its longest ray, one ballot per node is the bookkeeping, and the rays in flight
// on the GPU stay a contiguous stretch of the queue (neighbouring pixels, shared nodes in L2).
// Every ray is traversed exactly as by a plain loop. Measured on the NEE workload (K = 24):
// shadow rays 12 % and closest-hit rays 6 % faster than one ray per thread to completion; a
// contiguous chunk of the queue per warp instead of the interleaved order lost 5 % on the
// closest-hit rays (the rays in flight spread over the whole image), and handing a lane a new
// ray as soon as it finished (a shared queue cursor) lost more than the idle lanes cost.
// The group stack stays in local memory: its top entries live in L1 anyway, and staging them
// in shared memory (YG_TRACE_SHARED_STACK, 8 KB per block, plain loop only) measured 3 % slower
// on the NEE workload's traversal, the smaller L1 costing more node hits than the stack saves.
// With `stop`, a ray's traversal also ends as soon as stop(state) holds after a node.
// YG_TRACE_REFILL (closest hit) and YG_SHADOW_REFILL (any hit) set K; 0 is the plain loop.
#ifndef YG_TRACE_REFILL
#define YG_TRACE_REFILL 24
#endif
#ifndef YG_SHADOW_REFILL
#define YG_SHADOW_REFILL 24
#endif
template <int K, bool COUNT, typename Begin, typename End, typename Stop>
__device__ __forceinline__ void traceGridRefill(uint32_t n, Begin begin, End end, Stop stop, TraversalCount& tc,
                                                uint32_t& rays)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t span = gridDim.x * blockDim.x; // rays per round of the grid-stride order
    const uint32_t warpBase = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    uint32_t next = 0; // the warp's next position k in its order
    TraceState t;
    TraceStack st;
    uint32_t cur = 0;
    bool busy = false, pending = false;
    for (;;)
    {
        uint32_t busyMask = __ballot_sync(0xffffffffu, busy);
        if (__popc(busyMask) < K)
        {
            if (pending)
            {
                end(t, cur);
                ++rays;
                pending = false;
            }
            const uint32_t idle = ~busyMask;
            const uint32_t k = next + (uint32_t)__popc(idle & ((1u << lane) - 1u));
            const uint64_t r = (uint64_t)(k >> 5) * span + warpBase + (k & 31u);
            if (!busy && r < n)
            {
                cur = (uint32_t)r;
                begin(t, cur);
                busy = true;
            }
            next += (uint32_t)__popc(idle);
            busyMask = __ballot_sync(0xffffffffu, busy);
            if (busyMask == 0u) break;
        }
        if (busy && (!traceStep<COUNT>(t, st, &tc) || stop(t)))
        {
            busy = false;
            pending = true;
        }
    }
}

template <bool COUNT, typename Begin, typename End, typename Stop>
__device__ __forceinline__ void traceGridStop(uint32_t n, Begin begin, End end, Stop stop, TraversalCount& tc,
                                              uint32_t& rays)
{
#if YG_SHADOW_REFILL > 0
    traceGridRefill<YG_SHADOW_REFILL, COUNT>(n, begin, end, stop, tc, rays);
#else
    TraceState t;
#ifdef YG_TRACE_SHARED_STACK
    __shared__ uint2 stackTop[kSharedStack * kTraceBlock];
    SharedTraceStack st;
    st.sh = threadIdx.x < (uint32_t)kTraceBlock ? stackTop + threadIdx.x : nullptr;
#else
    TraceStack st;
#endif
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        begin(t, i);
        while (traceStep<COUNT>(t, st, &tc))
            if (stop(t)) break;
        end(t, i);
        ++rays;
    }
#endif
}
template <bool COUNT, typename Begin, typename End>
__device__ __forceinline__ void traceGrid(uint32_t n, Begin begin, End end, TraversalCount& tc, uint32_t& rays)
{
#if YG_TRACE_REFILL > 0
    traceGridRefill<YG_TRACE_REFILL, COUNT>(n, begin, end, [](const TraceState&) { return false; }, tc, rays);
#else
    TraceState t;
#ifdef YG_TRACE_SHARED_STACK
    __shared__ uint2 stackTop[kSharedStack * kTraceBlock];
    SharedTraceStack st;
    st.sh = threadIdx.x < (uint32_t)kTraceBlock ? stackTop + threadIdx.x : nullptr;
#else
    TraceStack st;
#endif
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        begin(t, i);
        while (traceStep<COUNT>(t, st, &tc)) {}
        end(t, i);
        ++rays;
    }
#endif
}

} // namespace yg
