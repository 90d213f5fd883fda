// Closest-hit ray traversal of the device BVH (replaces DXR TraceRay / RayQuery,
// rayGenPrimaryRays.hlsl:62 and rayHitDefault.hlsl:83-133).
//
// Node format (64 B, four float4, loaded with 128-bit read-only loads):
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0, child1, count0, count1) as int: count > 0 -> leaf of `count`
//        triangles starting at triangle `child`; count == 0 -> inner node `child`;
//        child < 0 -> empty slot.
// Triangles (48 B): (v0.xyz, instance) (e1.xyz, primitive) (e2.xyz, 0), world space.
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

constexpr int kTraversalStack = 64;

YG_HD bool keyLess(uint32_t ia, uint32_t pa, uint32_t ib, uint32_t pb)
{
    return ia < ib || (ia == ib && pa < pb);
}

__device__ __forceinline__ void intersectTri(const float4* __restrict__ tris, int ti, float3 o, float3 d, float tmin,
                                             Hit& h, bool& found)
{
    float4 a = __ldg(tris + 3 * ti);
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

// Returns true if something was hit in (tmin, tmax); h.t starts at tmax.
template <bool COUNT>
__device__ __noinline__ bool traceClosest(const SceneView& S, float3 o, float3 d, float tmin, float tmax, Hit& h,
                                          TraversalCount* tc)
{
    h.t = tmax;
    bool found = false;
    float3 inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float3 oi = mk3(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    int stack[kTraversalStack];
    int sp = 0;
    int node = 0;
    const float4* __restrict__ nodes = S.nodes;
    const float4* __restrict__ tris = S.tris;
    while (true)
    {
        float4 n0 = __ldg(nodes + 4 * node);
        float4 n1 = __ldg(nodes + 4 * node + 1);
        float4 n2 = __ldg(nodes + 4 * node + 2);
        float4 n3 = __ldg(nodes + 4 * node + 3);
        if (COUNT) tc->nodes++;
        // slab tests; tfar widened by 4 ulp so grazing hits on box faces are kept
        float c0lx = fmaf(n0.x, inv.x, -oi.x), c0hx = fmaf(n0.y, inv.x, -oi.x);
        float c0ly = fmaf(n0.z, inv.y, -oi.y), c0hy = fmaf(n0.w, inv.y, -oi.y);
        float c0lz = fmaf(n2.x, inv.z, -oi.z), c0hz = fmaf(n2.y, inv.z, -oi.z);
        float c1lx = fmaf(n1.x, inv.x, -oi.x), c1hx = fmaf(n1.y, inv.x, -oi.x);
        float c1ly = fmaf(n1.z, inv.y, -oi.y), c1hy = fmaf(n1.w, inv.y, -oi.y);
        float c1lz = fmaf(n2.z, inv.z, -oi.z), c1hz = fmaf(n2.w, inv.z, -oi.z);
        float tn0 = fmaxf(fmaxf(fminf(c0lx, c0hx), fminf(c0ly, c0hy)), fmaxf(fminf(c0lz, c0hz), tmin));
        float tf0 = fminf(fminf(fmaxf(c0lx, c0hx), fmaxf(c0ly, c0hy)), fminf(fmaxf(c0lz, c0hz), h.t)) * 1.0000005f;
        float tn1 = fmaxf(fmaxf(fminf(c1lx, c1hx), fminf(c1ly, c1hy)), fmaxf(fminf(c1lz, c1hz), tmin));
        float tf1 = fminf(fminf(fmaxf(c1lx, c1hx), fmaxf(c1ly, c1hy)), fminf(fmaxf(c1lz, c1hz), h.t)) * 1.0000005f;
        int ch0 = __float_as_int(n3.x), ch1 = __float_as_int(n3.y);
        int cnt0 = __float_as_int(n3.z), cnt1 = __float_as_int(n3.w);
        bool hit0 = ch0 >= 0 && tn0 <= tf0;
        bool hit1 = ch1 >= 0 && tn1 <= tf1;
        if (hit0 && cnt0 > 0)
        {
            for (int i = 0; i < cnt0; ++i) intersectTri(tris, ch0 + i, o, d, tmin, h, found);
            if (COUNT) tc->tris += cnt0;
            hit0 = false;
        }
        if (hit1 && cnt1 > 0)
        {
            for (int i = 0; i < cnt1; ++i) intersectTri(tris, ch1 + i, o, d, tmin, h, found);
            if (COUNT) tc->tris += cnt1;
            hit1 = false;
        }
        if (hit0 && hit1)
        {
            int nearN = tn0 <= tn1 ? ch0 : ch1;
            int farN = tn0 <= tn1 ? ch1 : ch0;
            if (sp < kTraversalStack) stack[sp++] = farN;
            node = nearN;
        }
        else if (hit0)
        {
            node = ch0;
        }
        else if (hit1)
        {
            node = ch1;
        }
        else
        {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return found;
}

} // namespace yg
