// Binned-SAH binary BVH over world-space triangles, written in the node format the
// traversal kernel reads (yg_trace.cuh). Replaces YAPT's DXR BLAS/TLAS builds
// (AccelerationStructureHelper.cpp:96-213): every (instance, submesh) is flattened
// into one world-space triangle set, so a ray needs one traversal, no instance
// transform per node, and closest-hit keys stay (instance, primitive).
#include "yg_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace yg
{
namespace
{
struct Box
{
    float lo[3], hi[3];
    void reset()
    {
        for (int a = 0; a < 3; ++a)
        {
            lo[a] = std::numeric_limits<float>::infinity();
            hi[a] = -std::numeric_limits<float>::infinity();
        }
    }
    void grow(const Box& b)
    {
        for (int a = 0; a < 3; ++a)
        {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(const float* p)
    {
        for (int a = 0; a < 3; ++a)
        {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    float area() const
    {
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = std::max(0.0f, hi[a] - lo[a]);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct Ref
{
    Box box;
    float c[3];
    uint32_t tri;
};

constexpr int kBins = 16;
constexpr int kMaxLeaf = 8;
constexpr int kMaxDepth = 56; // keeps the traversal stack (64) from overflowing

struct Builder
{
    std::vector<Ref> refs;
    std::vector<float4>* nodes;
    std::vector<uint32_t> order;

    struct Child
    {
        int index; // node index or first triangle
        int count; // 0 for an inner node
        Box box;
    };

    int newNode()
    {
        int n = (int)(nodes->size() / 4);
        nodes->resize(nodes->size() + 4);
        return n;
    }

    void writeNode(int n, const Child& a, const Child& b)
    {
        float4* p = nodes->data() + 4 * n;
        p[0] = make_float4(a.box.lo[0], a.box.hi[0], a.box.lo[1], a.box.hi[1]);
        p[1] = make_float4(b.box.lo[0], b.box.hi[0], b.box.lo[1], b.box.hi[1]);
        p[2] = make_float4(a.box.lo[2], a.box.hi[2], b.box.lo[2], b.box.hi[2]);
        int ia = a.index, ib = b.index, ca = a.count, cb = b.count;
        float4 q;
        std::memcpy(&q.x, &ia, 4);
        std::memcpy(&q.y, &ib, 4);
        std::memcpy(&q.z, &ca, 4);
        std::memcpy(&q.w, &cb, 4);
        p[3] = q;
    }

    Child leaf(int begin, int end, const Box& b) { return Child{begin, end - begin, b}; }

    Child build(int begin, int end, int depth)
    {
        Box bounds, cb;
        bounds.reset();
        cb.reset();
        for (int i = begin; i < end; ++i)
        {
            bounds.grow(refs[i].box);
            cb.grow(refs[i].c);
        }
        int n = end - begin;
        if (n <= 2 || depth >= kMaxDepth) return leaf(begin, end, bounds);
        // binned SAH over the three axes
        float bestCost = std::numeric_limits<float>::infinity();
        int bestAxis = -1, bestSplit = -1;
        for (int a = 0; a < 3; ++a)
        {
            float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.0f)) continue;
            Box bb[kBins];
            int cnt[kBins] = {0};
            for (int k = 0; k < kBins; ++k) bb[k].reset();
            float scale = kBins / ext;
            for (int i = begin; i < end; ++i)
            {
                int k = std::min(kBins - 1, (int)((refs[i].c[a] - cb.lo[a]) * scale));
                cnt[k]++;
                bb[k].grow(refs[i].box);
            }
            float rightArea[kBins];
            int rightCnt[kBins];
            Box acc;
            acc.reset();
            int c = 0;
            for (int k = kBins - 1; k > 0; --k)
            {
                acc.grow(bb[k]);
                c += cnt[k];
                rightArea[k] = acc.area();
                rightCnt[k] = c;
            }
            acc.reset();
            c = 0;
            for (int k = 0; k < kBins - 1; ++k)
            {
                acc.grow(bb[k]);
                c += cnt[k];
                if (c == 0 || rightCnt[k + 1] == 0) continue;
                float cost = acc.area() * c + rightArea[k + 1] * rightCnt[k + 1];
                if (cost < bestCost)
                {
                    bestCost = cost;
                    bestAxis = a;
                    bestSplit = k;
                }
            }
        }
        float parentArea = bounds.area();
        float leafCost = (float)n;
        float splitCost = parentArea > 0.0f ? 1.0f + bestCost / parentArea : std::numeric_limits<float>::infinity();
        int mid;
        if (bestAxis < 0)
        {
            if (n <= kMaxLeaf) return leaf(begin, end, bounds);
            mid = begin + n / 2; // all centroids coincide: split the list in two
        }
        else
        {
            if (n <= kMaxLeaf && leafCost <= splitCost) return leaf(begin, end, bounds);
            float ext = cb.hi[bestAxis] - cb.lo[bestAxis];
            float scale = kBins / ext;
            auto it = std::partition(refs.begin() + begin, refs.begin() + end, [&](const Ref& r) {
                int k = std::min(kBins - 1, (int)((r.c[bestAxis] - cb.lo[bestAxis]) * scale));
                return k <= bestSplit;
            });
            mid = (int)(it - refs.begin());
            if (mid == begin || mid == end) mid = begin + n / 2;
        }
        int node = newNode();
        Child l = build(begin, mid, depth + 1);
        Child r = build(mid, end, depth + 1);
        writeNode(node, l, r);
        return Child{node, 0, bounds};
    }
};
} // namespace

void buildBvh(const std::vector<float3>& v0, const std::vector<float3>& v1, const std::vector<float3>& v2,
              const std::vector<uint32_t>& instance, const std::vector<uint32_t>& prim, std::vector<float4>& trisOut,
              std::vector<float4>& nodesOut)
{
    size_t n = v0.size();
    Builder B;
    B.nodes = &nodesOut;
    nodesOut.clear();
    B.refs.resize(n);
    for (size_t i = 0; i < n; ++i)
    {
        Ref& r = B.refs[i];
        r.box.reset();
        float a[3] = {v0[i].x, v0[i].y, v0[i].z}, b[3] = {v1[i].x, v1[i].y, v1[i].z}, c[3] = {v2[i].x, v2[i].y, v2[i].z};
        r.box.grow(a);
        r.box.grow(b);
        r.box.grow(c);
        // pad by a few ulp: the kernel tests the triangle (v0, v0 + e1, v0 + e2) with
        // rounded edges, whose corners may sit an ulp outside the box of v0, v1, v2
        for (int k = 0; k < 3; ++k)
        {
            r.box.lo[k] -= 4e-7f * std::max(1.0f, std::fabs(r.box.lo[k]));
            r.box.hi[k] += 4e-7f * std::max(1.0f, std::fabs(r.box.hi[k]));
        }
        for (int k = 0; k < 3; ++k) r.c[k] = 0.5f * (r.box.lo[k] + r.box.hi[k]);
        r.tri = (uint32_t)i;
    }
    if (n == 0)
    {
        Box e;
        e.reset();
        int node = B.newNode();
        B.writeNode(node, Builder::Child{-1, 0, e}, Builder::Child{-1, 0, e});
    }
    else
    {
        int node = B.newNode(); // node 0 is always an inner node
        Builder::Child c = B.build(0, (int)n, 1);
        if (c.count > 0)
        {
            Box e;
            e.reset();
            B.writeNode(node, c, Builder::Child{-1, 0, e});
        }
        else
        {
            // move the built root into slot 0
            for (int k = 0; k < 4; ++k) nodesOut[k] = nodesOut[4 * c.index + k];
            Box e;
            e.reset();
            // leave the old slot as an unreachable empty node
            B.writeNode(c.index, Builder::Child{-1, 0, e}, Builder::Child{-1, 0, e});
        }
    }
    trisOut.resize(3 * n);
    for (size_t i = 0; i < n; ++i)
    {
        uint32_t t = B.refs[i].tri;
        float3 e1 = make_float3(v1[t].x - v0[t].x, v1[t].y - v0[t].y, v1[t].z - v0[t].z);
        float3 e2 = make_float3(v2[t].x - v0[t].x, v2[t].y - v0[t].y, v2[t].z - v0[t].z);
        float iw, pw;
        std::memcpy(&iw, &instance[t], 4);
        std::memcpy(&pw, &prim[t], 4);
        trisOut[3 * i] = make_float4(v0[t].x, v0[t].y, v0[t].z, iw);
        trisOut[3 * i + 1] = make_float4(e1.x, e1.y, e1.z, pw);
        trisOut[3 * i + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    }
}

} // namespace yg
