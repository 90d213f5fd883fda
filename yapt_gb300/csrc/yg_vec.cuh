// Small vector helpers with a fixed evaluation order.
//
// Every operation is written out so that the arithmetic sequence is the same on
// every compiler: dot products sum left to right, normalize multiplies by one
// reciprocal, no operation relies on contraction into FMA (device code is built
// with -fmad=false). Row-vector/matrix conventions follow HLSL: a float3x3 built
// from (a, b, c) has those as rows, mul(M, v) = (a.v, b.v, c.v) and
// mul(v, M) = v.x a + v.y b + v.z c.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/yapt_fmath.h"

#define YG_HD __host__ __device__ __forceinline__

namespace yg
{

YG_HD float3 mk3(float x, float y, float z) { float3 r; r.x = x; r.y = y; r.z = z; return r; }
YG_HD float4 mk4(float x, float y, float z, float w) { float4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
YG_HD float3 xyz(const float4& v) { return mk3(v.x, v.y, v.z); }

YG_HD float3 operator+(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
YG_HD float3 operator-(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
YG_HD float3 operator-(float3 a) { return mk3(-a.x, -a.y, -a.z); }
YG_HD float3 operator*(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
YG_HD float3 operator*(float s, float3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
YG_HD float3 operator*(float3 a, float3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
YG_HD float3 operator/(float3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }

YG_HD float4 operator+(float4 a, float4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
YG_HD float4 operator-(float4 a, float4 b) { return mk4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
YG_HD float4 operator*(float4 a, float4 b) { return mk4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
YG_HD float4 operator/(float4 a, float4 b) { return mk4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
YG_HD float4 operator*(float4 a, float s) { return mk4(a.x * s, a.y * s, a.z * s, a.w * s); }
YG_HD float4 operator/(float4 a, float s) { return mk4(a.x / s, a.y / s, a.z / s, a.w / s); }
YG_HD float4 splat4(float s) { return mk4(s, s, s, s); }

YG_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
YG_HD float3 cross(float3 a, float3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
YG_HD float length(float3 v) { return sqrtf(dot(v, v)); }
YG_HD float3 normalize(float3 v)
{
    float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
YG_HD bool isZero3(float3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
YG_HD bool isZero4(float4 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f && v.w == 0.0f; }
YG_HD bool allEqual4(float4 v, float s) { return v.x == s && v.y == s && v.z == s && v.w == s; }
YG_HD float sqr(float x) { return x * x; }
YG_HD float saturate(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
YG_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
YG_HD float lerpf(float a, float b, float t) { return a + t * (b - a); }
YG_HD float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
YG_HD float safeDiv(float n, float d) { return d == 0.0f ? 0.0f : n / d; }
YG_HD float4 safeDiv4(float4 n, float d) { return d == 0.0f ? splat4(0.0f) : n / d; }
YG_HD float3 safeDiv3(float3 n, float d) { return d == 0.0f ? mk3(0.f, 0.f, 0.f) : n / d; }
YG_HD float lane(const float4& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w)); }
YG_HD void setLane(float4& v, int i, float s)
{
    if (i == 0) v.x = s; else if (i == 1) v.y = s; else if (i == 2) v.z = s; else v.w = s;
}
YG_HD float max4(float4 v) { return fmaxf(fmaxf(fmaxf(v.x, v.y), v.z), v.w); }

// HLSL reflect(i, n) = i - 2 dot(n, i) n
YG_HD float3 reflect3(float3 i, float3 n) { return i - n * (2.0f * dot(n, i)); }
// HLSL refract(i, n, eta): 0 on total internal reflection
YG_HD float3 refract3(float3 i, float3 n, float eta)
{
    float ni = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - ni * ni);
    if (k < 0.0f) return mk3(0.f, 0.f, 0.f);
    return i * eta - n * (eta * ni + sqrtf(k));
}

// 3x3 basis with rows t, n, b (constructBasisTransform, commonMath.hlsl:128-133)
struct Basis
{
    float3 t, n, b;
};
YG_HD float3 makeOrthogonal(float3 ortho, float3 v) { return normalize(v - ortho * dot(ortho, v)); }
YG_HD Basis constructBasis(float3 n, float3 t)
{
    Basis B;
    B.t = makeOrthogonal(n, t);
    B.n = n;
    B.b = cross(B.t, n);
    return B;
}
YG_HD float3 toLocal(const Basis& B, float3 v) { return mk3(dot(B.t, v), dot(B.n, v), dot(B.b, v)); }
YG_HD float3 fromLocal(const Basis& B, float3 v)
{
    return mk3(v.x * B.t.x + v.y * B.n.x + v.z * B.b.x,
               v.x * B.t.y + v.y * B.n.y + v.z * B.b.y,
               v.x * B.t.z + v.y * B.n.z + v.z * B.b.z);
}

// 3x4 row-major transform rows r[0..2]
YG_HD float3 xformPoint(const float4* r, float3 p)
{
    return mk3(r[0].x * p.x + r[0].y * p.y + r[0].z * p.z + r[0].w,
               r[1].x * p.x + r[1].y * p.y + r[1].z * p.z + r[1].w,
               r[2].x * p.x + r[2].y * p.y + r[2].z * p.z + r[2].w);
}
YG_HD float3 xformVector(const float4* r, float3 v)
{
    return mk3(r[0].x * v.x + r[0].y * v.y + r[0].z * v.z,
               r[1].x * v.x + r[1].y * v.y + r[1].z * v.z,
               r[2].x * v.x + r[2].y * v.y + r[2].z * v.z);
}
// v * M (row vector): transpose multiply, used for normals with the inverse matrix
YG_HD float3 xformVectorT(const float4* r, float3 v)
{
    return mk3(v.x * r[0].x + v.y * r[1].x + v.z * r[2].x,
               v.x * r[0].y + v.y * r[1].y + v.z * r[2].y,
               v.x * r[0].z + v.y * r[1].z + v.z * r[2].z);
}
// 4x4 row-major times (x, y, z, w)
YG_HD float4 mul44(const float* m, float4 v)
{
    return mk4(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w,
               m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * v.w,
               m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * v.w,
               m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15] * v.w);
}

} // namespace yg
