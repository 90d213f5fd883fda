// Principled spectral BSDF, spectral utilities and the Owen-scrambled Sobol sampler,
// restated for CUDA from YAPT's HLSL (Source/Renderer/shaders/...). Each function
// names the reference function and file:line it follows. All arithmetic is FP32.
#pragma once
#include "yg_types.h"
#include "yg_vec.cuh"

#define YG_DEV __device__ __forceinline__

namespace yg
{

constexpr float kPI = 3.14159265f;        // commonMath.hlsl:5
constexpr float kINVPI = 0.31830988f;     // commonMath.hlsl:6
constexpr float kPI_OVER_2 = 1.57079633f;
constexpr float kPI_OVER_4 = 0.785398163f;

// ------------------------------------------------------------------ sampler
// random.hlsl:35-92, randomSampler.hlsl:23-102
YG_HD uint32_t reverseBits(uint32_t v)
{
#if defined(__CUDA_ARCH__)
    return __brev(v);
#else
    v = ((v >> 1) & 0x55555555u) | ((v & 0x55555555u) << 1);
    v = ((v >> 2) & 0x33333333u) | ((v & 0x33333333u) << 2);
    v = ((v >> 4) & 0x0F0F0F0Fu) | ((v & 0x0F0F0F0Fu) << 4);
    v = ((v >> 8) & 0x00FF00FFu) | ((v & 0x00FF00FFu) << 8);
    return (v >> 16) | (v << 16);
#endif
}
YG_HD uint32_t finalizeHashMurmur(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}
// hash(a, b) with the reference's wrapping uint arithmetic (random.hlsl:50-54)
YG_HD uint32_t hash2(uint32_t a, uint32_t b)
{
    uint32_t key = ((a + b) * (a + b + 1u)) / (2u + b);
    return finalizeHashMurmur(key);
}
YG_HD uint32_t owenScrambleBase2Fast(uint32_t v, uint32_t seed)
{
    v = reverseBits(v);
    v ^= v * 0x3d20adeau;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526c56u;
    v ^= v * 0x53a22864u;
    return reverseBits(v);
}
// [0, 2^32) -> [0, 1) (random.hlsl:89-92)
YG_HD float uintToFloat01(uint32_t r)
{
    return fminf((float)r * 0x1p-32f, 0x1.fffffep-1f);
}
YG_HD float sampleDim(const uint32_t* point, uint32_t dim, uint32_t seed)
{
    // reads past the uploaded dimensions return 0, as a DX12 ByteAddressBuffer does
    uint32_t sob = dim < (uint32_t)kSobolDims ? point[dim] : 0u;
    return uintToFloat01(owenScrambleBase2Fast(sob, hash2(seed, dim)));
}

struct RandomSampler
{
    const uint32_t* point; // Sobol point (kSobolDims uint32) of this sample index
    uint32_t dim;
    uint32_t seed;
    YG_DEV float r1() { float v = sampleDim(point, dim, seed); dim += 1; return v; }
    YG_DEV float2 r2()
    {
        float2 v = make_float2(sampleDim(point, dim, seed), sampleDim(point, dim + 1, seed));
        dim += 2;
        return v;
    }
    YG_DEV float4 r4()
    {
        float4 v = mk4(sampleDim(point, dim, seed), sampleDim(point, dim + 1, seed),
                       sampleDim(point, dim + 2, seed), sampleDim(point, dim + 3, seed));
        dim += 4;
        return v;
    }
};

// ------------------------------------------------------------------ LUTs
// Explicit FP32 equivalents of sampleLUT with LINEAR_CLAMP and the texel-centre
// remap of materialsCommonResources.hlsl:132-169: coordinate u maps to texel u*(dim-1).
YG_HD void lutCoord(float u, int dim, int& i0, float& t)
{
    float x = clampf(u * (float)(dim - 1), 0.0f, (float)(dim - 1));
    int i = (int)x;
    if (i > dim - 2) i = dim - 2;
    i0 = i;
    t = x - (float)i;
}
YG_DEV float lut1(const float* L, int dim, float u)
{
    int i; float t;
    lutCoord(u, dim, i, t);
    return lerpf(__ldg(L + i), __ldg(L + i + 1), t);
}
YG_DEV float lut2(const float* L, int dx, int dy, float u, float v)
{
    int i, j; float tx, ty;
    lutCoord(u, dx, i, tx);
    lutCoord(v, dy, j, ty);
    const float* r0 = L + j * dx;
    const float* r1 = r0 + dx;
    float a = lerpf(__ldg(r0 + i), __ldg(r0 + i + 1), tx);
    float b = lerpf(__ldg(r1 + i), __ldg(r1 + i + 1), tx);
    return lerpf(a, b, ty);
}
YG_DEV float lut3(const float* L, int dx, int dy, int dz, float u, float v, float w)
{
    int k; float tz;
    lutCoord(w, dz, k, tz);
    float a = lut2(L + k * dx * dy, dx, dy, u, v);
    float b = lut2(L + (k + 1) * dx * dy, dx, dy, u, v);
    return lerpf(a, b, tz);
}

// ------------------------------------------------------------------ spectral
// spectralDistribution.hlsl:21-48
YG_DEV float4 getSpectralSampleLambdas(float hero, float lmin, float lmax)
{
    float step = (lmax - lmin) / 4.0f;
    float4 res;
    float prev = hero;
    res.x = prev;
    float l = prev + step; if (l > lmax) l = lmin + (l - lmax); prev = l; res.y = prev;
    l = prev + step; if (l > lmax) l = lmin + (l - lmax); prev = l; res.z = prev;
    l = prev + step; if (l > lmax) l = lmin + (l - lmax); prev = l; res.w = prev;
    return res;
}

struct Spectral
{
    float4 lambdas;
    float hero;
};

YG_DEV float4 cieAt(const SceneView& s, float lambda)
{
    float u = (lambda - s.lambdaMin) / (s.lambdaMax - s.lambdaMin);
    int i; float t;
    lutCoord(u, (int)s.cieN, i, t);
    float4 a = __ldg(s.cie + i);
    float4 b = __ldg(s.cie + i + 1);
    return mk4(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t), lerpf(a.w, b.w, t));
}

// sigmoid / sigmoidInv (spectralDistribution.hlsl:72-83)
YG_HD float sigmoidF(float x)
{
    if (isinf(x)) return x > 0.0f ? 1.0f : 0.0f;
    return 0.5f * x / sqrtf(1.0f + x * x) + 0.5f;
}
YG_HD float sigmoidInv(float x)
{
    if (x == 1.0f) return 1.0f / 0.0f;
    if (x == 0.0f) return -1.0f / 0.0f;
    return (x - 0.5f) / sqrtf(x * (1.0f - x));
}

// setWithPolynomialCoeffs (spectralDistribution.hlsl:204-217)
YG_DEV float4 spectrumFromCoeffs(const SceneView& s, const Spectral& sp, float3 c)
{
    float4 out;
    for (int i = 0; i < 4; ++i)
    {
        float lam = (lane(sp.lambdas, i) - s.lambdaMin) / (s.lambdaMax - s.lambdaMin);
        float poly = c.x * lam * lam + c.y * lam + c.z;
        setLane(out, i, sigmoidF(poly));
    }
    return out;
}

YG_DEV float3 rgbToSpdCoeffs(const SceneView& s, float3 rgb)
{
    // 64^3 trilinear lookup (getRGBToSPDCoeffs, spectralDistribution.hlsl:62-70), x = r fastest
    const int R = kRgbLutRes;
    int i, j, k; float tx, ty, tz;
    lutCoord(rgb.x, R, i, tx);
    lutCoord(rgb.y, R, j, ty);
    lutCoord(rgb.z, R, k, tz);
    float3 res;
    float* out = &res.x;
    for (int c = 0; c < 3; ++c)
    {
        const float* L = s.rgbToSpd;
        auto at = [&](int x, int y, int z) { return __ldg(L + ((size_t)((z * R + y) * R + x)) * 3 + c); };
        float a = lerpf(lerpf(at(i, j, k), at(i + 1, j, k), tx), lerpf(at(i, j + 1, k), at(i + 1, j + 1, k), tx), ty);
        float b = lerpf(lerpf(at(i, j, k + 1), at(i + 1, j, k + 1), tx), lerpf(at(i, j + 1, k + 1), at(i + 1, j + 1, k + 1), tx), ty);
        out[c] = lerpf(a, b, tz);
    }
    return res;
}

// setFromRGB (spectralDistribution.hlsl:183-202)
YG_DEV float4 fromRGB(const SceneView& s, const Spectral& sp, float3 v)
{
    float3 coeffs;
    if (v.x == v.y && v.x == v.z)
        coeffs = mk3(0.0f, 0.0f, sigmoidInv(v.x));
    else
        coeffs = s.rgbToSpd ? rgbToSpdCoeffs(s, v) : mk3(0.0f, 0.0f, sigmoidInv(v.y));
    return spectrumFromCoeffs(s, sp, coeffs);
}
// setFromRGBUnboundedNoIlluminant (spectralDistribution.hlsl:140-151)
YG_DEV float4 fromRGBUnboundedNoIllum(const SceneView& s, const Spectral& sp, float3 v)
{
    float m = fmaxf(fmaxf(v.x, v.y), v.z);
    float scale = 2.0f * m;
    return fromRGB(s, sp, safeDiv3(v, scale)) * scale;
}
// setFromRGBUnbounded (spectralDistribution.hlsl:153-181): times D65 * 100 / sum(D65)
YG_DEV float4 fromRGBUnbounded(const SceneView& s, const Spectral& sp, float3 v)
{
    float4 r = fromRGBUnboundedNoIllum(s, sp, v);
    for (int i = 0; i < 4; ++i)
    {
        float d65 = cieAt(s, lane(sp.lambdas, i)).w;
        setLane(r, i, lane(r, i) * (d65 * s.d65SumInv * 100.0f));
    }
    return r;
}
// tabulated curve (spectral extension): piecewise linear on a uniform grid
YG_DEV float4 fromCurve(const SceneView& s, const Spectral& sp, int curve)
{
    const float* c = s.spectra + (size_t)curve * s.specPoints;
    float4 r;
    for (int i = 0; i < 4; ++i)
    {
        float u = (lane(sp.lambdas, i) - s.specLmin) / (s.specLmax - s.specLmin);
        int k; float t;
        lutCoord(u, (int)s.specPoints, k, t);
        setLane(r, i, lerpf(__ldg(c + k), __ldg(c + k + 1), t));
    }
    return r;
}

// ToXYZ (spectralDistribution.hlsl:345-365)
YG_DEV float3 toXYZ(const SceneView& s, const Spectral& sp, float4 L)
{
    float pdf = 1.0f / (s.lambdaMax - s.lambdaMin);
    float k = safeDiv(s.cieYSumInv, pdf);
    float3 acc = mk3(0.f, 0.f, 0.f);
    for (int i = 0; i < 4; ++i)
    {
        float4 c = cieAt(s, lane(sp.lambdas, i));
        float li = lane(L, i);
        acc = acc + (mk3(li * c.x, li * c.y, li * c.z) * k);
    }
    return acc / 4.0f;
}

// applyRussianRoulette (spectralDistribution.hlsl:124-138): true = terminate
YG_DEV bool russianRoulette(float4& t, float rnd)
{
    float p = max4(t) / 1.0f;
    p = clampf(p, 0.05f, 1.0f);
    if (rnd > p) return true;
    t = t * (1.0f / p);
    return false;
}
YG_DEV void terminateSecondary(float4& w)
{
    w.x *= 4.0f;
    w.y = 0.0f; w.z = 0.0f; w.w = 0.0f;
}

// ------------------------------------------------------------------ math helpers
// commonMath.hlsl:30-64, miscBrdf.hlsl
YG_HD float jReflection(float3 wi, float3 wm) { return safeDiv(1.0f, 4.0f * saturate(dot(wi, wm))); }
YG_HD float jRefraction(float eta, float3 wo, float3 wm, float3 wi)
{
    float mo = dot(wo, wm);
    float mi = dot(wi, wm);
    float denom = sqr(mo / eta + mi);
    return safeDiv(fabsf(mi), denom);
}
YG_HD bool onSameHemisphere(float3 r, float3 d) { return r.y * d.y >= 0.0f; }
YG_HD float3 forceSameHemisphere(float3 r, float3 d) { return onSameHemisphere(r, d) ? d : -d; }
YG_HD float2 sampleConcentricDisk(float2 u)
{
    float2 sq = make_float2(2.0f * u.x - 1.0f, 2.0f * u.y - 1.0f);
    if (sq.x == 0.0f && sq.y == 0.0f) return make_float2(0.f, 0.f);
    float theta, r;
    if (fabsf(sq.x) > fabsf(sq.y)) { r = sq.x; theta = kPI_OVER_4 * (sq.y / sq.x); }
    else { r = sq.y; theta = kPI_OVER_2 - kPI_OVER_4 * (sq.x / sq.y); }
    float sn, cs;
    ygm_sincosf(theta, &sn, &cs);
    return make_float2(r * cs, r * sn);
}
YG_HD float3 sampleCosineWeightedHemisphere(float2 rnd)
{
    float y = sqrtf(1.0f - rnd.x);
    float r = sqrtf(rnd.x);
    float phi = 2.0f * kPI * rnd.y;
    float sn, cs;
    ygm_sincosf(phi, &sn, &cs);
    return mk3(r * cs, y, r * sn);
}
YG_HD float pdfCosineWeightedHemisphere(float d) { return saturate(d) * kINVPI; }
// evaluateEmissionProfile (miscBrdf.hlsl:124-130)
YG_HD float evaluateEmissionProfile(float dotIN, float exponent)
{
    float profile = exponent > 0.0f ? ygm_powf(fabsf(dotIN), exponent) : 1.0f;
    return (exponent + 2.0f) * 0.5f * profile;
}
// sheen (miscBrdf.hlsl:147-203)
YG_HD float GLSheen(float x, float a, float b, float c, float d, float e)
{
    return (a / (1.0f + b * ygm_powf(x, c))) + d * x + e;
}
YG_HD float GLambdaSheen(float roughness, float cosTheta)
{
    float t = 1.0f - roughness;
    t *= t;
    float a = lerpf(21.5473f, 25.3245f, t);
    float b = lerpf(3.82987f, 3.32435f, t);
    float c = lerpf(0.19823f, 0.16801f, t);
    float d = lerpf(-1.97760f, -1.27393f, t);
    float e = lerpf(-4.32054f, -4.85967f, t);
    float ex;
    if (cosTheta < 0.5f) ex = GLSheen(cosTheta, a, b, c, d, e);
    else ex = 2.0f * GLSheen(0.5f, a, b, c, d, e) - GLSheen(1.0f - cosTheta, a, b, c, d, e);
    return ygm_expf(ex);
}
YG_HD float DSheen(float3 wm, float r)
{
    float rInv = 1.0f / r;
    float sin2 = fmaxf(1.0f - wm.y * wm.y, 0.0001f);
    float v = (2.0f + rInv) * ygm_powf(sin2, rInv * 0.5f);
    return v / (2.0f * kPI);
}
YG_HD float GSheen(float3 wo, float3 wi, float r)
{
    return 1.0f / (1.0f + GLambdaSheen(r, wi.y) + GLambdaSheen(r, wo.y));
}

// ------------------------------------------------------------------ GGX (ggx.hlsl:11-122)
YG_HD float smithLambdaGGX(float3 d, float ax, float ay)
{
    float s = 1.0f + (d.x * d.x * (ax * ax) + d.z * d.z * (ay * ay)) / (d.y * d.y);
    return (sqrtf(s) - 1.0f) * 0.5f;
}
YG_HD float G1GGX(float3 wo, float3 wm, float ax, float ay)
{
    float lambda = smithLambdaGGX(wo, ax, ay);
    return (dot(wo, wm) >= 0.0f ? 1.0f : 0.0f) / (1.0f + lambda);
}
YG_HD float G2GGX(float3 wo, float3 wi, float3 wm, float ax, float ay)
{
    float li = smithLambdaGGX(wi, ax, ay);
    float lo = smithLambdaGGX(wo, ax, ay);
    return 1.0f / (1.0f + li + lo);
}
YG_HD float DGGX(float3 wm, float ax, float ay)
{
    float denom = sqr(wm.x / ax) + sqr(wm.z / ay) + sqr(wm.y);
    denom *= denom;
    denom *= ax * ay * kPI;
    return safeDiv(1.0f, denom);
}
// Heitz VNDF sampling with y up (ggx.hlsl:59-84)
YG_HD float3 sampleVisibleNormalsGGX(float3 wo, float ax, float ay, float u1, float u2)
{
    float3 Vh = normalize(mk3(ax * wo.x, ay * wo.z, wo.y));
    float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    float3 T1 = lensq > 0.0f ? mk3(-Vh.y, Vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : mk3(1.f, 0.f, 0.f);
    float3 T2 = cross(Vh, T1);
    float r = sqrtf(u1);
    float phi = 2.0f * kPI * u2;
    float sn, cs;
    ygm_sincosf(phi, &sn, &cs);
    float t1 = r * cs;
    float t2 = r * sn;
    float s = 0.5f * (1.0f + Vh.z);
    t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
    float3 Nh = T1 * t1 + T2 * t2 + Vh * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
    return normalize(mk3(ax * Nh.x, fmaxf(0.0f, Nh.z), ay * Nh.y));
}
YG_HD float DVGGX(float3 wo, float3 wm, float ax, float ay)
{
    float D = DGGX(wm, ax, ay);
    float G1 = G1GGX(wo, wm, ax, ay);
    return safeDiv(G1 * fabsf(dot(wo, wm)) * D, fabsf(wo.y));
}
YG_HD float3 sampleWMGGX(float3 wo, float ax, float ay, float u1, float u2)
{
    bool flip = wo.y < 0.0f;
    wo.y = fabsf(wo.y);
    float3 wh = sampleVisibleNormalsGGX(wo, ax, ay, u1, u2);
    if (flip)
    {
        wo.y = -wo.y;
        wh.y = -wh.y;
    }
    return forceSameHemisphere(wo, wh);
}
YG_HD float pdfWMGGX(float3 wo, float3 wm, float ax, float ay) { return DVGGX(wo, wm, ax, ay); }

// ------------------------------------------------------------------ Fresnel (fresnel.hlsl:8-78)
YG_HD float2 conductorNK2(float r, float g)
{
    float rc = clampf(r, 0.0f, 0.99f);
    float sq = sqrtf(rc);
    float n = g * ((1.0f - rc) / (1.0f + rc)) + (1.0f - g) * ((1.0f + sq) / (1.0f - sq));
    float nr = (n + 1.0f) * (n + 1.0f) * rc - (n - 1.0f) * (n - 1.0f);
    return make_float2(n, nr / (1.0f - rc));
}
YG_HD float fresnelDielectricConductor(float etaReal, float etaImg, float cosTheta)
{
    float c2 = cosTheta * cosTheta;
    float s2 = 1.0f - c2;
    float er2 = etaReal * etaReal;
    float ei2 = etaImg * etaImg;
    float t0 = er2 - ei2 - s2;
    float a2b2 = sqrtf(er2 * ei2 * 4.0f + t0 * t0);
    float t1 = a2b2 + c2;
    float a = sqrtf((a2b2 + t0) * 0.5f);
    float t2 = a * c2 * 2.0f;
    float rs = (t1 - t2) / (t1 + t2);
    float t3 = a2b2 + s2 * s2 * c2;
    float t4 = t2 * s2;
    float rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}
YG_HD float fresnelDielectricDielectric2(float eta, float cosTheta)
{
    float c = saturate(cosTheta);
    float temp = eta * eta + c * c - 1.0f;
    if (temp < 0.0f) return 1.0f;
    float g = sqrtf(temp);
    return 0.5f * sqr((g - c) / fmaxf(g + c, 0.00001f)) * (1.0f + sqr(((g + c) * c - 1.0f) / ((g - c) * c + 1.0f)));
}

// ------------------------------------------------------------------ delta tests (bsdfSample.hlsl:7-23)
YG_HD bool isDeltaGGX1(float r) { return r < 0.002f; }
YG_HD bool isDeltaGGX(float2 a2) { return isDeltaGGX1(fmaxf(a2.x, a2.y)); }
YG_HD bool isDeltaSheen(float r) { return r < 0.01f; }
YG_HD float2 calculateRoughnessParams(float roughness, float anisotropy)
{
    float a2 = roughness * roughness;
    return make_float2(clampf(a2 * (1.0f + anisotropy), 0.0f, 1.0f), clampf(a2 * (1.0f - anisotropy), 0.0f, 1.0f));
}

// ------------------------------------------------------------------ multiple scattering (multiScatter.hlsl)
struct Luts
{
    const float *ss, *ssAvg, *ssms, *ssmsAvg, *trD, *trL, *trAvgD, *trAvgL, *sheen;
};
YG_DEV float getAverageSSDirectionalAlbedoNoFresnel(const Luts& L, float r) { return lut1(L.ssAvg, kLutSS, r); }
YG_DEV float getSSDirectionalAlbedoNoFresnel(const Luts& L, float c, float r) { return lut2(L.ss, kLutSS, kLutSS, c, r); }
YG_DEV float getSSMSDirectionalAlbedo(const Luts& L, float eta, float c, float r)
{
    float e = saturate((eta - 1.0f) * 0.333333f);
    return lut3(L.ssms, kLutSSMS, kLutSSMS, kLutSSMS, c, r, e);
}
YG_DEV float getSSDirectionalAlbedoTranslucentLighter(const Luts& L, float eta, float c, float r)
{
    float e = saturate((eta - 0.3f) * (1.0f / 0.69f));
    return lut3(L.trL, kLutTrans, kLutTrans, kLutTrans, c, r, e);
}
YG_DEV float getSSDirectionalAlbedoTranslucentDenser(const Luts& L, float eta, float c, float r)
{
    float e = saturate((eta - 1.0f) * 0.333333f);
    return lut3(L.trD, kLutTrans, kLutTrans, kLutTrans, c, r, e);
}
YG_DEV float getSheenDirectionalAlbedo(const Luts& L, float c, float r)
{
    r = saturate(r - 0.07f);
    return lut2(L.sheen, kLutSheen, kLutSheen, c, r);
}
YG_DEV float getDirectionalAlbedoTranslucent(const Luts& L, float etaR, float d, float lr)
{
    if (etaR < 1.0f) return getSSDirectionalAlbedoTranslucentLighter(L, etaR, fabsf(d), lr);
    return getSSDirectionalAlbedoTranslucentDenser(L, etaR, fabsf(d), lr);
}
// Turquin energy compensation (the uni/NEE configuration, RECIPROCAL_MULTISCATTER off)
YG_DEV float getEnergyCompensation(const Luts& L, float fms, float dotWo, float dotWi, float lr, float ss)
{
    float dirWo = getSSDirectionalAlbedoNoFresnel(L, fabsf(fabsf(dotWo)), lr);
    float comp = fms * (1.0f - dirWo) / dirWo;
    return ss * comp;
}
YG_DEV float getEnergyRemainingAfterSpecular(const Luts& L, float etaR, float dotWo, float lr, float amount)
{
    return 1.0f - getSSMSDirectionalAlbedo(L, etaR, fabsf(dotWo), lr) * amount;
}
YG_DEV float getEnergyRemainingAfterSheen(const Luts& L, float dotWo, float lr, float amount)
{
    return 1.0f - getSheenDirectionalAlbedo(L, fabsf(dotWo), lr) * amount;
}
YG_DEV float getEnergyCompensationTranslucent(const Luts& L, float etaR, float dotWo, float lr, float ss)
{
    float dirWo = fmaxf(getDirectionalAlbedoTranslucent(L, etaR, fabsf(dotWo), lr), 0.1f);
    return (ss / dirWo) - ss;
}

// Kulla-Conty compensation and the reciprocal multiple-scattering terms
// (RECIPROCAL_MULTISCATTER, which BDPTCommon.hlsl:6 switches on for the bidirectional integrator)
YG_DEV float getAvgFresnel(float etaR)
{
    if (etaR < 1.0f) return 0.997118f + 0.1014f * etaR - 0.965241f * etaR * etaR - 0.130607f * etaR * etaR * etaR;
    return (etaR - 1.0f) / (4.08567f + 1.00071f * etaR);
}
YG_DEV float getAverageAlbedoTranslucent(const Luts& L, float etaR, float lr)
{
    if (etaR < 1.0f) return lut2(L.trAvgL, kLutTrans, kLutTrans, lr, saturate((etaR - 0.3f) * (1.0f / 0.69f)));
    return lut2(L.trAvgD, kLutTrans, kLutTrans, lr, saturate((etaR - 1.0f) * 0.333333f));
}
YG_DEV float getMsTransmissionRatio(const Luts& L, float etaR, float lr)
{
    float etaOut = fmaxf(etaR, 1.0f / etaR);
    float tOut = 1.0f - getAvgFresnel(etaOut);
    if (etaR >= 1.0f) return tOut;
    float eAvgOut = getAverageAlbedoTranslucent(L, etaOut, lr);
    float eAvgIn = getAverageAlbedoTranslucent(L, etaR, lr);
    return saturate(safeDiv(tOut * (1.0f - eAvgOut), etaOut * etaOut * (1.0f - eAvgIn)));
}
YG_DEV float getEnergyCompensationKulla(const Luts& L, float fms, float dotWo, float dotWi, float lr)
{
    float dWo = getSSDirectionalAlbedoNoFresnel(L, fabsf(dotWo), lr);
    float dWi = getSSDirectionalAlbedoNoFresnel(L, fabsf(dotWi), lr);
    float eAvg = getAverageSSDirectionalAlbedoNoFresnel(L, lr);
    float ems = safeDiv((1.0f - dWo) * (1.0f - dWi), (1.0f - eAvg) * kPI);
    return fms * ems;
}
YG_DEV float getEnergyCompensationTranslucentKulla(const Luts& L, float etaR, float dotWo, float dotWi, float lr)
{
    bool transmission = dotWo * dotWi < 0.0f;
    float ratioT = getMsTransmissionRatio(L, etaR, lr);
    float dWo, dWi, eAvg, ratio;
    if (transmission)
    {
        float etaInv = 1.0f / etaR;
        dWo = getDirectionalAlbedoTranslucent(L, etaR, dotWo, lr);
        dWi = getDirectionalAlbedoTranslucent(L, etaInv, dotWi, lr);
        eAvg = getAverageAlbedoTranslucent(L, etaInv, lr);
        ratio = ratioT;
    }
    else
    {
        dWo = getDirectionalAlbedoTranslucent(L, etaR, dotWo, lr);
        dWi = getDirectionalAlbedoTranslucent(L, etaR, dotWi, lr);
        eAvg = getAverageAlbedoTranslucent(L, etaR, lr);
        ratio = 1.0f - ratioT;
    }
    return ratio * safeDiv((1.0f - dWo) * (1.0f - dWi), (1.0f - eAvg) * kPI);
}
// getEnergyCompensation / getFmsDielectric / getEnergyCompensationTranslucent for either model
template <bool RECIP>
YG_DEV float energyComp(const Luts& L, float fms, float dotWo, float dotWi, float lr, float ss)
{
    if constexpr (RECIP) return getEnergyCompensationKulla(L, fms, fabsf(dotWo), fabsf(dotWi), lr);
    else return getEnergyCompensation(L, fms, fabsf(dotWo), fabsf(dotWi), lr, ss);
}
template <bool RECIP>
YG_DEV float fmsDielectric(const Luts& L, float etaR, float lr, float cosTheta)
{
    if constexpr (RECIP)
    {
        float fAvg = getAvgFresnel(etaR);
        float eAvg = getAverageSSDirectionalAlbedoNoFresnel(L, lr);
        return fAvg * eAvg / (1.0f - fAvg * (1.0f - eAvg));
    }
    else
    {
        return fresnelDielectricDielectric2(etaR, cosTheta);
    }
}
template <bool RECIP>
YG_DEV float energyCompTrans(const Luts& L, float etaR, float dotWo, float dotWi, float lr, float ss)
{
    if constexpr (RECIP) return getEnergyCompensationTranslucentKulla(L, etaR, dotWo, dotWi, lr);
    else return getEnergyCompensationTranslucent(L, etaR, dotWo, lr, ss);
}

// ------------------------------------------------------------------ lobes (bsdfSample.hlsl)
YG_DEV float3 sampleGGXReflectionConductor(float ax, float ay, float3 wo, float2 s)
{
    float3 wm = isDeltaGGX(make_float2(ax, ay)) ? mk3(0.f, 1.f, 0.f) : sampleWMGGX(wo, ax, ay, s.x, s.y);
    float3 wi = reflect3(-wo, wm);
    if (wi.y < 0.0f) return mk3(0.f, 0.f, 0.f);
    return wi;
}
YG_DEV float pdfGGXReflectionConductor(float3 wo, float3 wi, float ax, float ay)
{
    float3 wm = normalize(wo + wi);
    if (dot(wm, wo) < 0.0f) return 0.0f;
    if (isDeltaGGX(make_float2(ax, ay))) return 1.0f;
    return pdfWMGGX(wo, wm, ax, ay) * jReflection(wo, wm);
}
YG_DEV float3 sampleGGXReflectionDielectric(float ax, float ay, float3 wo, float2 s)
{
    float3 wm = isDeltaGGX(make_float2(ax, ay)) ? mk3(0.f, 1.f, 0.f) : sampleWMGGX(wo, ax, ay, s.x, s.y);
    float3 wi = reflect3(-wo, wm);
    if (!onSameHemisphere(wo, wi)) return mk3(0.f, 0.f, 0.f);
    return wi;
}
YG_DEV float pdfGGXReflectionDielectric(float3 wo, float3 wi, float ax, float ay)
{
    if (!onSameHemisphere(wo, wi)) return 0.0f;
    if (isDeltaGGX(make_float2(ax, ay))) return 1.0f;
    float3 wm = normalize(wo + wi);
    return pdfWMGGX(wo, wm, ax, ay) * jReflection(wo, wm);
}
YG_DEV float evaluateGGXReflectionDielectric(float etaR, float ax, float ay, float3 wo, float3 wi)
{
    float3 wm = normalize(wo + wi);
    if (!onSameHemisphere(wo, wi)) return 0.0f;
    if (dot(wi, wm) > 0.0f && dot(wo, wm) > 0.0f)
    {
        float F = fresnelDielectricDielectric2(etaR, dot(wo, wm));
        if (isDeltaGGX(make_float2(ax, ay))) return F / fabsf(wi.y);
        float D = DGGX(wm, ax, ay);
        float G2 = G2GGX(wo, wi, wm, ax, ay);
        return F * G2 * D / fmaxf(4.0f * wo.y * wi.y, 0.00001f);
    }
    return 0.0f;
}
YG_DEV float3 getWMTranslucent(float3 wo, float3 wi, float etaR)
{
    if (onSameHemisphere(wo, wi)) return normalize(wo + wi);
    if (etaR == 1.0f) etaR = 1.001f;
    float3 wm = normalize(wo + wi * etaR);
    return forceSameHemisphere(wo, wm);
}
YG_DEV float pdfGGXTransmitted(float etaR, float3 wo, float3 wi, float ax, float ay)
{
    if (etaR == 1.0f) etaR = 1.001f;
    float3 wm = getWMTranslucent(wo, wi, etaR);
    if (onSameHemisphere(wo, wi)) return 0.0f;
    if (isDeltaGGX(make_float2(ax, ay))) return 1.0f;
    float pdf = pdfWMGGX(wo, wm, ax, ay);
    if (dot(wo, wm) <= 0.0f || dot(wi, wm) >= 0.0f) return 0.0f;
    return pdf * jRefraction(etaR, wo, wm, wi);
}
YG_DEV float evaluateGGXTransmitted(float etaR, float ax, float ay, float3 wo, float3 wi)
{
    if (etaR == 1.0f) etaR = 1.001f;
    float3 wm = getWMTranslucent(wo, wi, etaR);
    if (onSameHemisphere(wo, wi)) return 0.0f;
    if (dot(wo, wm) <= 0.0f || dot(wi, wm) >= 0.0f) return 0.0f;
    float VdotH = fabsf(dot(wo, wm));
    float F = fresnelDielectricDielectric2(etaR, VdotH);
    if (isDeltaGGX(make_float2(ax, ay))) return (1.0f - F) / fabsf(wi.y);
    float G2 = G2GGX(wo, wi, wm, ax, ay);
    float D = DGGX(wm, ax, ay);
    float denom = fabsf(wo.y * wi.y);
    float w = (1.0f - F) * G2 * D * VdotH * jRefraction(etaR, wo, wm, wi);
    return safeDiv(w, denom);
}
YG_DEV float2 getReflAndRefrProbabilities(float etaR, float3 wo, float3 wm, bool allowRefl, bool allowTrans)
{
    float VdotH = saturate(dot(wo, wm));
    float refl = fresnelDielectricDielectric2(etaR, VdotH);
    float refr = 1.0f - refl;
    if (!allowRefl) refl = 0.0f;
    if (!allowTrans) refr = 0.0f;
    if (refl == 0.0f && refr == 0.0f) return make_float2(0.f, 0.f);
    float sum = refl + refr;
    return make_float2(safeDiv(refl, sum), safeDiv(refr, sum));
}
YG_DEV float3 sampleDielectric(float etaR, float ax, float ay, float3 wo, float2 s, float sc, bool allowRefl, bool allowTrans)
{
    float3 wm;
    if (isDeltaGGX(make_float2(ax, ay))) wm = wo.y < 0.0f ? mk3(0.f, -1.f, 0.f) : mk3(0.f, 1.f, 0.f);
    else wm = sampleWMGGX(wo, ax, ay, s.x, s.y);
    if (dot(wo, wm) < 0.0f) return mk3(0.f, 0.f, 0.f);
    if (etaR == 1.0f) etaR = 1.001f;
    float2 p = getReflAndRefrProbabilities(etaR, wo, wm, allowRefl, allowTrans);
    if (p.x == 0.0f && p.y == 0.0f) return mk3(0.f, 0.f, 0.f);
    if (sc < p.x || p.y == 0.0f)
    {
        float3 wi = reflect3(-wo, wm);
        if (!onSameHemisphere(wo, wi)) return mk3(0.f, 0.f, 0.f);
        return wi;
    }
    float3 wi = refract3(-wo, wm, 1.0f / etaR);
    if (onSameHemisphere(wo, wi)) return mk3(0.f, 0.f, 0.f);
    return wi;
}
YG_DEV float pdfDielectric(float etaR, float3 wo, float3 wi, float ax, float ay, bool allowRefl, bool allowTrans)
{
    float3 wm = getWMTranslucent(wo, wi, etaR);
    float2 p = getReflAndRefrProbabilities(etaR, wo, wm, allowRefl, allowTrans);
    if (onSameHemisphere(wo, wi)) return pdfGGXReflectionDielectric(wo, wi, ax, ay) * p.x;
    return pdfGGXTransmitted(etaR, wo, wi, ax, ay) * p.y;
}
YG_DEV float3 sampleDiffuseLambertian(float3 wo, float2 s)
{
    float3 wi = sampleCosineWeightedHemisphere(s);
    if (wi.y < 0.0f) return mk3(0.f, 0.f, 0.f);
    return wi;
}
YG_DEV float pdfDiffuseLambertian(float3 wi)
{
    if (wi.y < 0.0f) return 0.0f;
    return pdfCosineWeightedHemisphere(wi.y);
}
YG_DEV float3 sampleSheen(float r, float3 wo, float2 s)
{
    float3 wi = isDeltaSheen(r) ? reflect3(-wo, mk3(0.f, 1.f, 0.f)) : sampleCosineWeightedHemisphere(s);
    if (wi.y < 0.0f) return mk3(0.f, 0.f, 0.f);
    return wi;
}
YG_DEV float pdfSheen(float3 wi, float r)
{
    if (wi.y < 0.0f) return 0.0f;
    return isDeltaSheen(r) ? 1.0f : pdfCosineWeightedHemisphere(wi.y);
}
YG_DEV float4 evaluateSheen(float4 color, float r, float3 wo, float3 wi)
{
    if (wi.y < 0.0f) return splat4(0.0f);
    float3 wm = normalize(wo + wi);
    if (dot(wi, wm) > 0.0f && dot(wo, wm) > 0.0f)
    {
        if (isDeltaSheen(r)) return safeDiv4(color, fabsf(wi.y));
        float D = DSheen(wm, r);
        float G = GSheen(wo, wi, r);
        float DG = fabsf(safeDiv(D * G, 4.0f * wo.y * wi.y));
        return color * DG;
    }
    return splat4(0.0f);
}

// ------------------------------------------------------------------ layers (materialLayers.hlsl)
// SpecularLayer (materialLayers.hlsl:297-405), RECIPROCAL_MULTISCATTER off: no MS lobe
struct SpecularLayer
{
    float2 a2;
    float lr;
    float etaR;
    bool allowRefl, allowRefr;
};
// sampling probability of the cosine lobe that carries the Kulla-Conty multiple scattering
// (getMsSamplingProbability, materialLayers.hlsl:310-320); zero in the Turquin configuration
template <bool RECIP>
YG_DEV float specMsProbability(const Luts& L, const SpecularLayer& l, float3 wo)
{
    if constexpr (RECIP)
    {
        if (!l.allowRefr || isDeltaGGX(l.a2)) return 0.0f;
        return saturate(1.0f - getDirectionalAlbedoTranslucent(L, l.etaR, wo.y, l.lr));
    }
    else
    {
        return 0.0f;
    }
}
template <bool RECIP = false>
YG_DEV float3 specSampleWi(const Luts& L, const SpecularLayer& l, float3 wo, float2 rnd, float sel)
{
    float msProb = specMsProbability<RECIP>(L, l, wo);
    if (sel < msProb)
    {
        float sc = sel / msProb;
        float3 wi = sampleCosineWeightedHemisphere(rnd);
        float refrSel = l.allowRefl ? getMsTransmissionRatio(L, l.etaR, l.lr) : 1.0f;
        bool msRefract = sc < refrSel;
        wi.y = ((wo.y < 0.0f) != msRefract) ? -wi.y : wi.y;
        return wi;
    }
    float fsel = (sel - msProb) / (1.0f - msProb);
    return sampleDielectric(l.etaR, l.a2.x, l.a2.y, wo, rnd, fsel, l.allowRefl, l.allowRefr);
}
template <bool RECIP = false>
YG_DEV float specEvaluate(const Luts& L, const SpecularLayer& l, float3 wo, float3 wi)
{
    if (onSameHemisphere(wo, wi))
    {
        float w = evaluateGGXReflectionDielectric(l.etaR, l.a2.x, l.a2.y, wo, wi);
        float ms;
        if (l.allowRefl && l.allowRefr)
        {
            ms = energyCompTrans<RECIP>(L, l.etaR, wo.y, wi.y, l.lr, w);
        }
        else
        {
            float3 wm = normalize(wo + wi);
            float fms = fmsDielectric<RECIP>(L, l.etaR, l.lr, fabsf(dot(wo, wm)));
            ms = energyComp<RECIP>(L, fms, fabsf(wo.y), fabsf(wi.y), l.lr, w);
        }
        w += ms;
        w *= fabsf(wi.y);
        return w;
    }
    float w = evaluateGGXTransmitted(l.etaR, l.a2.x, l.a2.y, wo, wi);
    float ms = energyCompTrans<RECIP>(L, l.etaR, wo.y, wi.y, l.lr, w);
    w += ms;
    w *= fabsf(wi.y);
    return w;
}
template <bool RECIP = false>
YG_DEV float specPdf(const Luts& L, const SpecularLayer& l, float3 wo, float3 wi)
{
    float pdfSS = pdfDielectric(l.etaR, wo, wi, l.a2.x, l.a2.y, l.allowRefl, l.allowRefr);
    float msProb = specMsProbability<RECIP>(L, l, wo);
    if (msProb == 0.0f) return pdfSS;
    float refrSel = l.allowRefl ? getMsTransmissionRatio(L, l.etaR, l.lr) : 1.0f;
    float pdfMS = pdfCosineWeightedHemisphere(fabsf(wi.y)) * (onSameHemisphere(wo, wi) ? 1.0f - refrSel : refrSel);
    return lerpf(pdfSS, pdfMS, msProb);
}
YG_DEV float specEnergyLeft(const Luts& L, const SpecularLayer& l, float3 wo, float3 wi, float weight)
{
    if (onSameHemisphere(wo, wi)) return getEnergyRemainingAfterSpecular(L, l.etaR, wo.y, l.lr, weight);
    return 0.0f;
}

// ------------------------------------------------------------------ surface
// SurfaceDefinition (hitShadersCommon.hlsl:13-47) after the RGB -> spectral conversion
struct Surface
{
    float4 specular, albedo, absorption, emissive, sheenColor;
    float3 coatingLayerNormal, baseLayerNormal, geometryNormal, tangent;
    float transparency, metalness, dielectricIOR, roughness;
    float cauchyA, cauchyB, specularAmount, clearCoatAmount;
    float clearCoatIOR, clearCoatRoughness, anisotropy, anisotropyRotation;
    float thinFilmNM, sheenRoughness, sheenAmount, emissionFocus;
    float subsurfaceAmount;
    float occlusion; // unpackOcclusion of the ORM texture's occlusion, diffuse = specular (1 without one)
    uint32_t flags;
    float4 subsurfaceRadius; // diffuse mean free path per lane (world units); set when subsurfaceAmount > 0
};

constexpr int LAYER_COAT = 0, LAYER_SHEEN = 1, LAYER_COND = 2, LAYER_DIEL = 3, LAYER_DIFF = 4, LAYER_SSS = 5;
constexpr int LAYER_COUNT = 6;

// PrecalculatedSurfaceData + sampling probabilities (materialSample.hlsl:26-49, 564-611)
struct SurfaceCtx
{
    Basis coatB, baseB;
    float3 woBase, woCoating;
    float fromIOR, toIOR;
    float2 a2;
    bool exiting;
    float probs[LAYER_COUNT];
};

YG_DEV bool isTwoSided(uint32_t f) { return (f & 1u) != 0; }
YG_DEV bool hasDispersion(uint32_t f) { return (f & 2u) != 0; }

// isDeltaDistribution (materialsCommon.hlsl:65-80)
YG_DEV bool isDeltaDistribution(float2 a2, const Surface& s)
{
    if (s.metalness == 1.0f || s.transparency == 1.0f)
    {
        bool coatRough = (s.clearCoatAmount > 0.0f && !isDeltaGGX1(s.clearCoatRoughness)) ||
                         (s.sheenAmount > 0.0f && !isDeltaSheen(s.sheenRoughness));
        bool baseRough = !isDeltaGGX(a2);
        return !coatRough && !baseRough;
    }
    return false;
}

YG_DEV float cauchyIOR(const Surface& s, float lambdaNM)
{
    float um = lambdaNM * 0.001f;
    return s.cauchyA + (s.cauchyB / (um * um));
}

YG_DEV void makeSurfaceCtx(const Surface& s, float currentIOR, float previousIOR, float3 woOS, bool frontFace, SurfaceCtx& c)
{
    c.a2 = calculateRoughnessParams(s.roughness, s.anisotropy);
    c.exiting = !frontFace;
    c.fromIOR = currentIOR;
    c.toIOR = c.exiting ? previousIOR : s.dielectricIOR;
    c.coatB = constructBasis(s.coatingLayerNormal, s.tangent);
    c.baseB = constructBasis(s.baseLayerNormal, s.tangent);
    c.woCoating = normalize(toLocal(c.coatB, woOS));
    c.woBase = normalize(toLocal(c.baseB, woOS));
    // calculateNormalizedMaterialLayerSamplingProbabilities (materialSample.hlsl:89-127)
    float inside = c.woBase.y < 0.0f ? 0.0f : 1.0f;
    float diel = 1.0f - s.metalness;
    float opaqueDiel = diel * (1.0f - s.transparency);
    float sum = 0.0f;
    c.probs[LAYER_COAT] = s.clearCoatAmount * inside; sum += c.probs[LAYER_COAT];
    c.probs[LAYER_SHEEN] = s.sheenAmount * inside; sum += c.probs[LAYER_SHEEN];
    c.probs[LAYER_COND] = s.metalness * inside; sum += c.probs[LAYER_COND];
    c.probs[LAYER_DIEL] = diel * (s.specularAmount + s.transparency); sum += c.probs[LAYER_DIEL];
    c.probs[LAYER_DIFF] = opaqueDiel * (1.0f - s.subsurfaceAmount) * inside; sum += c.probs[LAYER_DIFF];
    c.probs[LAYER_SSS] = opaqueDiel * s.subsurfaceAmount * inside; sum += c.probs[LAYER_SSS];
    sum = fmaxf(0.000001f, sum);
    for (int i = 0; i < LAYER_COUNT; ++i) c.probs[i] /= sum;
}

YG_DEV int selectMaterialLayer(float rnd, const float* probs)
{
    float r = fmaxf(0.0f, rnd + 0.00001f);
    int layer;
    for (layer = 0; layer < LAYER_COUNT; ++layer)
    {
        if (r < probs[layer] && probs[layer] > 0.0f) break;
        r -= probs[layer];
    }
    return layer;
}

// getSampleDirectionOSForLayer (materialSample.hlsl:147-257)
template <bool RECIP = false>
YG_DEV float3 sampleLayerDirection(const Luts& L, const Surface& s, const SurfaceCtx& c, int layer, float selRnd, float2 rnd,
                                   float hero, bool& isDiffuse, bool& isDelta)
{
    float3 wi = mk3(0.f, 0.f, 0.f);
    bool allowTrans = s.transparency > 0.0f;
    float fromIOR = c.fromIOR, toIOR = c.toIOR;
    isDiffuse = false;
    isDelta = false;
    if (layer == LAYER_COAT)
    {
        if (c.woCoating.y > 0.0f)
        {
            float2 a2cc = calculateRoughnessParams(s.clearCoatRoughness, 0.0f);
            wi = sampleGGXReflectionDielectric(a2cc.x, a2cc.y, c.woCoating, rnd);
            wi = fromLocal(c.coatB, wi);
            isDiffuse = fminf(a2cc.x, a2cc.y) > 0.05f;
            isDelta = isDeltaGGX(a2cc);
        }
    }
    else if (layer == LAYER_SHEEN)
    {
        if (c.woBase.y > 0.0f)
        {
            wi = sampleSheen(s.sheenRoughness, c.woBase, rnd);
            wi = fromLocal(c.baseB, wi);
            isDiffuse = s.sheenRoughness > 0.15f;
            isDelta = isDeltaSheen(s.sheenRoughness);
        }
    }
    else if (layer == LAYER_COND)
    {
        if (c.woBase.y > 0.0f)
        {
            wi = sampleGGXReflectionConductor(c.a2.x, c.a2.y, c.woBase, rnd);
            wi = fromLocal(c.baseB, wi);
            isDiffuse = fminf(c.a2.x, c.a2.y) > 0.05f;
            isDelta = isDeltaGGX(c.a2);
        }
    }
    else if (layer == LAYER_DIEL)
    {
        if (hasDispersion(s.flags))
        {
            if (c.exiting) fromIOR = cauchyIOR(s, hero);
            else toIOR = cauchyIOR(s, hero);
        }
        SpecularLayer sl;
        sl.a2 = c.a2; sl.lr = s.roughness; sl.etaR = toIOR / fromIOR;
        sl.allowRefl = s.specularAmount > 0.0f; sl.allowRefr = s.transparency > 0.0f;
        wi = specSampleWi<RECIP>(L, sl, c.woBase, rnd, selRnd);
        wi = fromLocal(c.baseB, wi);
        isDiffuse = fminf(c.a2.x, c.a2.y) > 0.05f;
        isDelta = isDeltaGGX(c.a2);
    }
    else if (layer == LAYER_DIFF)
    {
        if (c.woBase.y > 0.0f)
        {
            wi = sampleDiffuseLambertian(c.woBase, rnd);
            wi = fromLocal(c.baseB, wi);
            isDiffuse = true;
            isDelta = false;
        }
    }
    if (!allowTrans && dot(s.geometryNormal, wi) < 0.0f) wi = mk3(0.f, 0.f, 0.f);
    // REJECT_SHADING_GEOMETRY_FRAME_MISMATCH (materialSample.hlsl:236-250)
    if (allowTrans && layer == LAYER_DIEL && !isZero3(wi))
    {
        float3 woOS = fromLocal(c.baseB, c.woBase);
        bool transGeom = dot(woOS, s.geometryNormal) * dot(wi, s.geometryNormal) < 0.0f;
        bool transShading = c.woBase.y * dot(wi, c.baseB.n) < 0.0f;
        if (transGeom != transShading) wi = mk3(0.f, 0.f, 0.f);
    }
    return wi;
}

// thin film (materialsCommon.hlsl:515-568)
YG_DEV float4 applyThinFilm(float4 lambdas, float4 A1, float4 A2, float nFilm, float etaRTop, float phaseShift, float cosI, float thick)
{
    if (isZero4(A1)) return A2;
    if (isZero4(A2)) return A1;
    float4 m;
    if (thick > 1200.0f)
    {
        m = splat4(0.0f);
    }
    else
    {
        float cr2 = 1.0f - (1.0f - cosI * cosI) / (etaRTop * etaRTop);
        float opd = cr2 < 0.0f ? 0.0f : 2.0f * nFilm * thick * sqrtf(cr2);
        for (int i = 0; i < 4; ++i)
        {
            float mm = opd / lane(lambdas, i) + phaseShift;
            setLane(m, i, ygm_cosf(2.0f * mm * kPI));
        }
        float f = fmaxf(0.0f, thick - 1200.0f + 200.0f) * (1.0f / 200.0f);
        m = m + (splat4(0.0f) - m) * f;
    }
    float4 r;
    for (int i = 0; i < 4; ++i)
    {
        float a1 = lane(A1, i), a2 = lane(A2, i);
        setLane(r, i, fmaxf(0.0f, a1 + a2 + 2.0f * sqrtf(fmaxf(0.0f, a1 * a2)) * lane(m, i)));
    }
    return r;
}

struct Eval
{
    float4 weight;
    float pdf;
    uint32_t transmission; // bit0 entered, bit1 exited, bit2 dispersed
};
constexpr uint32_t kTransEntered = 1, kTransExited = 2, kTransDispersed = 4;
constexpr uint32_t kEvalNone = 1, kEvalPdfOnly = 2, kEvalLightPath = 4, kEvalTreatAsDelta = 8;

// evaluateSurface (materialSample.hlsl:264-562). RECIP selects the multiple-scattering model
// of the bidirectional integrator; kEvalLightPath adds the shading-normal compensation of light
// subpaths and drops the camera-side solid-angle compression of refraction.
template <bool RECIP = false>
YG_DEV Eval evaluateSurface(const Luts& L, const Surface& s, const SurfaceCtx& c, float3 woOS, float3 wiOS, uint32_t flags,
                            const Spectral& sp)
{
    Eval res;
    float2 a2 = c.a2;
    float2 a2cc = calculateRoughnessParams(s.clearCoatRoughness, 0.0f);
    float3 woC = c.woCoating, woB = c.woBase;
    bool exiting = c.exiting;
    float fromIOR = c.fromIOR, toIOR = c.toIOR;
    float4 wsum = splat4(0.0f);
    float pdfSum = 0.0f;
    float3 wiC = normalize(toLocal(c.coatB, wiOS));
    float3 wiB = normalize(toLocal(c.baseB, wiOS));
    res.transmission = 0;
    bool onlyPDF = (flags & kEvalPdfOnly) != 0;
    bool treatAsDelta = (flags & kEvalTreatAsDelta) != 0;
    float dWoG = dot(woOS, s.geometryNormal);
    float dWiG = dot(wiOS, s.geometryNormal);
    bool baseRefl = dWoG * dWiG > 0.0f;
    bool baseRefr = dWoG * dWiG < 0.0f;
    float energyLeft = 1.0f, energyLayer = 1.0f;
    const bool lightPath = (flags & kEvalLightPath) != 0;
    // compensateForShadingNormal (materialSample.hlsl:259-262), light paths only
    const float compC = lightPath ? (fabsf(woC.y) * fabsf(dWiG)) / (fabsf(dWoG) * fabsf(wiC.y)) : 1.0f;
    const float compB = lightPath ? (fabsf(woB.y) * fabsf(dWiG)) / (fabsf(dWoG) * fabsf(wiB.y)) : 1.0f;
    float diel = 1.0f - s.metalness;
    float specAmount = diel * s.specularAmount;
    bool applyInference = s.thinFilmNM > 0.0f && s.clearCoatAmount > 0.0f && (s.metalness > 0.0f || specAmount > 0.0f);
    applyInference = applyInference && (isDeltaGGX(a2cc) == isDeltaGGX(a2));
    float4 coatAmp = splat4(0.0f);
    // coating: GGX clear coat (ReflectionDielectric) and sheen
    if (s.clearCoatAmount > 0.0f)
    {
        float etaR = s.clearCoatIOR / fromIOR;
        if (isDeltaGGX(a2cc) == treatAsDelta)
        {
            float pdf = onSameHemisphere(woC, wiC) ? (isDeltaGGX(a2cc) ? 1.0f : pdfWMGGX(woC, normalize(woC + wiC), a2cc.x, a2cc.y) * jReflection(woC, normalize(woC + wiC))) : 0.0f;
            bool coatRefl = dot(woOS, s.geometryNormal) * dot(wiOS, s.geometryNormal) > 0.0f;
            if (pdf > 0.0f && coatRefl)
            {
                if (!onlyPDF)
                {
                    float w = 0.0f;
                    if (onSameHemisphere(woC, wiC))
                    {
                        w = evaluateGGXReflectionDielectric(etaR, a2cc.x, a2cc.y, woC, wiC);
                        w *= fabsf(wiC.y);
                        float3 wm = normalize(woC + wiC);
                        float fms = fmsDielectric<RECIP>(L, etaR, s.clearCoatRoughness, fabsf(dot(woC, wm)));
                        w += energyComp<RECIP>(L, fms, fabsf(woC.y), fabsf(wiC.y), s.clearCoatRoughness, w);
                    }
                    float4 weight = splat4(w) * (s.clearCoatAmount * energyLeft) * compC * s.occlusion;
                    if (applyInference) coatAmp = weight;
                    else wsum = wsum + weight;
                }
                pdfSum += c.probs[LAYER_COAT] * pdf;
            }
        }
        energyLayer *= getEnergyRemainingAfterSpecular(L, etaR, woC.y, s.clearCoatRoughness, s.clearCoatAmount);
    }
    if (s.sheenAmount > 0.0f)
    {
        if (isDeltaSheen(s.sheenRoughness) == treatAsDelta)
        {
            float pdf = onSameHemisphere(woB, wiB) ? pdfSheen(wiB, s.sheenRoughness) : 0.0f;
            if (pdf > 0.0f && baseRefl)
            {
                if (!onlyPDF)
                {
                    float4 w = onSameHemisphere(woB, wiB) ? evaluateSheen(s.sheenColor, s.sheenRoughness, woB, wiB) * fabsf(wiB.y) : splat4(0.0f);
                    wsum = wsum + w * (s.sheenAmount * energyLeft) * compB * s.occlusion;
                }
                pdfSum += c.probs[LAYER_SHEEN] * pdf;
            }
        }
        energyLayer *= getEnergyRemainingAfterSheen(L, woB.y, s.sheenRoughness, s.sheenAmount);
    }
    energyLeft *= energyLayer;
    energyLayer = 1.0f;
    // conductor
    if (s.metalness > 0.0f)
    {
        if (isDeltaGGX(a2) == treatAsDelta)
        {
            float pdf = onSameHemisphere(woB, wiB) ? pdfGGXReflectionConductor(woB, wiB, a2.x, a2.y) : 0.0f;
            if (pdf > 0.0f && baseRefl)
            {
                if (!onlyPDF)
                {
                    float4 w = splat4(0.0f);
                    if (onSameHemisphere(woB, wiB))
                    {
                        float3 wm = normalize(woB + wiB);
                        bool delta = isDeltaGGX(a2);
                        float G2 = 0.f, D = 0.f, denom = 1.f;
                        if (!delta)
                        {
                            G2 = G2GGX(woB, wiB, wm, a2.x, a2.y);
                            D = DGGX(wm, a2.x, a2.y);
                            denom = fmaxf(4.0f * woB.y * wiB.y, 0.00001f);
                        }
                        float dOM = dot(woB, wm);
                        float dirWo = getSSDirectionalAlbedoNoFresnel(L, fabsf(woB.y), s.roughness);
                        for (int i = 0; i < 4; ++i)
                        {
                            float2 nk = conductorNK2(lane(s.albedo, i), lane(s.specular, i));
                            float er = nk.x / fromIOR;
                            float ek = sqrtf(nk.y) / fromIOR;
                            float F = fresnelDielectricConductor(er, ek, dOM);
                            float ss = delta ? F / fabsf(wiB.y) : F * G2 * D / denom;
                            // multiscatter: getFmsConductor = Fresnel, Turquin compensation
                            float fms = fresnelDielectricConductor(er, ek, dOM);
                            float ms;
                            if constexpr (RECIP) ms = getEnergyCompensationKulla(L, fms, fabsf(woB.y), fabsf(wiB.y), s.roughness);
                            else ms = ss * (fms * (1.0f - dirWo) / dirWo);
                            setLane(w, i, (ss + ms) * fabsf(wiB.y));
                        }
                    }
                    float4 weight = w * (s.metalness * energyLeft) * compB * s.occlusion;
                    if (applyInference)
                    {
                        float etaRC = s.clearCoatIOR / fromIOR;
                        float3 wm = normalize(woC + wiC);
                        float phase = etaRC > 1.0f ? 0.0f : 0.5f;
                        weight = applyThinFilm(sp.lambdas, coatAmp, weight, s.clearCoatIOR, etaRC, phase, dot(woC, wm), s.thinFilmNM);
                    }
                    wsum = wsum + weight;
                }
                pdfSum += c.probs[LAYER_COND] * pdf;
            }
        }
        energyLayer *= (1.0f - s.metalness);
    }
    // dielectric specular reflection
    if (specAmount > 0.0f && baseRefl)
    {
        if (hasDispersion(s.flags))
        {
            if (exiting) fromIOR = cauchyIOR(s, sp.hero);
            else toIOR = cauchyIOR(s, sp.hero);
        }
        SpecularLayer sl;
        sl.a2 = a2; sl.lr = s.roughness; sl.etaR = toIOR / fromIOR;
        sl.allowRefl = s.specularAmount > 0.0f; sl.allowRefr = s.transparency > 0.0f;
        if (isDeltaGGX(a2) == treatAsDelta)
        {
            float pdf = specPdf<RECIP>(L, sl, woB, wiB);
            if (pdf > 0.0f)
            {
                if (!onlyPDF)
                {
                    float4 weight = splat4(specEvaluate<RECIP>(L, sl, woB, wiB)) * (specAmount * energyLeft) * compB * s.occlusion;
                    if (applyInference)
                    {
                        float etaRC = s.clearCoatIOR / fromIOR;
                        float3 wm = normalize(woC + wiC);
                        float phase = ((etaRC > 1.0f) != (toIOR > s.clearCoatIOR)) ? 0.5f : 0.0f;
                        weight = applyThinFilm(sp.lambdas, coatAmp, weight, s.clearCoatIOR, etaRC, phase, dot(woC, wm), s.thinFilmNM);
                    }
                    wsum = wsum + weight;
                }
                pdfSum += c.probs[LAYER_DIEL] * pdf;
            }
        }
        energyLayer *= specEnergyLeft(L, sl, woB, wiB, specAmount);
    }
    energyLeft *= energyLayer;
    energyLayer = 1.0f;
    // diffuse
    float diffAmount = (1.0f - s.transparency) * diel * (1.0f - s.subsurfaceAmount);
    if (diffAmount > 0.0f && !treatAsDelta)
    {
        float pdf = onSameHemisphere(woB, wiB) ? pdfDiffuseLambertian(wiB) : 0.0f;
        if (pdf > 0.0f && baseRefl)
        {
            if (!onlyPDF)
            {
                float4 w = onSameHemisphere(woB, wiB) ? (s.albedo / kPI) * fabsf(wiB.y) : splat4(0.0f);
                wsum = wsum + w * (diffAmount * energyLeft) * compB * s.occlusion;
            }
            pdfSum += c.probs[LAYER_DIFF] * pdf;
        }
    }
    // specular transmission
    float transAmount = s.transparency * diel;
    if (transAmount > 0.0f && baseRefr && (isDeltaGGX(a2) == treatAsDelta))
    {
        if (hasDispersion(s.flags))
        {
            if (exiting) fromIOR = cauchyIOR(s, sp.hero);
            else toIOR = cauchyIOR(s, sp.hero);
            res.transmission |= kTransDispersed;
        }
        SpecularLayer sl;
        sl.a2 = a2; sl.lr = s.roughness; sl.etaR = toIOR / fromIOR;
        sl.allowRefl = s.specularAmount > 0.0f; sl.allowRefr = s.transparency > 0.0f;
        float pdf = specPdf<RECIP>(L, sl, woB, wiB);
        if (pdf > 0.0f)
        {
            pdfSum += c.probs[LAYER_DIEL] * pdf;
            bool twoSided = isTwoSided(s.flags);
            float compression = 1.0f;
            if (!twoSided)
            {
                if (!lightPath) compression *= sqr(1.0f / sl.etaR);
                res.transmission |= exiting ? kTransExited : kTransEntered;
            }
            else
            {
                res.transmission |= kTransEntered | kTransExited;
            }
            if (!onlyPDF)
            {
                wsum = wsum + splat4(specEvaluate<RECIP>(L, sl, woB, wiB)) * (transAmount * energyLeft) * compression * compB * s.occlusion;
            }
        }
    }
    res.pdf = pdfSum;
    res.weight = wsum;
    return res;
}

} // namespace yg
