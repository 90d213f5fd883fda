// Subsurface scattering: the Christensen-Burley diffusion profile as a separable BSSRDF,
// S(po, wo, pi, wi) = entry(po, wo) * Rd(|po - pi|) * Sw(pi, wi), restating
// raytracing/subsurface.hlsl:1-394 and the subsurface branch of scatteringSample.hlsl:30-77.
// A path that takes the subsurface layer at an entry point continues from an exit point found
// by probe rays against the same instance (King et al. 2013: an axis of the entry frame, a
// spectral lane's profile radius, up to eight hits chosen in proportion to the profile); the
// exit has a cosine lobe and its own light connection.
#pragma once
#include "yg_shading.cuh"

namespace yg
{

constexpr int kSssLanes = 4;              // SUBSURFACE_SPECTRAL_LANES
constexpr int kSssMaxProbeHits = 8;       // SUBSURFACE_MAX_PROBE_HITS
constexpr float kSssMinD = 1e-6f;         // SUBSURFACE_MIN_D
constexpr float kSssRMaxFactor = 20.7232658f; // SUBSURFACE_RMAX_FACTOR: 3 ln 1000

YG_DEV float burleyScale(float albedo)
{
    float x = fabsf(albedo - 0.8f);
    return 1.85f - albedo + 7.f * x * x * x;
}
YG_DEV float burleyD(float radius, float albedo) { return fmaxf(radius, kSssMinD) / burleyScale(albedo); }
YG_DEV float burleyRMax(float d) { return kSssRMaxFactor * d; }
// area density over the plane, (e^(-r/d) + e^(-r/(3d))) / (8 pi d r)
YG_DEV float burleyProfileArea(float r, float d)
{
    r = fmaxf(r, d * 1e-4f);
    return (ygm_expf(-r / d) + ygm_expf(-r / (3.f * d))) / (8.f * kPI * d * r);
}
// the radial density is (1/4) e^(-r/d)/d + (3/4) e^(-r/(3d))/(3d)
YG_DEV float burleySampleRadius(float u, float d)
{
    float scale = d;
    if (u < 0.25f)
    {
        u *= 4.f;
    }
    else
    {
        u = (u - 0.25f) / 0.75f;
        scale = 3.f * d;
    }
    return -scale * ygm_logf(fmaxf(1.f - u, 1e-7f));
}
YG_DEV float4 subsurfaceRd(const Surface& s, float distance)
{
    const float* al = &s.albedo.x;
    const float* ra = &s.subsurfaceRadius.x;
    float4 rd;
    float* o = &rd.x;
    for (int lane = 0; lane < kSssLanes; ++lane) o[lane] = al[lane] * burleyProfileArea(distance, burleyD(ra[lane], al[lane]));
    return rd;
}

// constructVectorBase (commonMath.hlsl:84-90)
YG_DEV void constructVectorBase(float3 v, float3& v2, float3& v3)
{
    if (fabsf(v.x) > fabsf(v.y)) v2 = mk3(-v.z, 0.0f, v.x) / sqrtf(v.x * v.x + v.z * v.z);
    else v2 = mk3(0.0f, v.z, -v.y) / sqrtf(v.y * v.y + v.z * v.z);
    v3 = cross(v, v2);
}
// probe axis k: 0 the normal (probability 1/2), 1 the tangent, 2 the bitangent (1/4 each)
YG_DEV void subsurfaceProbeFrame(float3 n, uint32_t axisIndex, float3& axis, float3& u, float3& v)
{
    float3 t, b;
    constructVectorBase(n, t, b);
    if (axisIndex == 0)
    {
        axis = n;
        u = t;
        v = b;
    }
    else if (axisIndex == 1)
    {
        axis = t;
        u = b;
        v = n;
    }
    else
    {
        axis = b;
        u = n;
        v = t;
    }
}
YG_DEV float subsurfaceAxisProbability(uint32_t axisIndex) { return axisIndex == 0 ? 0.5f : 0.25f; }

// area density of the exit point, over the three probe axes and the four lanes (one-sample MIS)
YG_DEV float pdfSubsurfaceExit(const Surface& s, float3 fromPos, float3 fromN, float3 toPos, float3 toN)
{
    const float* al = &s.albedo.x;
    const float* ra = &s.subsurfaceRadius.x;
    float3 d = toPos - fromPos;
    float pdf = 0.f;
    for (uint32_t axisIndex = 0; axisIndex < 3; ++axisIndex)
    {
        float3 axis, pu, pv;
        subsurfaceProbeFrame(fromN, axisIndex, axis, pu, pv);
        float du = dot(d, pu), dv = dot(d, pv);
        float rProj = sqrtf(du * du + dv * dv);
        float axisPdf = 0.f;
        for (int lane = 0; lane < kSssLanes; ++lane)
        {
            float dl = burleyD(ra[lane], al[lane]);
            if (rProj < burleyRMax(dl)) axisPdf += burleyProfileArea(rProj, dl);
        }
        pdf += subsurfaceAxisProbability(axisIndex) * (1.f / kSssLanes) * axisPdf * fabsf(dot(toN, axis));
    }
    return pdf;
}

// getSubsurfaceLayerWeight / getEnergyLeftForBaseLayer / getSubsurfaceEntryFactor
// (subsurface.hlsl:25-85): the share of the energy that reaches the diffuse base and goes under
YG_DEV float subsurfaceEntryFactor(const Luts& L, const Surface& s, const SurfaceCtx& c, float hero)
{
    float energyLeft = 1.f;
    float fromIOR = c.fromIOR, toIOR = c.toIOR;
    if (s.clearCoatAmount > 0.0f)
        energyLeft *= getEnergyRemainingAfterSpecular(L, s.clearCoatIOR / fromIOR, c.woCoating.y, s.clearCoatRoughness,
                                                      s.clearCoatAmount);
    if (s.sheenAmount > 0.0f) energyLeft *= getEnergyRemainingAfterSheen(L, c.woBase.y, s.sheenRoughness, s.sheenAmount);
    if (s.metalness > 0.0f) energyLeft *= 1.f - s.metalness;
    float specAmount = (1.f - s.metalness) * s.specularAmount;
    if (specAmount > 0.0f)
    {
        if (hasDispersion(s.flags))
        {
            if (c.exiting) fromIOR = cauchyIOR(s, hero);
            else toIOR = cauchyIOR(s, hero);
        }
        energyLeft *= getEnergyRemainingAfterSpecular(L, toIOR / fromIOR, c.woBase.y, s.roughness, specAmount);
    }
    float layer = (1.f - s.metalness) * (1.f - s.transparency) * s.subsurfaceAmount;
    return layer * energyLeft * s.occlusion;
}

// the exit lobe: cosine about the base normal, never to the inside of the geometry
YG_DEV float3 sampleSubsurfaceExitLobe(const Surface& s, const SurfaceCtx& c, float3 woOS, float2 rnd)
{
    float3 wi = fromLocal(c.baseB, sampleCosineWeightedHemisphere(rnd));
    if (dot(wi, s.geometryNormal) * dot(woOS, s.geometryNormal) <= 0.0f) return mk3(0.f, 0.f, 0.f);
    return wi;
}
YG_DEV void evaluateSubsurfaceExitLobe(const Surface& s, const SurfaceCtx& c, float3 woOS, float3 wiOS, uint32_t flags,
                                       float4& weight, float& pdf)
{
    weight = splat4(0.0f);
    pdf = 0.0f;
    float dWo = dot(woOS, s.geometryNormal), dWi = dot(wiOS, s.geometryNormal);
    if (dWo * dWi <= 0.0f) return;
    float3 wiB = normalize(toLocal(c.baseB, wiOS));
    if (wiB.y <= 0.0f) return;
    pdf = pdfCosineWeightedHemisphere(wiB.y);
    if ((flags & kEvalPdfOnly) == 0)
    {
        float cosine = (flags & kEvalLightPath) ? fabsf(dWi) : wiB.y;
        weight = splat4(kINVPI * cosine);
    }
}

// the entry point of a subsurface event, oriented to the side the path arrived from
struct SurfacePoint
{
    float3 pos, normal; // world space; normal on the outside
    uint32_t instance, prim;
    float b1, b2;
    bool front;
};
struct SubsurfaceExit
{
    SurfacePoint exit;
    float4 weight;      // Rd / (area pdf * probe-hit selection probability)
    float pdfPosition;  // area density of the exit point
};

} // namespace yg
