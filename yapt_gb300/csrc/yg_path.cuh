// Per-vertex path logic shared by the megakernel and the wavefront kernels: camera
// ray generation, surface setup, emitter hits with MIS, NEE light sampling (split
// into a shadow-ray request and its resolution) and BSDF sampling with Russian
// roulette. Restates, for CUDA, YAPT's DXR ray generation / closest-hit / miss shaders:
//   rayGenPrimaryRays.hlsl:10-145   (camera ray, bounce loop, Russian roulette, ToXYZ)
//   rayHitDefault.hlsl:36-585       (surface setup, emitter MIS, NEE, BSDF sampling)
//   rayMissEnvironment.hlsl:13-31   (environment)
//   lightSampling.hlsl:31-188, 360-370 (alias light pick, area light sampling)
//   hitShadersCommon.hlsl:138-222   (absorption, spawn offset, medium start)
// Each path's arithmetic is the same sequence whichever kernel runs it, so the
// wavefront and the megakernel give bit-identical samples.
#pragma once
#include "yg_shading.cuh"
#include <cuda_fp16.h>
#include "yg_subsurface.cuh"
#include "yg_trace.cuh"

namespace yg
{

constexpr uint32_t kFlagSecondaryTerminated = 1u << 0; // RAYSTATE_FLAGS_* (RayState.hlsl:4-6)
constexpr uint32_t kFlagRegularize = 1u << 1;
constexpr uint32_t kFlagDelta = 1u << 2;

struct PathState
{
    float4 throughput;
    float4 total;
    float3 origin;
    float3 dir;
    float pdfThisRay;
    uint32_t flags;
    uint32_t pathLength;
    uint32_t nVol;
    float volIOR[kMaxVolumes];
    float4 volAbs[kMaxVolumes];
    uint32_t volMat[kMaxVolumes];
};

// Payload volume stack (payload.hlsl:15-103)
YG_DEV float currentIOR(const PathState& p) { return p.nVol != 0 ? p.volIOR[p.nVol - 1] : 1.0f; }
YG_DEV float previousIOR(const PathState& p) { return p.nVol > 1 ? p.volIOR[p.nVol - 2] : 1.0f; }
YG_DEV void enteredVolume(PathState& p, float ior, float4 absorption, uint32_t mat)
{
    p.nVol = min(p.nVol + 1, (uint32_t)kMaxVolumes);
    p.volIOR[p.nVol - 1] = ior;
    p.volAbs[p.nVol - 1] = absorption;
    p.volMat[p.nVol - 1] = mat;
}
YG_DEV void exitedVolume(PathState& p, uint32_t mat)
{
    if (p.nVol == 0) return;
    int index = -1;
    for (int i = (int)p.nVol - 1; i >= 0; --i)
    {
        if (p.volMat[i] == mat) { index = i; break; }
    }
    if (index < 0) index = (int)p.nVol - 1;
    for (uint32_t i = (uint32_t)index; i + 1 < p.nVol; ++i)
    {
        p.volIOR[i] = p.volIOR[i + 1];
        p.volAbs[i] = p.volAbs[i + 1];
        p.volMat[i] = p.volMat[i + 1];
    }
    --p.nVol;
}

// spawnRayOrigin, Ray Tracing Gems ch. 6 (hitShadersCommon.hlsl:147-160)
YG_DEV float spawnComp(float p, float n, int oi)
{
    int so = p < 0.0f ? -oi : oi;
    float off = __int_as_float(__float_as_int(p) + so);
    return fabsf(p) < (1.0f / 32.0f) ? p + (1.0f / 65536.0f) * n : off;
}
YG_DEV float3 spawnRayOrigin(float3 p, float3 gn, float3 dir)
{
    float3 n = dot(dir, gn) < 0.0f ? -gn : gn;
    int ox = (int)(256.0f * n.x), oy = (int)(256.0f * n.y), oz = (int)(256.0f * n.z);
    return mk3(spawnComp(p.x, n.x, ox), spawnComp(p.y, n.y, oy), spawnComp(p.z, n.z, oz));
}

YG_DEV float weightMIS(float a, float b)
{
    float a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}
YG_DEV float areaToSolidAngle(float3 v, float3 n)
{
    float invD2 = 1.0f / dot(v, v);
    float absDot = fabsf(dot(n, v * sqrtf(invD2)));
    return 1.0f / (absDot * invD2);
}

struct TriGeom
{
    float3 p1, p2, p3;
    uint32_t i1, i2, i3;
};
YG_DEV TriGeom fetchTri(const SceneView& S, const GpuInstance& I, uint32_t prim)
{
    TriGeom g;
    const uint32_t* ix = S.indices + I.firstIndex + 3u * prim;
    g.i1 = __ldg(ix) + I.vertexBase;
    g.i2 = __ldg(ix + 1) + I.vertexBase;
    g.i3 = __ldg(ix + 2) + I.vertexBase;
    const float* P = S.positions;
    g.p1 = mk3(__ldg(P + 3 * g.i1), __ldg(P + 3 * g.i1 + 1), __ldg(P + 3 * g.i1 + 2));
    g.p2 = mk3(__ldg(P + 3 * g.i2), __ldg(P + 3 * g.i2 + 1), __ldg(P + 3 * g.i2 + 2));
    g.p3 = mk3(__ldg(P + 3 * g.i3), __ldg(P + 3 * g.i3 + 1), __ldg(P + 3 * g.i3 + 2));
    return g;
}
YG_DEV float3 interp3(const float* A, const TriGeom& g, float b0, float b1, float b2)
{
    float3 a = mk3(__ldg(A + 3 * g.i1), __ldg(A + 3 * g.i1 + 1), __ldg(A + 3 * g.i1 + 2));
    float3 b = mk3(__ldg(A + 3 * g.i2), __ldg(A + 3 * g.i2 + 1), __ldg(A + 3 * g.i2 + 2));
    float3 c = mk3(__ldg(A + 3 * g.i3), __ldg(A + 3 * g.i3 + 1), __ldg(A + 3 * g.i3 + 2));
    return a * b0 + b * b1 + c * b2;
}

// a scene texture, sampled as bilinearWrap does
YG_DEV float4 sampleTexture(const SceneView& S, int id, float2 uv)
{
    const GpuTexture T = S.textures[id];
    return bilinearWrap(T.texels, T.width, T.height, uv);
}

// fetchMeshUV, or (0.5, 0.5) for a mesh without texture coordinates (hitShadersCommon.hlsl:198)
YG_DEV float2 meshUV(const SceneView& S, const GpuInstance& I, const TriGeom& g, float b0, float b1, float b2)
{
    if (!I.hasUVs) return make_float2(0.5f, 0.5f);
    const float2 a = __ldg(S.uvs + g.i1), b = __ldg(S.uvs + g.i2), c = __ldg(S.uvs + g.i3);
    return make_float2(a.x * b0 + b.x * b1 + c.x * b2, a.y * b0 + b.y * b1 + c.y * b2);
}

YG_DEV float2 scaleUV(float2 uv, float sx, float sy) { return make_float2(uv.x * sx, uv.y * sy); }

// TextureCube.SampleLevel(LINEAR, dir, 0) on six square faces stacked in layer order +X, -X,
// +Y, -Y, +Z, -Z: the major axis picks the face and (sc, tc, ma) of the Vulkan cube map face
// selection table give s = (sc / |ma| + 1) / 2, t = (tc / |ma| + 1) / 2; then bilinear between
// texel centres in FP32, clamped to the face's edge texels (the hardware filters across the
// seam into the neighbouring face; here the outer half texel repeats the edge).
YG_DEV float4 sampleCube(const GpuTexture& T, float3 d)
{
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    uint32_t face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az)
    {
        face = d.x >= 0.0f ? 0u : 1u;
        sc = d.x >= 0.0f ? -d.z : d.z;
        tc = -d.y;
        ma = ax;
    }
    else if (ay >= az)
    {
        face = d.y >= 0.0f ? 2u : 3u;
        sc = d.x;
        tc = d.y >= 0.0f ? d.z : -d.z;
        ma = ay;
    }
    else
    {
        face = d.z >= 0.0f ? 4u : 5u;
        sc = d.z >= 0.0f ? d.x : -d.x;
        tc = -d.y;
        ma = az;
    }
    const float s = 0.5f * (sc / ma + 1.0f), t = 0.5f * (tc / ma + 1.0f);
    const int W = (int)T.width;
    const float x = s * (float)W - 0.5f, y = t * (float)W - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float tx = x - fx, ty = y - fy;
    const int xi = (int)fx, yi = (int)fy;
    const int x0 = min(max(xi, 0), W - 1), x1 = min(max(xi + 1, 0), W - 1);
    const int y0 = min(max(yi, 0), W - 1), y1 = min(max(yi + 1, 0), W - 1);
    const float4* F = T.texels + (size_t)face * W * W;
    const float4 c00 = __ldg(F + (size_t)y0 * W + x0), c10 = __ldg(F + (size_t)y0 * W + x1);
    const float4 c01 = __ldg(F + (size_t)y1 * W + x0), c11 = __ldg(F + (size_t)y1 * W + x1);
    const float sx = 1.0f - tx, sy = 1.0f - ty;
    return (c00 * sx + c10 * tx) * sy + (c01 * sx + c11 * tx) * ty;
}

// getSkyBoxColor (materialsCommonResources.hlsl:181-224): a cube map, a longitude-latitude
// texture (cartesianToSpherical, commonMath.hlsl:144-151) or, without one, |dir|; times the scale
YG_DEV __noinline__ float3 skyTexture(const SceneView& S, float3 dir, float scale)
{
    float3 v = normalize(dir);
    if (S.envCube)
    {
        const float4 c = sampleCube(S.textures[S.envTexture], v);
        return mk3(c.x * scale, c.y * scale, c.z * scale);
    }
    float theta = atan2f(v.z, v.x), phi = acosf(clampf(v.y, -1.0f, 1.0f));
    float4 c = sampleTexture(S, S.envTexture, make_float2(theta * kINVPI * 0.5f + 0.5f, phi * kINVPI));
    return mk3(c.x * scale, c.y * scale, c.z * scale);
}
YG_DEV float3 skyColor(const SceneView& S, float3 dir, float scale)
{
    if (S.envTexture < 0) return mk3(fabsf(dir.x) * scale, fabsf(dir.y) * scale, fabsf(dir.z) * scale);
    return skyTexture(S, dir, scale);
}

// Scalar material parameters before the spectral conversion (SurfaceDefinitionRGB)
struct SurfaceRGB
{
    float3 albedo, specular, absorption, emissive, sheenColor;
};

YG_DEV float4 rgbOrCurve(const SceneView& S, const Spectral& sp, float3 rgb, int curve)
{
    if (curve >= 0) return fromCurve(S, sp, curve);
    return fromRGB(S, sp, rgb);
}
YG_DEV float4 emissionSpectrum(const SceneView& S, const Spectral& sp, float3 rgb, int curve)
{
    if (curve >= 0) return fromCurve(S, sp, curve) * fmaxf(fmaxf(rgb.x, rgb.y), rgb.z);
    if (isZero3(rgb)) return splat4(0.0f);
    return fromRGBUnbounded(S, sp, rgb);
}

// regularize (materialsCommon.hlsl:399-418)
YG_DEV float regularizeR(float lr, bool squared)
{
    float r = squared ? lr * lr : lr;
    if (r < 0.3f)
    {
        r = clampf(r * 2.0f, 0.1f, 0.3f);
        return squared ? sqrtf(r) : r;
    }
    return lr;
}

struct HitSurface
{
    Surface s;
    float3 rayDirOS;
    uint32_t material;
    float3 albedoRGB; // first-hit features
};

// modifySurfaceMaterialParametersWithTextures (materialsCommon.hlsl:354-397), out of line so
// that untextured shading keeps its instruction footprint
YG_DEV __noinline__ void applyTextures(const SceneView& S, const GpuMaterial& M, const GpuInstance& I, const TriGeom& g,
                                       float b0, float b1, float b2, SurfaceRGB& rgb, Surface& s)
{
    const int4 tex = M.textures;
    const float2 uv = meshUV(S, I, g, b0, b1, b2);
    const float4 sa = M.albedoNormalScale, so = M.ormEmissiveScale;
    if (tex.x >= 0)
    {
        float4 a = sampleTexture(S, tex.x, scaleUV(uv, sa.x, sa.y));
        rgb.albedo = mk3(rgb.albedo.x * a.x, rgb.albedo.y * a.y, rgb.albedo.z * a.z);
        if (s.flags & 4u) s.transparency = 1.0f - a.w * (1.0f - s.transparency); // alpha blended
    }
    if (tex.y >= 0)
    {
        float4 t = sampleTexture(S, tex.y, scaleUV(uv, sa.z, sa.w));
        float3 n = normalize(mk3(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f));
        s.baseLayerNormal = fromLocal(constructBasis(s.baseLayerNormal, s.tangent), mk3(n.x, n.z, n.y));
    }
    if (tex.z >= 0)
    {
        float4 o = sampleTexture(S, tex.z, scaleUV(uv, so.x, so.y));
        // packOcclusion / unpackOcclusion: the occlusion travels as a half
        float occ = __half2float(__float2half_rn(o.x));
        s.occlusion = occ;
        s.roughness = s.roughness * o.y;
        s.metalness = s.metalness * o.z;
    }
    if (tex.w >= 0)
    {
        float4 e = sampleTexture(S, tex.w, scaleUV(uv, so.z, so.w));
        rgb.emissive = mk3(rgb.emissive.x * e.x, rgb.emissive.y * e.y, rgb.emissive.z * e.z);
    }
}

// modifySurfaceEmissionWithTexture (materialsCommon.hlsl:420-428) at a sampled light point
YG_DEV __noinline__ float3 emissionTextured(const SceneView& S, const GpuMaterial& M, const GpuInstance& I, const TriGeom& g,
                                           float b0, float b1, float b2, float3 erg)
{
    const float2 uv = meshUV(S, I, g, b0, b1, b2);
    float4 t = sampleTexture(S, M.textures.w, scaleUV(uv, M.ormEmissiveScale.z, M.ormEmissiveScale.w));
    return mk3(erg.x * t.x, erg.y * t.y, erg.z * t.z);
}

// fetch + fetchSurfaceMaterialParameters + two-sided orientation + tangent rotation +
// regularisation + RGB -> spectral conversion (rayHitDefault.hlsl:470-520)
YG_DEV void setupSurface(const SceneView& S, const LaunchParams& P, const Spectral& sp, const Hit& hit, const GpuInstance& I,
                         float3 rayDirWS, PathState& ps, HitSurface& hs, bool orient = true)
{
    TriGeom g = fetchTri(S, I, hit.prim);
    float b0 = 1.0f - hit.b1 - hit.b2;
    float3 gn = normalize(cross(g.p2 - g.p1, g.p3 - g.p1));
    float3 nrm = normalize(interp3(S.normals, g, b0, hit.b1, hit.b2));
    float3 tan = mk3(1.f, 0.f, 0.f);
    if (I.hasTangents)
    {
        float4 t1 = __ldg(S.tangents + g.i1), t2 = __ldg(S.tangents + g.i2), t3 = __ldg(S.tangents + g.i3);
        float3 a = mk3(t1.x * t1.w, t1.y * t1.w, t1.z * t1.w);
        float3 b = mk3(t2.x * t2.w, t2.y * t2.w, t2.z * t2.w);
        float3 c = mk3(t3.x * t3.w, t3.y * t3.w, t3.z * t3.w);
        tan = normalize(a * b0 + b * hit.b1 + c * hit.b2);
    }
    float3 rd = normalize(xformVector(I.w2o, rayDirWS));
    hs.rayDirOS = rd;
    hs.material = I.material;
    const GpuMaterial& M = S.materials[I.material];
    Surface& s = hs.s;
    float4 a_t = M.albedo_transparency, s_m = M.specular_metalness, ab_i = M.absorption_ior, e_r = M.emissive_roughness;
    float4 sc = M.specAmount_ccAmount_ccIOR_ccRough, sh = M.sheenColor_roughness;
    SurfaceRGB rgb;
    rgb.albedo = mk3(a_t.x, a_t.y, a_t.z);
    rgb.specular = mk3(s_m.x, s_m.y, s_m.z);
    rgb.absorption = mk3(ab_i.x, ab_i.y, ab_i.z);
    rgb.emissive = mk3(e_r.x, e_r.y, e_r.z);
    rgb.sheenColor = mk3(sh.x, sh.y, sh.z);
    s.transparency = a_t.w;
    s.metalness = s_m.w;
    s.dielectricIOR = ab_i.w;
    s.roughness = e_r.w;
    s.emissionFocus = M.emissionFocus;
    s.specularAmount = sc.x;
    s.clearCoatAmount = sc.y;
    s.clearCoatIOR = sc.z;
    s.clearCoatRoughness = sc.w;
    s.cauchyA = M.cauchyA;
    s.cauchyB = M.cauchyB;
    s.anisotropy = M.anisotropy;
    s.anisotropyRotation = M.anisotropyRotation;
    s.thinFilmNM = M.thinFilmNM;
    s.flags = M.mask;
    s.sheenRoughness = fmaxf(sh.w, 0.07f);
    s.sheenAmount = M.sheenAmount;
    s.subsurfaceAmount = M.subsurfaceRadius_amount.w;
    s.coatingLayerNormal = nrm;
    s.baseLayerNormal = nrm;
    s.geometryNormal = gn;
    s.tangent = tan;
    // handleTwoSidedMaterialOrientation (materialsCommon.hlsl:440-448), wo = -rayDir; light
    // subpath vertices evaluated for a connection keep their normals (BDPTCommon.hlsl:845-852)
    if (orient && s.transparency == 0.0f && isTwoSided(s.flags))
    {
        float3 wo = -rd;
        if (dot(wo, s.baseLayerNormal) < 0.0f) s.baseLayerNormal = -s.baseLayerNormal;
        if (dot(wo, s.coatingLayerNormal) < 0.0f) s.coatingLayerNormal = -s.coatingLayerNormal;
        if (dot(wo, s.geometryNormal) < 0.0f) s.geometryNormal = -s.geometryNormal;
    }
    // setupSurfaceOrientation (materialsCommon.hlsl:487-501)
    if (s.anisotropyRotation > 0.0f)
    {
        float ang = s.anisotropyRotation * 2.0f * kPI;
        float sa, ca;
        ygm_sincosf(ang, &sa, &ca);
        float3 t = s.tangent;
        s.tangent = mk3(ca * t.x + 0.0f * t.y + sa * t.z, 0.0f * t.x + 1.0f * t.y + 0.0f * t.z, -sa * t.x + 0.0f * t.y + ca * t.z);
    }
    // modifySurfaceMaterialParametersWithTextures (materialsCommon.hlsl:354-397)
    s.occlusion = 1.0f;
    if (M.mask & kMaterialTextured)
    {
        // the out-of-line call works on copies, so that the surface itself never has its
        // address taken
        SurfaceRGB rgbX = rgb;
        Surface sX = s;
        applyTextures(S, M, I, g, b0, hit.b1, hit.b2, rgbX, sX);
        rgb = rgbX;
        s = sX;
    }
    // regularisation (rayHitDefault.hlsl:494-502)
    if (P.regularizeEnable)
    {
        if (ps.pathLength >= P.regularizeAfter) ps.flags |= kFlagRegularize;
        if (ps.flags & kFlagRegularize)
        {
            s.roughness = regularizeR(s.roughness, true);
            s.sheenRoughness = regularizeR(s.sheenRoughness, false);
            s.clearCoatRoughness = regularizeR(s.clearCoatRoughness, true);
        }
    }
    hs.albedoRGB = rgb.albedo;
    // convertSurfaceDefinitionFromRGB (hitShadersCommon.hlsl:51-91)
    s.specular = rgbOrCurve(S, sp, rgb.specular, M.specularSpectrum);
    s.albedo = rgbOrCurve(S, sp, rgb.albedo, M.albedoSpectrum);
    s.absorption = isZero3(rgb.absorption) ? splat4(0.0f) : fromRGBUnboundedNoIllum(S, sp, rgb.absorption);
    s.emissive = emissionSpectrum(S, sp, rgb.emissive, M.emissionSpectrum);
    s.sheenColor = s.sheenAmount > 0.0f ? fromRGB(S, sp, rgb.sheenColor) : splat4(0.0f);
    // distances, not limited to [0, 1] (setFromRGBUnboundedNoIlluminant)
    const float4 sr = M.subsurfaceRadius_amount;
    s.subsurfaceRadius = s.subsurfaceAmount > 0.0f ? fromRGBUnboundedNoIllum(S, sp, mk3(sr.x, sr.y, sr.z)) : splat4(0.0f);
}

// sampleLight for mesh lights (lightSampling.hlsl:122-188), position part only
struct LightPoint
{
    float4 radiance;
    float3 pos, n;
    float pdfPos, focus;
    uint32_t instance, prim;
    bool twoSided;
};
YG_DEV void sampleMeshLight(const SceneView& S, const Spectral& sp, uint32_t li, float3 r, LightPoint& out)
{
    const uint32_t inst = S.lights[li].instance;
    const GpuInstance& I = S.instances[inst];
    uint32_t primCount = I.primCount;
    uint32_t prim = (uint32_t)fminf((float)primCount * r.z, (float)(primCount - 1u));
    float bx = r.x, by = r.y;
    if (bx + by > 1.0f)
    {
        bx = 1.0f - bx;
        by = 1.0f - by;
    }
    float b0 = 1.0f - bx - by;
    TriGeom g = fetchTri(S, I, prim);
    float3 p1 = xformPoint(I.o2w, g.p1), p2 = xformPoint(I.o2w, g.p2), p3 = xformPoint(I.o2w, g.p3);
    float3 gn = cross(p2 - p1, p3 - p1);
    float len = length(gn);
    gn = gn / len;
    float area = len * 0.5f;
    out.pos = p1 * b0 + p2 * bx + p3 * by;
    out.n = gn;
    const GpuMaterial& M = S.materials[I.material];
    float4 e = M.emissive_roughness;
    float3 erg = mk3(e.x, e.y, e.z);
    if (M.textures.w >= 0) erg = emissionTextured(S, M, I, g, b0, bx, by, erg);
    out.radiance = emissionSpectrum(S, sp, erg, M.emissionSpectrum);
    out.pdfPos = 1.0f / ((float)primCount * area);
    out.focus = M.emissionFocus;
    out.instance = inst;
    out.prim = prim;
    out.twoSided = (M.mask & 1u) != 0;
}

YG_DEV uint32_t sampleLightIndex(const SceneView& S, float u)
{
    float scaled = u * (float)S.nLights;
    uint32_t index = min((uint32_t)scaled, S.nLights - 1u);
    const GpuLight& e = S.lights[index];
    return (scaled - (float)index) < e.aliasThreshold ? index : e.aliasIndex;
}

// samplePunctualLightIndex (lightSampling.hlsl:46-53): the alias table over the punctual lights
YG_DEV uint32_t samplePunctualLightIndex(const SceneView& S, float u)
{
    const uint32_t first = S.nLights - S.nPunctual;
    float scaled = u * (float)S.nPunctual;
    uint32_t index = min((uint32_t)scaled, S.nPunctual - 1u);
    const GpuLight& e = S.lights[first + index];
    return first + ((scaled - (float)index) < e.punctualAliasThreshold ? index : e.punctualAliasIndex);
}

// spotFalloff + punctualLightAngularFalloff (lightSampling.hlsl:228-246)
YG_DEV float punctualFalloff(const GpuLight& L, float3 dirFromLight)
{
    if (L.type != kLightSpot) return 1.0f;
    float cosTheta = dot(dirFromLight, mk3(L.directionCosOuter.x, L.directionCosOuter.y, L.directionCosOuter.z));
    float cosInner = L.positionCosInner.w, cosOuter = L.directionCosOuter.w;
    if (cosInner <= cosOuter) return cosTheta >= cosOuter ? 1.0f : 0.0f;
    float t = saturate((cosTheta - cosOuter) / (cosInner - cosOuter));
    return t * t * (3.0f - 2.0f * t); // smoothstep
}

// calculateExplicitLightConnectionPDF (rayHitDefault.hlsl:137-166)
YG_DEV float explicitLightPdf(const SceneView& S, float3 fromTo, uint32_t inst, uint32_t prim)
{
    const GpuInstance& I = S.instances[inst];
    TriGeom g = fetchTri(S, I, prim);
    float3 p1 = xformPoint(I.o2w, g.p1), p2 = xformPoint(I.o2w, g.p2), p3 = xformPoint(I.o2w, g.p3);
    float3 gn = cross(p2 - p1, p3 - p1);
    float len = length(gn);
    gn = gn / len;
    float area = len * 0.5f;
    float posPdf = 1.0f / ((float)I.primCount * area);
    return posPdf * I.lightPdf * areaToSolidAngle(fromTo, gn);
}

struct TraceStats
{
    uint32_t rays;
    TraversalCount tc;
};


// NEE connection prepared at a vertex: the shadow ray and the contribution it adds
// to the path total when the sampled light point is visible (connectToExplicitLight,
// rayHitDefault.hlsl:204-257, with the visibility test deferred).
struct ShadowRequest
{
    float3 origin, dir;
    float tmax;
    uint32_t instance, prim;
    float4 contrib;
    bool valid;
};

// sampleSubsurfaceExit (subsurface.hlsl:212-337)
YG_DEV bool sampleSubsurfaceExit(const SceneView& S, const Surface& s, const SurfacePoint& entry, float3 rnd,
                                 SubsurfaceExit& out)
{
    float u = rnd.x;
    uint32_t axisIndex;
    if (u < 0.5f)
    {
        axisIndex = 0;
        u *= 2.f;
    }
    else if (u < 0.75f)
    {
        axisIndex = 1;
        u = (u - 0.5f) * 4.f;
    }
    else
    {
        axisIndex = 2;
        u = (u - 0.75f) * 4.f;
    }
    uint32_t lane = min((uint32_t)(u * kSssLanes), (uint32_t)kSssLanes - 1u);
    float uSelect = saturate(u * kSssLanes - (float)lane);
    const float dLane = burleyD((&s.subsurfaceRadius.x)[lane], (&s.albedo.x)[lane]);
    const float rMax = burleyRMax(dLane);
    const float r = burleySampleRadius(rnd.y, dLane);
    if (r >= rMax) return false;
    float3 axis, pu, pv;
    subsurfaceProbeFrame(entry.normal, axisIndex, axis, pu, pv);
    float sinPhi, cosPhi;
    ygm_sincosf(2.f * kPI * rnd.z, &sinPhi, &cosPhi);
    // chord of the r_max sphere through the disk point, with a minimum length
    const float3 ep = entry.pos;
    const float maxCoord = fmaxf(fmaxf(fabsf(ep.x), fabsf(ep.y)), fabsf(ep.z));
    const float halfLength = fmaxf(sqrtf(rMax * rMax - r * r), 1e-3f + 1e-5f * maxCoord);
    const float3 probeOrigin = ep + (pu * cosPhi + pv * sinPhi) * r - axis * halfLength;
    float weightSum = 0.f, selectedWeight = 0.f;
    float4 selectedRd = splat4(0.0f);
    Hit sel;
    sel.t = 0.f;
    sel.b1 = sel.b2 = 0.f;
    sel.instance = entry.instance;
    sel.prim = 0;
    sel.front = false;
    float tMin = 0.f;
    for (int i = 0; i < kSssMaxProbeHits; ++i)
    {
        Hit h;
        if (!traceInstanceClosest(S, probeOrigin, axis, tMin, 2.f * halfLength, entry.instance, h)) break;
        // keep the k-th hit with probability w_k / (w_1 + ... + w_k)
        const float4 rd = subsurfaceRd(s, length(probeOrigin + axis * h.t - ep));
        const float w = rd.x + rd.y + rd.z + rd.w;
        weightSum += w;
        const float keep = weightSum > 0.f ? w / weightSum : 0.f;
        if (keep >= 1.f || uSelect < keep)
        {
            uSelect = keep >= 1.f ? uSelect : uSelect / keep;
            selectedWeight = w;
            selectedRd = rd;
            sel = h;
        }
        else
        {
            uSelect = (uSelect - keep) / (1.f - keep);
        }
        tMin = h.t + kRayMinT;
    }
    if (!(selectedWeight > 0.f)) return false;
    const GpuInstance& I = S.instances[entry.instance];
    TriGeom g = fetchTri(S, I, sel.prim);
    const float3 nOS = normalize(cross(g.p2 - g.p1, g.p3 - g.p1));
    const float3 nWS = normalize(xformVectorT(I.w2o, nOS));
    // the front face faces against the probe
    const float3 frontN = ((dot(nWS, axis) < 0.f) == sel.front) ? nWS : -nWS;
    out.exit.pos = probeOrigin + axis * sel.t;
    out.exit.instance = entry.instance;
    out.exit.normal = entry.front ? frontN : -frontN;
    out.exit.prim = sel.prim;
    out.exit.b1 = sel.b1;
    out.exit.b2 = sel.b2;
    out.exit.front = entry.front;
    const float pdf = pdfSubsurfaceExit(s, ep, entry.normal, out.exit.pos, out.exit.normal);
    if (!(pdf > 0.f)) return false;
    const float selection = selectedWeight / weightSum;
    out.weight = selectedRd / (pdf * selection);
    out.pdfPosition = pdf;
    return true;
}

// The unidirectional integrators evaluate the layered BSDF at three places (the punctual and
// the mesh light connection, and the sampled direction). It is inlined at each site: an
// out-of-line copy (YG_EVAL_OUTLINE) keeps a single copy of the layered evaluation in the
// instruction cache, but passing the surface and its frames by reference puts them in local
// memory for every path. Measured on the NEE workload (shading-class launch of bounce 0, 2^20
// paths): inlined, with the cold out-of-line calls (textures, subsurface) given copies, local
// stores fall from 13.9 M to 7.3 M sectors and DRAM writes from 173 to 39 MB at equal time.
#ifdef YG_EVAL_OUTLINE
static __device__ __noinline__ Eval evaluateSurfaceOnce(const Luts& L, const Surface& s, const SurfaceCtx& c, float3 woOS,
                                                        float3 wiOS, uint32_t flags, const Spectral& sp)
{
    return evaluateSurface(L, s, c, woOS, wiOS, flags, sp);
}
#else
#define evaluateSurfaceOnce evaluateSurface
#endif

// With NEE every light is sampled; without it only the punctual lights, which BSDF sampling
// can never hit (hasExplicitlySampledLights / sampleExplicitLight, rayHitDefault.hlsl:26-81).
// A punctual light is visible when nothing is hit before it (checkUnoccluded) and its
// connection has no MIS weight.
// At a subsurface exit point (exitLobe) the light is weighed by the exit lobe instead of the BSDF
// (connectToExplicitLight, rayHitDefault.hlsl:203-257).
template <bool NEE>
YG_DEV void prepareNee(const SceneView& S, const Luts& Lt, const Spectral& sp, const Surface& s, const SurfaceCtx& c,
                       float3 woOS, float3 posWS, float3 normalWS, const float4* w2o, const PathState& ps,
                       RandomSampler& rs, ShadowRequest& sr, bool exitLobe = false)
{
    auto evalToLight = [&](float3 toLightOS) {
        Eval ev;
        if (exitLobe)
        {
            evaluateSubsurfaceExitLobe(s, c, woOS, toLightOS, kEvalNone, ev.weight, ev.pdf);
            ev.transmission = 0;
        }
        else
        {
            ev = evaluateSurfaceOnce(Lt, s, c, woOS, toLightOS, kEvalNone, sp);
        }
        return ev;
    };
    float4 r = rs.r4();
    uint32_t li;
    float pick;
    if (NEE)
    {
        li = sampleLightIndex(S, r.w);
        pick = S.lights[li].selectionPdf;
    }
    else
    {
        li = samplePunctualLightIndex(S, r.w);
        pick = S.lights[li].punctualSelectionPdf;
    }
    const GpuLight& PL = S.lights[li];
    if (PL.type != kLightMesh)
    {
        // evaluatePunctualLightIncidence (lightSampling.hlsl:255-275)
        float3 toL, I3;
        float dist;
        if (PL.type == kLightDirectional)
        {
            toL = mk3(-PL.directionCosOuter.x, -PL.directionCosOuter.y, -PL.directionCosOuter.z);
            dist = __int_as_float(0x7f800000);
            I3 = mk3(PL.intensity.x, PL.intensity.y, PL.intensity.z);
        }
        else
        {
            float3 v = mk3(PL.positionCosInner.x, PL.positionCosInner.y, PL.positionCosInner.z) - posWS;
            float d2 = fmaxf(dot(v, v), 1e-10f);
            dist = sqrtf(d2);
            toL = v / dist;
            float f = punctualFalloff(PL, -toL) / d2;
            I3 = mk3(PL.intensity.x * f, PL.intensity.y * f, PL.intensity.z * f);
        }
        float4 emission = emissionSpectrum(S, sp, I3, -1);
        if (allEqual4(emission, 0.0f) || !(pick > 0.0f)) return;
        float3 toLightOS = normalize(xformVector(w2o, toL));
        Eval ev = evalToLight(toLightOS);
        float4 w = ev.weight;
        if ((ev.transmission & kTransDispersed) != 0 && !(ps.flags & kFlagSecondaryTerminated)) terminateSecondary(w);
        if (allEqual4(w, 0.0f)) return;
        w = (w / pick) * 1.0f;
        sr.origin = spawnRayOrigin(posWS, normalWS, toL);
        sr.dir = toL;
        sr.tmax = dist - kRayMinT;
        sr.instance = kPunctualShadow;
        sr.prim = li;
        sr.contrib = ps.throughput * w * emission;
        sr.valid = true;
        return;
    }
    LightPoint lp;
    sampleMeshLight(S, sp, li, mk3(r.x, r.y, r.z), lp);
    float3 toLight = lp.pos - posWS;
    float len = length(toLight);
    float cosEmit = -dot(lp.n, toLight / len);
    float4 emission = lp.radiance * evaluateEmissionProfile(cosEmit, lp.focus);
    float pdf = pick * lp.pdfPos * areaToSolidAngle(toLight, lp.n);
    float3 toLightWS = toLight / len;
    if (!lp.twoSided && dot(toLight, lp.n) >= 0.0f)
    {
        emission = splat4(0.0f);
        pdf = 0.0f;
    }
    if (allEqual4(emission, 0.0f) || !(pdf > 0.0f)) return;
    float3 toLightOS = normalize(xformVector(w2o, toLightWS));
    Eval ev = evalToLight(toLightOS);
    float4 w = ev.weight;
    if ((ev.transmission & kTransDispersed) != 0 && !(ps.flags & kFlagSecondaryTerminated)) terminateSecondary(w);
    if (allEqual4(w, 0.0f)) return;
    float wMIS = weightMIS(pdf, ev.pdf);
    w = (w / pdf) * wMIS;
    sr.origin = spawnRayOrigin(posWS, normalWS, toLightWS);
    sr.dir = toLightWS;
    sr.tmax = len + kRayMinT;
    sr.instance = lp.instance;
    sr.prim = lp.prim;
    sr.contrib = ps.throughput * w * emission;
    sr.valid = true;
}

// checkLightVisibility (rayHitDefault.hlsl:83-112): the closest hit must be the sampled light triangle
// checkUnoccluded (rayHitDefault.hlsl:114-133) for punctual lights: nothing may be hit
YG_DEV bool shadowVisible(bool any, const Hit& h, uint32_t inst, uint32_t prim)
{
    if (inst == kPunctualShadow) return !any;
    return any && h.instance == inst && h.prim == prim;
}

// The visibility test above as an any-hit traversal that gives the same answer. The target
// triangle is intersected first (the same test the traversal would make, so the same t); the
// closest hit starts as the target, and the first candidate the traversal finds that would
// replace it (nearer, or equally near with a smaller key) proves the segment occluded. A target
// without geometry (inst = kPunctualShadow) is occluded by any hit. shadowBegin returns whether
// the traversal may stop at such a candidate (shadowStopped); with the target missed it leaves
// nothing to traverse.
YG_DEV bool shadowBegin(TraceState& t, const SceneView& S, float3 o, float3 d, float tmin, float tmax, uint32_t inst,
                        uint32_t prim)
{
    traceBegin(t, S, o, d, tmin, tmax);
    if (inst == kPunctualShadow) return true;
    const uint32_t j = S.triOfPrim ? S.triOfPrim[S.instPrimStart[inst] + prim] : 0xffffffffu;
    if (j == 0xffffffffu) return false; // no position known: the full closest-hit traversal
    intersectTri<false>(t.tris, (int)j, o, d, tmin, t.h, t.found);
    if (!t.found || t.h.instance != inst || t.h.prim != prim) t.gHits = 0; // the target is not hit: occluded
    return true;
}
YG_DEV bool shadowStopped(const TraceState& t, bool early, uint32_t inst, uint32_t prim)
{
    return early && t.found && (inst == kPunctualShadow || t.h.instance != inst || t.h.prim != prim);
}
template <bool COUNT>
__device__ __noinline__ bool traceShadow(const SceneView& S, float3 o, float3 d, float tmin, float tmax, uint32_t inst, uint32_t prim,
                                         TraversalCount* tc)
{
    TraceState t;
    TraceStack st;
    const bool early = shadowBegin(t, S, o, d, tmin, tmax, inst, prim);
    while (traceStep<COUNT>(t, st, tc))
        if (shadowStopped(t, early, inst, prim)) break;
    return shadowVisible(t.found, t.h, inst, prim);
}

// generateCameraRay (raytraceCommonResources.hlsl:113-137) and the sample set-up of
// rayGenPrimaryRays.hlsl:13-37
YG_DEV void beginPath(const SceneView& S, const LaunchParams& P, uint32_t cx, uint32_t cy, RandomSampler& rs, Spectral& sp,
                      PathState& ps)
{
    sp.hero = S.lambdaMin + rs.r1() * (S.lambdaMax - S.lambdaMin);
    sp.lambdas = getSpectralSampleLambdas(sp.hero, S.lambdaMin, S.lambdaMax);
    float invW = 1.0f / (float)P.width, invH = 1.0f / (float)P.height;
    float2 uv = make_float2((float)cx * invW + 0.5f * invW, (float)cy * invH + 0.5f * invH);
    float2 texel = make_float2(sampleDim(rs.point, 0, rs.seed), sampleDim(rs.point, 1, rs.seed));
    float2 lensR = rs.r2();
    float2 to = make_float2(0.f, 0.f);
    if ((P.flags & 2u) == 0) to = make_float2(texel.x - 0.5f, texel.y - 0.5f);
    to = make_float2(to.x * invW, to.y * invH);
    float4 pn = mul44(S.cam.uvToView, mk4(uv.x + to.x, uv.y + to.y, 0.0f, 1.0f));
    pn = pn / pn.w;
    float3 pin = mk3(pn.x, pn.y, pn.z);
    float3 focusP = pin * safeDiv(S.cam.focusDistance, fabsf(pin.z));
    float2 disk = sampleConcentricDisk(lensR);
    float3 lensP = mk3(disk.x * S.cam.apertureRadius, disk.y * S.cam.apertureRadius, 0.0f);
    float4 ow = mul44(S.cam.viewToWorld, mk4(lensP.x, lensP.y, lensP.z, 1.0f));
    float4 dw = mul44(S.cam.viewToWorld, mk4(focusP.x - lensP.x, focusP.y - lensP.y, focusP.z - lensP.z, 0.0f));
    ps.throughput = splat4(1.0f);
    ps.total = splat4(0.0f);
    ps.origin = mk3(ow.x, ow.y, ow.z);
    ps.dir = normalize(mk3(dw.x, dw.y, dw.z));
    ps.pdfThisRay = 0.0f;
    ps.flags = 0;
    ps.pathLength = 0;
    ps.nVol = 0;
}

YG_DEV void spectralOf(const SceneView& S, float hero, Spectral& sp)
{
    sp.hero = hero;
    sp.lambdas = getSpectralSampleLambdas(hero, S.lambdaMin, S.lambdaMax);
}

struct FirstHit
{
    float3 albedo, normal;
    float depth;
};

// The subsurface event at an entry vertex (scatteringSample.hlsl:45-54; rayHitDefault.hlsl:261-320,
// 349-355): probe for the exit point, weigh the throughput by the entry, set the exit surface up
// and continue from it with its light connection and the exit lobe. The entry vertex's light
// connection (sr, prepared before the layer was chosen) is resolved here, so that it is added
// before the exit's and each path keeps one deferred shadow ray. Returns whether the path
// continues (before Russian roulette). Out of line: only paths on subsurface materials run it.
template <bool NEE>
static __device__ __noinline__ bool subsurfaceEvent(const SceneView& S, const LaunchParams& P, const Luts& Lt, const Spectral& sp, const Hit& hit,
                            const GpuInstance& I, const Surface& s, const SurfaceCtx& c, float3 hitPos, float3 normalWS,
                            float4 rB, PathState& ps, RandomSampler& rs, ShadowRequest& sr)
{
    if (sr.valid)
    {
        if (traceShadow<false>(S, sr.origin, sr.dir, kRayMinT, sr.tmax, sr.instance, sr.prim, nullptr))
            ps.total = ps.total + sr.contrib;
        sr.valid = false;
    }
    SurfacePoint entry;
    entry.pos = hitPos;
    entry.normal = dot(-ps.dir, normalWS) < 0.0f ? -normalWS : normalWS; // orientToSameSide
    entry.instance = hit.instance;
    entry.prim = hit.prim;
    entry.b1 = hit.b1;
    entry.b2 = hit.b2;
    entry.front = hit.front;
    SubsurfaceExit ex;
    if (!sampleSubsurfaceExit(S, s, entry, mk3(rB.y, rB.z, rB.w), ex))
    {
        // no exit point: the event has no direction, the path ends
        ps.pdfThisRay = 0.0f;
        ps.flags &= ~kFlagDelta;
        ps.throughput = ps.throughput * splat4(0.0f);
        return false;
    }
    // evaluateSubsurfaceEntry: the edge's area density cancels against the weight's
    float4 entryWeight = ex.weight * (subsurfaceEntryFactor(Lt, s, c, sp.hero) * ex.pdfPosition);
    float pdfForward = c.probs[LAYER_SSS] * ex.pdfPosition;
    ps.throughput = ps.throughput * entryWeight * safeDiv(1.0f, pdfForward);
    // continueFromSubsurfaceExit: the exit surface seen from the outside
    Hit xh;
    xh.t = 0.0f;
    xh.b1 = ex.exit.b1;
    xh.b2 = ex.exit.b2;
    xh.instance = ex.exit.instance;
    xh.prim = ex.exit.prim;
    xh.front = ex.exit.front;
    const GpuInstance& XI = S.instances[ex.exit.instance];
    HitSurface xs;
    setupSurface(S, P, sp, xh, XI, -ex.exit.normal, ps, xs);
    const float3 xwo = -xs.rayDirOS;
    SurfaceCtx xc;
    makeSurfaceCtx(xs.s, currentIOR(ps), previousIOR(ps), xwo, ex.exit.front, xc);
    if (NEE ? S.nLights > 0 : S.nPunctual > 0)
        prepareNee<NEE>(S, Lt, sp, xs.s, xc, xwo, ex.exit.pos, ex.exit.normal, XI.w2o, ps, rs, sr, true);
    const float4 rX = rs.r4();
    const float3 xwi = sampleSubsurfaceExitLobe(xs.s, xc, xwo, make_float2(rX.z, rX.w));
    float4 w = splat4(0.0f);
    float pdf = 0.0f;
    bool dirSet = false;
    if (!isZero3(xwi))
    {
        evaluateSubsurfaceExitLobe(xs.s, xc, xwo, xwi, kEvalNone, w, pdf);
        if (pdf > 0.0f)
        {
            w = w / pdf;
            float3 dW = normalize(xformVector(XI.o2w, xwi));
            ps.origin = spawnRayOrigin(ex.exit.pos, ex.exit.normal, dW);
            ps.dir = dW;
            dirSet = true;
        }
        else
        {
            w = splat4(0.0f);
        }
    }
    ps.flags |= kFlagRegularize;
    ps.flags &= ~kFlagDelta;
    ps.pdfThisRay = pdf;
    ps.throughput = ps.throughput * w;
    return dirSet && pdf != 0.0f;
}

// One traced segment: the miss shader, or the closest-hit shader at the vertex, then
// Russian roulette. Returns whether the path continues; the NEE shadow request (if
// any) must be resolved before the next segment is shaded.
template <bool NEE>
YG_DEV bool shadeSegment(const SceneView& S, const LaunchParams& P, const Luts& Lt, const Spectral& sp, bool found,
                         const Hit& hit, PathState& ps, RandomSampler& rs, ShadowRequest& sr, FirstHit* fh)
{
    sr.valid = false;
    bool alive = true;
    if (!found)
    {
        // rayMissEnvironment: |dir| * Env.IntensityScale, as an unbounded RGB emitter
        float3 col = skyColor(S, ps.dir, P.envScale);
        float4 Le = isZero3(col) ? splat4(0.0f) : fromRGBUnbounded(S, sp, col);
        ps.total = ps.total + ps.throughput * Le;
        alive = false;
    }
    else
    {
        const GpuInstance& I = S.instances[hit.instance];
        HitSurface hs;
        setupSurface(S, P, sp, hit, I, ps.dir, ps, hs);
        Surface& s = hs.s;
        float3 hitPos = ps.origin + ps.dir * hit.t;
        if (ps.pathLength == 0 && fh)
        {
            fh->albedo = hs.albedoRGB;
            fh->normal = normalize(xformVectorT(I.w2o, s.baseLayerNormal));
            float4 vp = mul44(S.cam.worldToView, mk4(hitPos.x, hitPos.y, hitPos.z, 1.0f));
            fh->depth = vp.z * S.cam.forwardZSign;
        }
        // handleRayStartInsideMedium (hitShadersCommon.hlsl:212-222)
        if (dot(hs.rayDirOS, s.geometryNormal) > 0.0f && ps.nVol == 0 && !isTwoSided(s.flags))
            enteredVolume(ps, s.dielectricIOR, s.absorption, hs.material);
        // absorption along the segment
        float4 ab = ps.nVol != 0 ? ps.volAbs[ps.nVol - 1] : splat4(0.0f);
        if (!allEqual4(ab, 0.0f))
        {
            float4 tr = mk4(ygm_expf(-ab.x * hit.t), ygm_expf(-ab.y * hit.t), ygm_expf(-ab.z * hit.t), ygm_expf(-ab.w * hit.t));
            ps.throughput = ps.throughput * tr;
        }
        if (!allEqual4(s.emissive, 0.0f))
        {
            float wMIS = 1.0f;
            if (NEE && S.nLights > 0 && ps.pdfThisRay > 0.0f && !(ps.flags & kFlagDelta))
            {
                float lightPdf = explicitLightPdf(S, hitPos - ps.origin, hit.instance, hit.prim);
                wMIS = weightMIS(ps.pdfThisRay, lightPdf);
            }
            float side = dot(s.geometryNormal, -hs.rayDirOS) < 0.0f ? 0.0f : 1.0f;
            float profile = 1.0f;
            if (s.emissionFocus > 0.0f)
            {
                float3 gnWS = normalize(xformVectorT(I.w2o, s.geometryNormal));
                profile = evaluateEmissionProfile(dot(gnWS, -normalize(ps.dir)), s.emissionFocus);
            }
            ps.total = ps.total + ps.throughput * s.emissive * wMIS * side * profile;
            alive = false;
        }
        else
        {
            // evaluateSurfaceAndGenerateNextSampleDirection (rayHitDefault.hlsl:316-435)
            float4 rB = rs.r4();
            float3 wo = -hs.rayDirOS;
            SurfaceCtx c;
            makeSurfaceCtx(s, currentIOR(ps), previousIOR(ps), wo, hit.front, c);
            float3 normalWS = normalize(xformVectorT(I.w2o, s.geometryNormal));
            if ((NEE ? S.nLights > 0 : S.nPunctual > 0) && !isDeltaDistribution(c.a2, s))
                prepareNee<NEE>(S, Lt, sp, s, c, wo, hitPos, normalWS, I.w2o, ps, rs, sr);
            // sampleScatteringEvent (scatteringSample.hlsl:30-65)
            int layer = selectMaterialLayer(rB.x, c.probs);
            if (layer == LAYER_SSS)
            {
                // the out-of-line event works on copies, so that the state every path uses
                // never has its address taken
                PathState psX = ps;
                RandomSampler rsX = rs;
                ShadowRequest srX = sr;
                const Hit hitX = hit;
                const Spectral spX = sp;
                const Luts ltX = Lt;
                const Surface sX = s;
                const SurfaceCtx cX = c;
                alive = subsurfaceEvent<NEE>(S, P, ltX, spX, hitX, I, sX, cX, hitPos, normalWS, rB, psX, rsX, srX);
                ps = psX;
                rs = rsX;
                sr = srX;
                ps.pathLength += 1;
                if (alive && russianRoulette(ps.throughput, rs.r1())) alive = false;
                return alive;
            }
            float3 wi = mk3(0.f, 0.f, 0.f);
            bool isDiffuse = false, isDelta = false;
            if (layer < LAYER_COUNT)
                wi = sampleLayerDirection(Lt, s, c, layer, rB.y, make_float2(rB.z, rB.w), sp.hero, isDiffuse, isDelta);
            Eval ev;
            ev.weight = splat4(0.0f);
            ev.pdf = 0.0f;
            ev.transmission = 0;
            if (!isZero3(wi))
            {
                ev = evaluateSurfaceOnce(Lt, s, c, wo, wi, isDelta ? kEvalTreatAsDelta : kEvalNone, sp);
                if (isDiffuse) ps.flags |= kFlagRegularize;
            }
            ps.pdfThisRay = ev.pdf;
            if (isDelta) ps.flags |= kFlagDelta;
            else ps.flags &= ~kFlagDelta;
            if (ev.pdf > 0.0f)
            {
                if (ev.transmission != 0)
                {
                    if ((ev.transmission & kTransDispersed) != 0)
                    {
                        if (!(ps.flags & kFlagSecondaryTerminated)) terminateSecondary(ev.weight);
                        ps.flags |= kFlagSecondaryTerminated;
                    }
                    bool entered = (ev.transmission & kTransEntered) != 0;
                    bool exited = (ev.transmission & kTransExited) != 0;
                    if (entered != exited)
                    {
                        if (exited) exitedVolume(ps, hs.material);
                        else enteredVolume(ps, s.dielectricIOR, s.absorption, hs.material);
                    }
                }
                ev.weight = ev.weight / ev.pdf;
            }
            ps.throughput = ps.throughput * ev.weight;
            if (isZero3(wi) || ps.pdfThisRay == 0.0f)
            {
                alive = false;
            }
            else
            {
                float3 nW = normalize(xformVector(I.o2w, s.geometryNormal));
                float3 dW = normalize(xformVector(I.o2w, wi));
                ps.origin = spawnRayOrigin(hitPos, nW, dW);
                ps.dir = dW;
            }
        }
    }
    ps.pathLength += 1;
    // Russian roulette after every traced segment (rayGenPrimaryRays.hlsl:91-101); a path
    // that already ended gains nothing from it, so it is skipped there
    if (alive && russianRoulette(ps.throughput, rs.r1())) alive = false;
    return alive;
}

} // namespace yg
