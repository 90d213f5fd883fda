// TEST INFRASTRUCTURE ONLY: the reference's shader math -- edited copies of its .hlsl files
// under oracle/_ref/hlsl, written by oracle/ref_build.py -- compiled on the CPU with
// oracle/hlsl_shim.h, behind the plain functions of refcheck.h (prefix ref_). Compiled a
// second time by hlsl_side_kulla.cpp with RECIPROCAL_MULTISCATTER defined, as the
// bidirectional integrator compiles it (BDPTCommon.hlsl:6), under the prefix refK_.
#ifndef REFCHECK_NS
#define REFCHECK_NS hlsl
#define REFCHECK_PREFIX ref_
#endif
#define HLSL_SHIM_NS REFCHECK_NS
#define REFCHECK_CAT2(a, b) a##b
#define REFCHECK_CAT(a, b) REFCHECK_CAT2(a, b)
#define FN(name) REFCHECK_CAT(REFCHECK_PREFIX, name)

#include "hlsl_shim.h"

#include <vector>

#include "refcheck.h"

namespace REFCHECK_NS
{
static float g_checkHeroLambda = 500.0f;
static ByteAddressBuffer g_randomSamples;
#define GET_SPECTRAL_SAMPLE_WAVELENGTH g_checkHeroLambda
#define GET_RANDOM_NUMBER_SEQUENCE_1(dimOffset) (g_randomSamples.Load((dimOffset) << 2))
#define GET_RANDOM_NUMBER_SEQUENCE_2(dimOffset) (g_randomSamples.Load2((dimOffset) << 2))
#define GET_RANDOM_NUMBER_SEQUENCE_3(dimOffset) (g_randomSamples.Load3((dimOffset) << 2))
#define GET_RANDOM_NUMBER_SEQUENCE_4(dimOffset) (g_randomSamples.Load4((dimOffset) << 2))
#define interface struct
#include "../_ref/hlsl/common/random.hlsl"
#include "../_ref/hlsl/common/randomSampler.hlsl"
#include "../_ref/hlsl/materials/materialsCommonResources.hlsl"
#include "../_ref/hlsl/raytracing/spectralDistribution.hlsl"
#include "../_ref/hlsl/SurfaceDefinition.inc"
#include "../_ref/hlsl/raytracing/materialSample.hlsl"
#include "../_ref/hlsl/subsurface_math.inc"
#undef interface
} // namespace REFCHECK_NS

namespace refcheck
{
using namespace REFCHECK_NS;

namespace
{
std::vector<float4> g_tex[12];

template <class Tex> void bindLut(Tex& t, int slot, const float* src, int n)
{
    g_tex[slot].resize(n);
    for (int i = 0; i < n; ++i) g_tex[slot][i] = float4(src[i], 0.0f, 0.0f, 0.0f);
    t.texels = g_tex[slot].data();
}
float3 v3(const float* p) { return float3(p[0], p[1], p[2]); }
void put3(float3 v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
SpectralSamples spec(const float* p)
{
    SpectralSamples s;
    s.samples = float4(p[0], p[1], p[2], p[3]);
    return s;
}

SurfaceDefinition surfaceOf(const Surface& s)
{
    SurfaceDefinition d;
    d.specular = spec(s.specular);
    d.albedo = spec(s.albedo);
    d.absorption = spec(s.absorption);
    d.emissive = spec(s.emissive);
    d.sheenColor = spec(s.sheenColor);
    d.subsurfaceRadius = spec(s.sssRadius);
    d.coatingLayerNormal = v3(s.coatN);
    d.baseLayerNormal = v3(s.baseN);
    d.geometryNormal = v3(s.geoN);
    d.tangent = v3(s.tangent);
    d.transparency = s.transparency;
    d.metalness = s.metalness;
    d.dielectricIOR = s.ior;
    d.roughness = s.roughness;
    d.cauchysCoeffs = float2(s.cauchyA, s.cauchyB);
    d.specularAmount = s.specAmount;
    d.clearCoatAmount = s.ccAmount;
    d.clearCoatIOR = s.ccIOR;
    d.clearCoatRoughness = s.ccRough;
    d.anisotropy = s.aniso;
    d.anisotropyRotation = s.anisoRot;
    d.thinFilmThicknessNM = s.thinFilm;
    d.sheenRoughness = s.sheenRough;
    d.sheenAmount = s.sheenAmount;
    d.emissionFocus = s.focus;
    d.subsurfaceAmount = s.sssAmount;
    d.occlusionSpecDiffPacked = packOcclusion(s.diffOcc, s.specOcc);
    d.flags = s.flags;
    return d;
}
} // namespace

void FN(setup)(const Tables& t)
{
    bindLut(g_dirAlbedoGGXNoFresnelLUT, 0, t.lut[0], 32 * 32);
    g_dirAlbedoGGXNoFresnelLUT.w = g_dirAlbedoGGXNoFresnelLUT.h = 32;
    bindLut(g_avgDirAlbedoGGXNoFresnelLUT, 1, t.lut[1], 32);
    g_avgDirAlbedoGGXNoFresnelLUT.w = 32;
    bindLut(g_dirAlbedoGGXSingleAndMultiScatterLUT, 2, t.lut[2], 16 * 16 * 16);
    g_dirAlbedoGGXSingleAndMultiScatterLUT.w = g_dirAlbedoGGXSingleAndMultiScatterLUT.h =
        g_dirAlbedoGGXSingleAndMultiScatterLUT.d = 16;
    bindLut(g_avgDirAlbedoGGXSingleAndMultiScatterLUT, 3, t.lut[3], 16 * 16);
    g_avgDirAlbedoGGXSingleAndMultiScatterLUT.w = g_avgDirAlbedoGGXSingleAndMultiScatterLUT.h = 16;
    bindLut(g_dirAlbedoGGXTranslucentDenserLUT, 4, t.lut[4], 16 * 16 * 16);
    g_dirAlbedoGGXTranslucentDenserLUT.w = g_dirAlbedoGGXTranslucentDenserLUT.h = g_dirAlbedoGGXTranslucentDenserLUT.d = 16;
    bindLut(g_dirAlbedoGGXTranslucentLighterLUT, 5, t.lut[5], 16 * 16 * 16);
    g_dirAlbedoGGXTranslucentLighterLUT.w = g_dirAlbedoGGXTranslucentLighterLUT.h = g_dirAlbedoGGXTranslucentLighterLUT.d = 16;
    bindLut(g_avgAlbedoGGXTranslucentDenserLUT, 6, t.lut[6], 16 * 16);
    g_avgAlbedoGGXTranslucentDenserLUT.w = g_avgAlbedoGGXTranslucentDenserLUT.h = 16;
    bindLut(g_avgAlbedoGGXTranslucentLighterLUT, 7, t.lut[7], 16 * 16);
    g_avgAlbedoGGXTranslucentLighterLUT.w = g_avgAlbedoGGXTranslucentLighterLUT.h = 16;
    bindLut(g_dirAlbedoSheenNoFresnelLUT, 8, t.lut[8], 16 * 16);
    g_dirAlbedoSheenNoFresnelLUT.w = g_dirAlbedoSheenNoFresnelLUT.h = 16;
    // CIE x y z and D65 at 1 nm over 380..700 (CIE_LUT_RESOLUTION texels)
    g_tex[9].resize(321);
    g_tex[10].resize(321);
    for (int i = 0; i < 321; ++i)
    {
        const float* c = t.cie321x4 + 4 * i;
        g_tex[9][i] = float4(c[0], c[1], c[2], 0.0f);
        g_tex[10][i] = float4(c[3], 0.0f, 0.0f, 0.0f);
    }
    g_cieXYZCoeffsLUT.texels = g_tex[9].data();
    g_cieXYZCoeffsLUT.w = 321;
    g_d65IlluminantLUT.texels = g_tex[10].data();
    g_d65IlluminantLUT.w = 321;
    g_tex[11].resize(64 * 64 * 64);
    for (int i = 0; i < 64 * 64 * 64; ++i)
        g_tex[11][i] = float4(t.rgb64[3 * i], t.rgb64[3 * i + 1], t.rgb64[3 * i + 2], 0.0f);
    g_srgbToSPDLUT.texels = g_tex[11].data();
    g_srgbToSPDLUT.w = g_srgbToSPDLUT.h = g_srgbToSPDLUT.d = 64;
    g_randomSamples.data = reinterpret_cast<const uint8_t*>(t.sobolPoint);
    g_randomSamples.bytes = 256 * 4;
}

uint32_t FN(hash2)(uint32_t a, uint32_t b) { return hash(a, b); }
uint32_t FN(owen)(uint32_t v, uint32_t seed) { return owenScrambleBase2Fast(v, seed); }
float FN(u01)(uint32_t v) { return uintToFloat01(v); }
void FN(sampler)(uint32_t pixelSeed, uint32_t n, float* out)
{
    RandomSampler rs;
    rs.init(0, pixelSeed);
    float2 t = rs.getTexelOffset();
    out[0] = t.x;
    out[1] = t.y;
    for (uint32_t i = 0; i < n; ++i) out[2 + i] = rs.getRandom1();
}
void FN(lambdas)(float u, float out[4])
{
    g_checkHeroLambda = calculateSpectralSampleWavelength(u);
    float4 l = getSpectralSampleLambdas();
    for (int k = 0; k < 4; ++k) out[k] = l[k];
}
float FN(sigmoid)(float x) { return sigmoid(x); }
void FN(rgb_spectrum)(int mode, const float rgb[3], float hero, float out[4])
{
    g_checkHeroLambda = hero;
    SpectralSamples s;
    if (mode == 0) s.setFromRGB(v3(rgb));
    else if (mode == 1) s.setFromRGBUnbounded(v3(rgb));
    else s.setFromRGBUnboundedNoIlluminant(v3(rgb));
    for (int k = 0; k < 4; ++k) out[k] = s.samples[k];
}
void FN(to_xyz)(float hero, const float L[4], float out[3])
{
    g_checkHeroLambda = hero;
    SpectralSamples s = spec(L);
    put3(s.ToXYZ(), out);
}
int FN(roulette)(const float w[4], float rand, float norm, float out[4])
{
    SpectralSamples s = spec(w);
    bool killed = s.applyRussianRoulette(rand, norm);
    for (int k = 0; k < 4; ++k) out[k] = s.samples[k];
    return killed ? 1 : 0;
}
float FN(lambda_ggx)(const float d[3], float ax, float ay) { return smithLambdaGGX(v3(d), ax, ay); }
float FN(g1)(const float wo[3], const float wm[3], float ax, float ay) { return G1GGX(v3(wo), v3(wm), ax, ay); }
float FN(g2)(const float wo[3], const float wi[3], const float wm[3], float ax, float ay)
{
    return G2GGX(v3(wo), v3(wi), v3(wm), ax, ay);
}
float FN(dggx)(const float wm[3], float ax, float ay) { return DGGX(v3(wm), ax, ay); }
float FN(dv)(const float wo[3], const float wm[3], float ax, float ay) { return DVGGX(v3(wo), v3(wm), ax, ay); }
void FN(sample_wm)(const float wo[3], float ax, float ay, float u1, float u2, float out[3])
{
    put3(sampleWMGGX(v3(wo), ax, ay, u1, u2), out);
}
void FN(conductor_nk)(float r, float g, float out[2])
{
    float2 v = getConductorRefractiveIndexAndExtinctionthroughputSquared(r, g);
    out[0] = v.x;
    out[1] = v.y;
}
float FN(fresnel_dc)(float er, float ei, float c) { return fresnelDielectricConductor(er, ei, c); }
float FN(fresnel_dd)(float eta, float c) { return fresnelDielectricDielectric2(eta, c); }
float FN(dsheen)(const float wm[3], float r) { return DSheen(v3(wm), r); }
float FN(gsheen)(const float wo[3], const float wi[3], float r) { return GSheen(v3(wo), v3(wi), r); }
float FN(emission_profile)(float d, float e) { return evaluateEmissionProfile(d, e); }
void FN(concentric_disk)(float u0, float u1, float out[2])
{
    float2 p = sampleConcentricDisk(float2(u0, u1));
    out[0] = p.x;
    out[1] = p.y;
}
// lobes: 0 conductor reflection, 1 dielectric reflection, 2 transmission, 3 dielectric
// (reflection or transmission), 4 Lambertian, 5 sheen
void FN(sample_lobe)(int lobe, float eta, float ax, float ay, const float wo[3], float s0, float s1, float sc, int aR,
                     int aT, float out[3])
{
    float3 w = v3(wo), r = 0.0f;
    float2 s = float2(s0, s1);
    switch (lobe)
    {
    case 0: r = sampleGGXReflectionConductor(ax, ay, w, s); break;
    case 1: r = sampleGGXReflectionDielectric(ax, ay, w, s); break;
    case 2: r = sampleGGXTransmitted(eta, ax, ay, w, s); break;
    case 3: r = sampleDielectric(eta, ax, ay, w, s, sc, aR != 0, aT != 0); break;
    case 4: r = sampleDiffuseLambertian(ax, ay, w, s); break;
    case 5: r = sampleSheen(ax, w, s); break;
    }
    put3(r, out);
}
float FN(pdf_lobe)(int lobe, float eta, float ax, float ay, const float wo[3], const float wi[3], int aR, int aT)
{
    float3 o = v3(wo), i = v3(wi);
    switch (lobe)
    {
    case 0: return pdfGGXReflectionConductor(o, i, ax, ay);
    case 1: return pdfGGXReflectionDielectric(o, i, ax, ay);
    case 2: return pdfGGXTransmitted(eta, o, i, ax, ay);
    case 3: return pdfDielectric(eta, o, i, ax, ay, aR != 0, aT != 0);
    case 4: return pdfDiffuseLambertian(o, i, ax, ay);
    case 5: return pdfSheen(o, i, ax);
    }
    return 0.0f;
}
// eval: conductor with (etaR, etaK) = (eta, k); Lambertian with albedo eta; sheen with colour eta
// and roughness ax
float FN(eval_lobe)(int lobe, float eta, float k, float ax, float ay, const float wo[3], const float wi[3])
{
    float3 o = v3(wo), i = v3(wi);
    switch (lobe)
    {
    case 0: return evaluateGGXReflectionConductor(eta, k, ax, ay, o, i);
    case 1: return evaluateGGXReflectionDielectric(eta, ax, ay, o, i);
    case 2: return evaluateGGXTransmitted(eta, ax, ay, o, i);
    case 4: return evaluateDiffuseLambertian(eta, ax, ay, o, i);
    case 5: return evaluateSheen(eta, ax, o, i);
    }
    return 0.0f;
}
// multiple scattering: see oracle_side.cpp for the list
float FN(ms)(int fn, float a, float dWo, float dWi, float lr, float x)
{
    switch (fn)
    {
    case 0: return getEnergyCompensationTurquin(a, dWo, dWi, lr, x);
    case 1: return getEnergyCompensationKulla(a, dWo, dWi, lr, x);
    case 2: return getEnergyRemainingAfterSpecular(a, dWo, dWi, lr, x);
    case 3: return getEnergyRemainingAfterSheen(dWo, dWi, lr, x);
    case 4: return getEnergyCompensationTranslucentTurquin(a, dWo, dWi, lr, x);
    case 5: return getEnergyCompensationTranslucentKulla(a, dWo, dWi, lr, x);
    case 6: return getAvgFresnel(a);
    case 7: return getMsTransmissionRatio(a, lr);
    case 8: return getFmsDielectric(a, lr, dWo);
    case 9: return getSheenDirectionalAlbedo(dWo, lr);
    case 10: return getDirectionalAlbedoTranslucent(a, dWo, lr);
    case 11: return getAverageAlbedoTranslucent(a, lr);
    }
    return 0.0f;
}
void FN(layer_probs)(const Surface& s, float cur, float prev, const float wo[3], int front, float out[6])
{
    SurfaceSamplingContext c = makeSurfaceSamplingContext(surfaceOf(s), cur, prev, v3(wo), front != 0);
    for (int k = 0; k < 6; ++k) out[k] = c.samplingProbabilities[k];
}
Eval FN(eval_surface)(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, const float wi[3],
                      uint32_t flags)
{
    g_checkHeroLambda = hero;
    SurfaceSamplingContext c = makeSurfaceSamplingContext(surfaceOf(s), cur, prev, v3(wo), front != 0);
    SurfaceEvaluation e = evaluateSurface(c, v3(wo), v3(wi), flags);
    Eval r;
    for (int k = 0; k < 4; ++k) r.w[k] = e.weight.samples[k];
    r.pdf = e.pdf;
    r.trans = e.transmissionType;
    return r;
}
void FN(sample_layer)(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, int layer, float sel,
                      float r0, float r1, float out[3], int* diffuse, int* delta)
{
    g_checkHeroLambda = hero;
    SurfaceSamplingContext c = makeSurfaceSamplingContext(surfaceOf(s), cur, prev, v3(wo), front != 0);
    bool d = false, dl = false;
    put3(getSampleDirectionOSForLayer(c, (uint)layer, sel, float2(r0, r1), d, dl), out);
    *diffuse = d ? 1 : 0;
    *delta = dl ? 1 : 0;
}
// the Burley profile: 0 burleyProfileArea(r = a, d = b), 1 burleySampleRadius(u = a, d = b),
// 2 burleyD(radius = a, albedo = b)
float FN(sss)(int fn, float a, float b)
{
    switch (fn)
    {
    case 0: return burleyProfileArea(a, b);
    case 1: return burleySampleRadius(a, b);
    case 2: return burleyD(a, b);
    }
    return 0.0f;
}
float FN(sss_pdf)(const Surface& s, const float fromP[3], const float fromN[3], const float toP[3], const float toN[3])
{
    return pdfSubsurfaceExit(surfaceOf(s), v3(fromP), v3(fromN), v3(toP), v3(toN));
}
float FN(sss_entry)(const Surface& s, float hero, float cur, float prev, const float wo[3], int front)
{
    g_checkHeroLambda = hero;
    SurfaceSamplingContext c = makeSurfaceSamplingContext(surfaceOf(s), cur, prev, v3(wo), front != 0);
    return getSubsurfaceEntryFactor(c.surfaceDef, c.precalculatedSurfaceData);
}
// out: sampled direction (3), weight (4) and pdf of the exit lobe at wi
void FN(sss_exit_lobe)(const Surface& s, float cur, float prev, const float wo[3], int front, float r0, float r1,
                       const float wi[3], uint32_t flags, float out[8])
{
    SurfaceSamplingContext c = makeSurfaceSamplingContext(surfaceOf(s), cur, prev, v3(wo), front != 0);
    put3(sampleSubsurfaceExitLobe(c.surfaceDef, c.precalculatedSurfaceData, v3(wo), float2(r0, r1)), out);
    SpectralSamples w;
    float pdf = 0.0f;
    evaluateSubsurfaceExitLobe(c.surfaceDef, c.precalculatedSurfaceData, v3(wo), v3(wi), flags, w, pdf);
    for (int k = 0; k < 4; ++k) out[3 + k] = w.samples[k];
    out[7] = pdf;
}
} // namespace refcheck
