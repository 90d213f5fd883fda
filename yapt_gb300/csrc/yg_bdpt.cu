// Bidirectional path tracing with MIS (the BDPT render pipeline), restated for CUDA from
// YAPT's compute shaders:
//   BDPTCommon.hlsl:26-1223           node format, MIS ratio sums, connections
//   BDPTTraceLightPath.comp:6-362     light subpaths
//   BDPTTraceCameraPath.comp:40-432   camera subpaths + connections to every light vertex
//   BDPTCalculatePureLightPaths.comp:107-206, BDPTAccumulatePureLightPaths.comp:7-31
//                                     light tracing to the lens (t = 1)
// The BSDF runs with the Kulla-Conty multiple-scattering model (RECIPROCAL_MULTISCATTER,
// BDPTCommon.hlsl:6), as in the reference.
//
// Layout on the device: light vertices are stored by (sample index, light path, vertex),
// so the reference's header/vertex counters, linked lists and sort pass are not needed.
// The light paths that produced vertices are compacted in index order, which makes the
// random light-path pick of a camera group deterministic (the reference orders them by
// atomic arrival). A camera group is 64 consecutive entries of a fixed pixel permutation and
// connects to one light path; the camera side runs as a wavefront (trace, shade with one
// connection record per light vertex, visibility, in-order accumulation), with every light
// vertex's spectral surface and forward shading frame set up once per wave: the group shares
// the hero wavelength of its light path, so those do not depend on the pixel. Light-tracing
// splats are summed in 64-bit fixed point, so the film does not depend on atomic order.
#include <algorithm>

#include "yg_path.cuh"
#include "yg_kernels.h"
#include "yg_wave.cuh"

namespace yg
{

constexpr uint32_t NF_TERMINATED = 1u << 0; // LIGHT_PATH_NODE_FLAG_* (BDPTCommon.hlsl:13-24)
constexpr uint32_t NF_FRONT = 1u << 1;
constexpr uint32_t NF_ENV = 1u << 2;
constexpr uint32_t NF_DELTA = 1u << 3;
constexpr uint32_t NF_REGULARIZED = 1u << 4;
constexpr uint32_t NF_SSS_EXIT = 1u << 5;   // reached through the subsurface from the previous node (no ray between)
constexpr uint32_t NF_PUNCTUAL = 1u << 6;    // origin at a punctual light; prim holds the light index
constexpr uint32_t NF_DIRECTIONAL = 1u << 7; // origin at a directional light (a point on its emitting disk)
constexpr uint32_t NF_INFINITE = NF_ENV | NF_DIRECTIONAL; // isInfiniteLightNode: the normal holds the direction
constexpr float kMaxPdfRatioSum = 1e16f;    // MAX_PDF_RATIO_SUM
constexpr float kVisibilityEps = 0.001f;    // VISIBILITY_RAY_EPSILON
constexpr double kSplatScale = 16777216.0;  // fixed-point units per XYZ unit (2^24)
constexpr int kGroupSize = 64;              // THREAD_GROUP_DIM_SIZE_CAM_RAY^2
constexpr uint32_t kWbAtExit = 1u << 12;    // camera wave flags: this vertex is a subsurface exit,
constexpr uint32_t kWbPrevExit = 1u << 13;  // the previous vertex was one

// LightPathNode (BDPTCommon.hlsl:52-67): 80 bytes, the normal kept in FP32 (the reference
// packs it to FP16 and spends the 4 bytes on a linked-list index instead).
struct alignas(16) LightNode
{
    float4 radiance;
    float3 normal;
    uint32_t flags;
    float3 pos;
    uint32_t instance;
    float2 bary;
    uint32_t prim;
    float pdfFwd;
    float pdfBwd, iorPrev, iorCur, pad;
};

struct BdptParams
{
    uint32_t frames;        // sample indices in this launch
    uint32_t lightPaths;    // light subpaths per sample index
    uint32_t maxLightVerts; // g_maxVerticesPerLightPath
    uint32_t groups;        // camera groups per sample index
    uint32_t camDimOffset;  // g_cameraPathRandomDimensionOffset
    uint32_t lensDimOffset; // g_pureLightPathLensRandomDimensionOffset
    LightNode* nodes;       // [frame][path][vertex]
    uint32_t* counts;       // [frame][path] stored vertices (0: no header)
    float* heroes;          // [frame][path]
    uint32_t* valid;        // [frame][header] path index of each header, ascending
    uint32_t* validCount;   // [frame] header count
    const uint32_t* perm;   // [cropW*cropH] pixel permutation (crop-relative indices)
    unsigned long long* splat; // [frame][crop pixel][3] fixed-point XYZ
    float3 worldCenter;
    float worldRadiusSqr;
};

YG_DEV Luts bdptLuts(const SceneView& S)
{
    return Luts{S.lutSS, S.lutSSAvg, S.lutSSMS, S.lutSSMSAvg, S.lutTransDenser, S.lutTransLighter,
                S.lutTransAvgDenser, S.lutTransAvgLighter, S.lutSheen};
}

// ------------------------------------------------------------------ densities and ratios
// solidAngleToAreaDensityMultiplier (commonMath.hlsl)
YG_DEV float solidAngleToArea(float3 v, float3 n)
{
    float invD2 = 1.0f / dot(v, v);
    return fabsf(dot(n, v * sqrtf(invD2))) * invD2;
}
// calculatePDFRatio / accumulateRISum (BDPTCommon.hlsl:555-577)
YG_DEV float pdfRatio(float nom, float denom)
{
    nom = nom < 0.0f ? 1.0f : nom;
    denom = denom < 0.0f ? 1.0f : denom;
    return fminf(safeDiv(nom, denom), kMaxPdfRatioSum);
}
YG_DEV float accumulateRISum(float riSum, float nom, float denom, bool connectable = true)
{
    float ri = pdfRatio(nom, denom);
    bool acc = connectable && nom > 0.0f && denom > 0.0f;
    riSum = ri * riSum;
    if (acc) riSum += ri;
    return fminf(riSum, kMaxPdfRatioSum);
}
// miscBrdf.hlsl:43-67, 108-118
YG_DEV float3 sampleCosPowHemi(float2 r, float e)
{
    float y = ygm_powf(1.0f - r.x, 1.0f / (e + 2.0f));
    float rr = sqrtf(fmaxf(0.0f, 1.0f - sqr(y)));
    float sn, cs;
    ygm_sincosf(2.0f * kPI * r.y, &sn, &cs);
    return mk3(rr * cs, y, rr * sn);
}
YG_DEV float3 sampleCosPowSphere(float2 s, float e)
{
    bool flip = s.x < 0.5f;
    s.x = flip ? s.x * 2.0f : (s.x - 0.5f) * 2.0f;
    float3 d = sampleCosPowHemi(s, e);
    d.y = flip ? -d.y : d.y;
    return d;
}
YG_DEV float pdfCosPowHemi(float d, float e) { return (e + 2.0f) * kINVPI * 0.5f * ygm_powf(saturate(d), e + 1.0f); }
YG_DEV float pdfCosPowSphere(float d, float e) { return (e + 2.0f) * kINVPI * 0.25f * ygm_powf(fabsf(d), e + 1.0f); }

// sampleSphere, sampleUniformCone (around +y), pdfUniformCone (miscBrdf.hlsl:70-94)
YG_DEV float3 sampleSphere(float2 r)
{
    float y = 1.0f - 2.0f * r.x;
    float rr = sqrtf(1.0f - y * y);
    float s, c;
    ygm_sincosf(2.0f * kPI * r.y, &s, &c);
    return mk3(rr * c, y, rr * s);
}
YG_DEV float3 sampleUniformCone(float2 r, float cosMax)
{
    float y = 1.0f - r.x * (1.0f - cosMax);
    float rr = sqrtf(fmaxf(0.0f, 1.0f - y * y));
    float s, c;
    ygm_sincosf(2.0f * kPI * r.y, &s, &c);
    return mk3(rr * c, y, rr * s);
}
YG_DEV float pdfUniformCone(float cosMax) { return safeDiv(1.0f, 2.0f * kPI * (1.0f - cosMax)); }

// environmentSelectionPDF / pdfEnvironmentDirection / pdfEnvironmentPosition (lightSampling.hlsl:23-76);
// ENV_LIGHT_SELECTION_PROBABILITY is 0, so the environment starts light paths only without lights
YG_DEV float envSelectionPdf(const SceneView& S) { return S.nLights == 0 ? 1.0f : 0.0f; }
YG_DEV float pdfEnvDirection(float3 d)
{
    float c = clampf(d.z, -1.0f, 1.0f);
    float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    return safeDiv(1.0f, 2.0f * kPI * kPI * s);
}
YG_DEV float pdfEnvPosition(const BdptParams& B) { return safeDiv(1.0f, kPI * B.worldRadiusSqr); }
// getSkyBoxColor without an environment map (|dir|) as an unbounded RGB emitter
YG_DEV float4 skyRadiance(const SceneView& S, const LaunchParams& P, const Spectral& sp, float3 d)
{
    float3 col = skyColor(S, d, P.envScale);
    return isZero3(col) ? splat4(0.0f) : fromRGBUnbounded(S, sp, col);
}
// constructVectorBase (commonMath.hlsl:87-93)
YG_DEV void vectorBase(float3 v, float3& a, float3& b)
{
    if (fabsf(v.x) > fabsf(v.y)) a = mk3(-v.z, 0.0f, v.x) / sqrtf(v.x * v.x + v.z * v.z);
    else a = mk3(0.0f, v.z, -v.y) / sqrtf(v.y * v.y + v.z * v.z);
    b = cross(v, a);
}

// calculateCameraDirectionalPDF (BDPTCommon.hlsl:536-550)
YG_DEV float cameraDirectionalPdf(const SceneView& S, const LaunchParams& P, float3 v)
{
    float4 mn = mul44(S.cam.uvToView, mk4(0.f, 0.f, 0.f, 1.f));
    float4 mx = mul44(S.cam.uvToView, mk4(1.f, 1.f, 0.f, 1.f));
    mn = mn / mn.w;
    mx = mx / mx.w;
    float ex = fabsf(mx.x - mn.x), ey = fabsf(mx.y - mn.y);
    float area = safeDiv(ex * ey, mn.z * mn.z);
    float4 vs = mul44(S.cam.worldToView, mk4(v.x, v.y, v.z, 0.0f));
    float3 vv = mk3(vs.x, vs.y, vs.z);
    float c = fabsf(vv.z) * (1.0f / sqrtf(fmaxf(0.0001f, dot(vv, vv))));
    return safeDiv((float)P.width * (float)P.height, area * c * c * c);
}

// pdfForSamplingLight (lightSampling.hlsl:191-230) for a point on a mesh light
YG_DEV void pdfForSamplingLight(const SceneView& S, uint32_t inst, uint32_t prim, float3 n, float3 towards, float& pick,
                                float& posPdf, float& dirPdf)
{
    const GpuInstance& I = S.instances[inst];
    pick = (1.0f - envSelectionPdf(S)) * I.lightPdf;
    const GpuMaterial& M = S.materials[I.material];
    TriGeom g = fetchTri(S, I, prim);
    float3 p1 = xformPoint(I.o2w, g.p1), p2 = xformPoint(I.o2w, g.p2), p3 = xformPoint(I.o2w, g.p3);
    float area = length(cross(p2 - p1, p3 - p1)) * 0.5f;
    posPdf = 1.0f / ((float)I.primCount * area);
    float c = dot(n, towards);
    if (M.mask & 1u) dirPdf = pdfCosPowSphere(c, M.emissionFocus);
    else dirPdf = c >= 0.0f ? pdfCosPowHemi(c, M.emissionFocus) : 0.0f;
}

// ------------------------------------------------------------------ scattering with both densities
struct ScatterEval
{
    float4 weight;
    float pdfFwd, pdfBwd;
    uint32_t transmission;
};

// evaluateSurfaceAndPDFs (BDPTCommon.hlsl:377-443) without the ray-state update: the forward
// evaluation, and the density of sampling wo from wi with the frame rebuilt for wi. Kept out
// of line: the camera-vertex kernel calls it for the connection's camera end, its light end
// and the continuation, and one shared copy of the layered BSDF keeps the kernel's code
// within the instruction cache.
__device__ __noinline__ ScatterEval evaluateBoth(const Luts& L, const Spectral& sp, const Surface& s, const SurfaceCtx& c, float curIOR,
                                float prevIOR, float3 wo, float3 wi, bool front, bool fromLight, bool treatAsDelta)
{
    ScatterEval r;
    uint32_t flags = kEvalNone | (fromLight ? kEvalLightPath : 0u) | (treatAsDelta ? kEvalTreatAsDelta : 0u);
    Eval fwd = evaluateSurface<true>(L, s, c, wo, wi, flags, sp);
    r.weight = fwd.weight;
    r.pdfFwd = fwd.pdf;
    r.transmission = fwd.transmission;
    bool transmitted = dot(wo, s.geometryNormal) * dot(wi, s.geometryNormal) < 0.0f;
    SurfaceCtx rc;
    makeSurfaceCtx(s, curIOR, prevIOR, wi, transmitted ? !front : front, rc);
    if (transmitted)
    {
        rc.fromIOR = c.toIOR;
        rc.toIOR = c.fromIOR;
    }
    r.pdfBwd = evaluateSurface<true>(L, s, rc, wi, wo, kEvalPdfOnly, sp).pdf;
    return r;
}

// evaluateSubsurfaceExitAndPDFs (BDPTCommon.hlsl:463-472): forward the exit lobe; backward the
// density of reaching the entry point from the exit through the subsurface, an area density
// (the subsurface layer's probability for the reversed direction times the probe density)
YG_DEV ScatterEval evaluateExitBoth(const Surface& s, const SurfaceCtx& c, float curIOR, float prevIOR, float3 wo, float3 wi,
                                    bool front, bool fromLight, float3 exitPos, float3 exitN, float3 entryPos, float3 entryN)
{
    ScatterEval r;
    evaluateSubsurfaceExitLobe(s, c, wo, wi, fromLight ? kEvalLightPath : kEvalNone, r.weight, r.pdfFwd);
    SurfaceCtx rc;
    makeSurfaceCtx(s, curIOR, prevIOR, wi, front, rc);
    r.pdfBwd = rc.probs[LAYER_SSS] * pdfSubsurfaceExit(s, exitPos, exitN, entryPos, entryN);
    r.transmission = 0;
    return r;
}

// evaluateSubsurfaceEntry (scatteringSample.hlsl:67-79): forward an area density over the
// subsurface edge (used as is by the exit vertex), backward the exit lobe's density of wo
YG_DEV ScatterEval evaluateEntry(const Luts& L, const Spectral& sp, const Surface& s, const SurfaceCtx& c, float3 wo,
                                 const SubsurfaceExit& ex)
{
    ScatterEval r;
    r.weight = ex.weight * (subsurfaceEntryFactor(L, s, c, sp.hero) * ex.pdfPosition);
    r.pdfFwd = c.probs[LAYER_SSS] * ex.pdfPosition;
    float4 unused;
    evaluateSubsurfaceExitLobe(s, c, wo, wo, kEvalPdfOnly, unused, r.pdfBwd);
    r.transmission = 0;
    return r;
}

// the probe rays of a subsurface entry, out of line: only vertices on subsurface materials run it
static __device__ __noinline__ bool sampleExitOutOfLine(const SceneView& S, const Surface& s, const SurfacePoint& entry,
                                                        float4 r, SubsurfaceExit& out)
{
    return sampleSubsurfaceExit(S, s, entry, mk3(r.y, r.z, r.w), out);
}

// the ray-state part of evaluateSurfaceAndPDFs; returns whether this event dispersed first
YG_DEV bool applyTransmission(PathState& st, uint32_t trans, const Surface& s, uint32_t material)
{
    bool dispersed = false;
    if (trans != 0)
    {
        if (trans & kTransDispersed)
        {
            dispersed = (st.flags & kFlagSecondaryTerminated) == 0;
            st.flags |= kFlagSecondaryTerminated;
        }
        if (trans & kTransExited) exitedVolume(st, material);
        else if (trans & kTransEntered) enteredVolume(st, s.dielectricIOR, s.absorption, material);
    }
    return dispersed;
}

// absorption of the medium on the far side of a connection: the state applyTransmission
// would leave, read without changing the path state
YG_DEV float4 absorptionAfter(const PathState& st, uint32_t trans, const Surface& s, uint32_t material)
{
    if (trans & kTransExited)
    {
        if (st.nVol == 0) return splat4(0.0f);
        int index = -1;
        for (int i = (int)st.nVol - 1; i >= 0; --i)
            if (st.volMat[i] == material)
            {
                index = i;
                break;
            }
        if (index < 0 || index == (int)st.nVol - 1) return st.nVol > 1 ? st.volAbs[st.nVol - 2] : splat4(0.0f);
        return st.volAbs[st.nVol - 1];
    }
    if (trans & kTransEntered) return s.absorption;
    return st.nVol ? st.volAbs[st.nVol - 1] : splat4(0.0f);
}

YG_DEV float4 transmittance(float4 ab, float d)
{
    return mk4(ygm_expf(-ab.x * d), ygm_expf(-ab.y * d), ygm_expf(-ab.z * d), ygm_expf(-ab.w * d));
}

// sampleScatteringEvent (scatteringSample.hlsl:30-65): at a subsurface exit only the exit lobe;
// elsewhere a layer, and for the subsurface layer an exit point found by probe rays
enum : uint32_t
{
    kEventNone = 0,
    kEventLocal = 1,
    kEventEntry = 2,
    kEventExitLobe = 3
};
YG_DEV uint32_t sampleEvent(const SceneView& S, const Luts& L, const Spectral& sp, const Surface& s, const SurfaceCtx& c,
                            float3 wo, float4 r, bool atExit, const SurfacePoint& vertex, float3& wi, SubsurfaceExit& ex,
                            bool& isDiffuse, bool& isDelta)
{
    wi = mk3(0.f, 0.f, 0.f);
    isDiffuse = false;
    isDelta = false;
    if (atExit)
    {
        wi = sampleSubsurfaceExitLobe(s, c, wo, make_float2(r.z, r.w));
        isDiffuse = true;
        return isZero3(wi) ? kEventNone : kEventExitLobe;
    }
    int layer = selectMaterialLayer(r.x, c.probs);
    if (layer == LAYER_SSS)
    {
        isDiffuse = true;
        return sampleExitOutOfLine(S, s, vertex, r, ex) ? kEventEntry : kEventNone;
    }
    if (layer >= LAYER_COUNT) return kEventNone;
    wi = sampleLayerDirection<true>(L, s, c, layer, r.y, make_float2(r.z, r.w), sp.hero, isDiffuse, isDelta);
    return isZero3(wi) ? kEventNone : kEventLocal;
}

// makeSurfacePoint (BDPTCommon.hlsl:523-533): the vertex with its normal on the side of wo
YG_DEV SurfacePoint vertexPoint(float3 pos, float3 normalWS, float3 woWS, const Hit& hit)
{
    SurfacePoint p;
    p.pos = pos;
    p.normal = dot(woWS, normalWS) < 0.0f ? -normalWS : normalWS;
    p.instance = hit.instance;
    p.prim = hit.prim;
    p.b1 = hit.b1;
    p.b2 = hit.b2;
    p.front = hit.front;
    return p;
}

// calculateCommonSurfaceParams (BDPTCommon.hlsl:653-684) at a ray hit; the regularisation flag
// of the path state has been set by the caller
YG_DEV void vertexSurface(const SceneView& S, const LaunchParams& P, const Spectral& sp, const Hit& hit, const GpuInstance& I,
                          float3 rayDirWS, PathState& st, HitSurface& hs, SurfaceCtx& c)
{
    LaunchParams Pn = P;
    Pn.regularizeAfter = 0xffffffffu;
    st.pathLength = 0;
    setupSurface(S, Pn, sp, hit, I, rayDirWS, st, hs);
    const Surface& s = hs.s;
    if (dot(hs.rayDirOS, s.geometryNormal) > 0.0f && st.nVol == 0 && !isTwoSided(s.flags))
        enteredVolume(st, s.dielectricIOR, s.absorption, hs.material);
    makeSurfaceCtx(s, currentIOR(st), previousIOR(st), -hs.rayDirOS, hit.front, c);
}

YG_DEV void initState(PathState& st)
{
    st.throughput = splat4(1.0f);
    st.total = splat4(0.0f);
    st.pdfThisRay = 0.0f;
    st.flags = 0;
    st.pathLength = 0;
    st.nVol = 0;
}

// ------------------------------------------------------------------ light subpaths
// sampleLightOrEnv (BDPTCommon.hlsl:697-721) with sampleLight (lightSampling.hlsl:122-188)
// or sampleEnvironmentLighting (lightSampling.hlsl:78-118)
YG_DEV bool startLightPath(const SceneView& S, const LaunchParams& P, const BdptParams& B, const Spectral& sp, float pickR,
                           float4 r0, float2 r1, LightNode& n0, float4& radiance, float3& origin, float3& dir, float& pdfDir,
                           float& originPosPdf)
{
    const float envPdf = envSelectionPdf(S);
    float4 Le;
    float3 pos, n;
    float pdfPos, sel, profile;
    if (pickR < envPdf)
    {
        float st, ct, sph, cph;
        ygm_sincosf(r0.x * kPI, &st, &ct);
        ygm_sincosf(r0.y * 2.0f * kPI, &sph, &cph);
        dir = mk3(st * cph, st * sph, ct);
        pdfDir = safeDiv(1.0f, 2.0f * kPI * kPI * st);
        float3 v1, v2;
        vectorBase(dir, v1, v2);
        float2 cd = sampleConcentricDisk(make_float2(r0.z, r0.w));
        float radius = sqrtf(B.worldRadiusSqr);
        pos = B.worldCenter - dir * radius + (v1 * cd.x + v2 * cd.y) * radius;
        pdfPos = pdfEnvPosition(B);
        Le = skyRadiance(S, P, sp, -dir);
        n = dir;
        sel = envPdf;
        profile = 1.0f;
        n0.instance = 0xffffffffu;
        n0.prim = 0xffffffffu;
        n0.flags = NF_ENV;
    }
    else
    {
        uint32_t li = sampleLightIndex(S, (pickR - envPdf) / (1.0f - envPdf));
        sel = (1.0f - envPdf) * S.lights[li].selectionPdf;
        const GpuLight& PL = S.lights[li];
        if (PL.type != kLightMesh)
        {
            // samplePunctualLightEmission (lightSampling.hlsl:290-336) with random values (r1, r0.xy)
            Le = emissionSpectrum(S, sp, mk3(PL.intensity.x, PL.intensity.y, PL.intensity.z), -1);
            const float3 ax = mk3(PL.directionCosOuter.x, PL.directionCosOuter.y, PL.directionCosOuter.z);
            profile = 1.0f;
            if (PL.type == kLightDirectional)
            {
                float3 v1, v2;
                vectorBase(ax, v1, v2);
                float2 cd = sampleConcentricDisk(r1);
                float radius = sqrtf(B.worldRadiusSqr);
                pos = B.worldCenter - ax * radius + (v1 * cd.x + v2 * cd.y) * radius;
                dir = ax;
                pdfPos = pdfEnvPosition(B);
                pdfDir = 1.0f;
                n0.flags = NF_PUNCTUAL | NF_DIRECTIONAL;
            }
            else
            {
                pos = mk3(PL.positionCosInner.x, PL.positionCosInner.y, PL.positionCosInner.z);
                pdfPos = 1.0f;
                if (PL.type == kLightSpot)
                {
                    float3 v1, v2;
                    vectorBase(ax, v1, v2);
                    float3 loc = sampleUniformCone(r1, PL.directionCosOuter.w);
                    dir = normalize(v1 * loc.x + ax * loc.y + v2 * loc.z);
                    pdfDir = pdfUniformCone(PL.directionCosOuter.w);
                    profile = punctualFalloff(PL, dir);
                }
                else
                {
                    dir = sampleSphere(r1);
                    pdfDir = 1.0f / (4.0f * kPI);
                }
                n0.flags = NF_PUNCTUAL;
            }
            n = dir;
            n0.instance = 0xffffffffu;
            n0.prim = li;
        }
        else
        {
        LightPoint lp;
        sampleMeshLight(S, sp, li, mk3(r0.x, r0.y, r0.z), lp);
        const GpuInstance& LI = S.instances[lp.instance];
        float3 tangent = mk3(1.f, 0.f, 0.f);
        if (LI.hasTangents)
        {
            TriGeom g = fetchTri(S, LI, lp.prim);
            float bx = r0.x, by = r0.y;
            if (bx + by > 1.0f)
            {
                bx = 1.0f - bx;
                by = 1.0f - by;
            }
            float b0 = 1.0f - bx - by;
            float4 t1 = __ldg(S.tangents + g.i1), t2 = __ldg(S.tangents + g.i2), t3 = __ldg(S.tangents + g.i3);
            tangent = normalize(mk3(t1.x * t1.w, t1.y * t1.w, t1.z * t1.w) * b0 + mk3(t2.x * t2.w, t2.y * t2.w, t2.z * t2.w) * bx +
                                mk3(t3.x * t3.w, t3.y * t3.w, t3.z * t3.w) * by);
        }
        tangent = normalize(xformVectorT(LI.w2o, tangent));
        float3 ld = lp.twoSided ? sampleCosPowSphere(r1, lp.focus) : sampleCosPowHemi(r1, lp.focus);
        pdfDir = lp.twoSided ? pdfCosPowSphere(ld.y, lp.focus) : pdfCosPowHemi(ld.y, lp.focus);
        profile = evaluateEmissionProfile(ld.y, lp.focus);
        dir = fromLocal(constructBasis(lp.n, tangent), ld);
        pos = lp.pos;
        n = lp.n;
        pdfPos = lp.pdfPos;
        Le = lp.radiance;
        n0.instance = lp.instance;
        n0.prim = lp.prim;
        n0.flags = 0;
        }
    }
    if (allEqual4(Le, 0.0f) || pdfPos == 0.0f || pdfDir == 0.0f || sel == 0.0f) return false;
    n0.bary = make_float2(-1.0f, -1.0f);
    n0.normal = n;
    n0.radiance = Le;
    n0.pos = pos;
    n0.pdfFwd = (n0.flags & NF_ENV) ? pdfDir * sel : pdfPos * sel;
    n0.pdfBwd = 0.0f;
    n0.iorPrev = 1.0f;
    n0.iorCur = 1.0f;
    n0.pad = 0.0f;
    originPosPdf = pdfPos;
    origin = spawnRayOrigin(pos, n, dir);
    radiance = Le * profile * fabsf(dot(n, dir)) / (sel * pdfPos * pdfDir);
    return true;
}

// traceLightRays (BDPTTraceLightPath.comp:6-362): one thread per (sample index, light path)
__global__ void __launch_bounds__(128) bdptLightPaths(const SceneView S, const LaunchParams P, BdptParams B)
{
    const Luts Lt = bdptLuts(S);
    const uint32_t total = B.frames * B.lightPaths;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        const uint32_t f = t / B.lightPaths, l = t - f * B.lightPaths;
        LightNode* out = B.nodes + (size_t)t * B.maxLightVerts;
        RandomSampler rs{S.sobol + (size_t)f * kSobolDims, 2u, l ^ (P.seed * 0x9E3779B9u)};
        Spectral sp;
        spectralOf(S, S.lambdaMin + rs.r1() * (S.lambdaMax - S.lambdaMin), sp);
        B.heroes[t] = sp.hero;
        B.counts[t] = 0;
        float4 r0 = rs.r4(), r1 = rs.r4();
        LightNode nodes[2];
        float4 radiance;
        float3 rayOrigin, rayDir;
        float pdfForward, originPosPdf;
        if (!startLightPath(S, P, B, sp, r1.w, r0, make_float2(r1.x, r1.y), nodes[0], radiance, rayOrigin, rayDir, pdfForward,
                            originPosPdf))
            continue;
        const bool originEnv = (nodes[0].flags & NF_ENV) != 0;
        const bool originInfinite = (nodes[0].flags & NF_INFINITE) != 0;
        const bool originPunctual = (nodes[0].flags & NF_PUNCTUAL) != 0;
        const float maxRadiance = max4(radiance);
        uint32_t stored = 0;
        bool prevDelta = false;
        PathState st;
        initState(st);
        // set when the previous vertex took the subsurface event: the next vertex is its exit
        // point, reached without a ray (rayOrigin then holds the exit point, rayDir its inward
        // normal, so that wo is the outward normal)
        bool pendingExit = false;
        SubsurfaceExit pex;
        for (uint32_t i = 1; i < B.maxLightVerts; ++i)
        {
            float4 rv = rs.r4();
            Hit hit;
            const bool atExit = pendingExit;
            if (atExit)
            {
                hit.t = 0.0f;
                hit.b1 = pex.exit.b1;
                hit.b2 = pex.exit.b2;
                hit.instance = pex.exit.instance;
                hit.prim = pex.exit.prim;
                hit.front = pex.exit.front;
                pendingExit = false;
            }
            else if (!traceClosest<false>(S, rayOrigin, rayDir, kRayMinT, __int_as_float(0x7f800000), hit, nullptr))
                break;
            LightNode& cur = nodes[i & 1];
            LightNode& prev = nodes[(i - 1) & 1];
            const GpuInstance& I = S.instances[hit.instance];
            if (P.regularizeEnable && i - 1 >= P.regularizeAfter) st.flags |= kFlagRegularize;
            uint32_t nflags = hit.front ? NF_FRONT : 0u;
            nflags |= (st.flags & kFlagSecondaryTerminated) ? NF_TERMINATED : 0u;
            nflags |= (st.flags & kFlagRegularize) ? NF_REGULARIZED : 0u;
            nflags |= atExit ? NF_SSS_EXIT : 0u;
            HitSurface hs;
            SurfaceCtx c;
            vertexSurface(S, P, sp, hit, I, rayDir, st, hs, c);
            const Surface& s = hs.s;
            // a subsurface exit has only the exit lobe
            if (!atExit && isDeltaDistribution(c.a2, s)) nflags |= NF_DELTA;
            float3 normalWS = normalize(xformVectorT(I.w2o, s.geometryNormal));
            // exit nodes keep the outward normal; connections set their surface up from it
            if (atExit && dot(-rayDir, normalWS) < 0.0f) normalWS = -normalWS;
            float3 posWS = rayOrigin + rayDir * hit.t;
            float pdfFwdMIS;
            if (atExit)
            {
                pdfFwdMIS = pdfForward; // the subsurface edge's density is an area density already
            }
            else
            {
                if (i == 1 && originInfinite) pdfFwdMIS = originPosPdf * fabsf(dot(rayDir, normalWS));
                else pdfFwdMIS = prevDelta ? -1.0f : pdfForward * solidAngleToArea(posWS - rayOrigin, normalWS);
                float4 ab = st.nVol ? st.volAbs[st.nVol - 1] : splat4(0.0f);
                if (!allEqual4(ab, 0.0f)) radiance = radiance * transmittance(ab, hit.t);
            }
            cur.instance = hit.instance;
            cur.prim = hit.prim;
            cur.bary = make_float2(hit.b1, hit.b2);
            cur.normal = normalWS;
            cur.radiance = radiance;
            cur.pos = posWS;
            cur.pdfFwd = pdfFwdMIS;
            cur.pdfBwd = 0.0f;
            cur.iorPrev = previousIOR(st);
            cur.iorCur = currentIOR(st);
            cur.flags = nflags;
            cur.pad = 0.0f;
            bool isDiffuse, sDelta;
            float3 wo = -hs.rayDirOS;
            float3 wi;
            SubsurfaceExit nex;
            const uint32_t event = sampleEvent(S, Lt, sp, s, c, wo, rv, atExit, vertexPoint(posWS, normalWS, -rayDir, hit), wi, nex,
                                               isDiffuse, sDelta);
            if (event == kEventNone) break;
            if (isDiffuse) st.flags |= kFlagRegularize;
            ScatterEval ev;
            if (event == kEventEntry) ev = evaluateEntry(Lt, sp, s, c, wo, nex);
            else if (event == kEventExitLobe)
                ev = evaluateExitBoth(s, c, currentIOR(st), previousIOR(st), wo, wi, hit.front, true, posWS, normalWS, prev.pos,
                                      prev.normal);
            else ev = evaluateBoth(Lt, sp, s, c, currentIOR(st), previousIOR(st), wo, wi, hit.front, true, sDelta);
            bool dispersed = applyTransmission(st, ev.transmission, s, hs.material);
            pdfForward = ev.pdfFwd;
            float4 w = ev.weight * safeDiv(1.0f, pdfForward);
            if (event == kEventExitLobe) prev.pdfBwd = ev.pdfBwd; // an area density
            else prev.pdfBwd = sDelta ? -1.0f : ev.pdfBwd * solidAngleToArea(rayOrigin - posWS, prev.normal);
            if (i == 1 && originPunctual) prev.pdfBwd = 0.0f; // a camera path never hits a delta light
            else if (i == 1 && originEnv && !sDelta) prev.pdfBwd = ev.pdfBwd;
            out[stored++] = prev;
            radiance = radiance * w;
            if (dispersed) terminateSecondary(radiance);
            // applyRussianRoulette normalised by the emitted radiance
            float p = clampf(max4(radiance) / maxRadiance, 0.05f, 1.0f);
            if (rs.r1() > p) break;
            radiance = radiance * (1.0f / p);
            if (allEqual4(radiance, 0.0f)) break;
            if (event == kEventEntry)
            {
                pendingExit = true;
                pex = nex;
                rayOrigin = nex.exit.pos;
                rayDir = -nex.exit.normal;
            }
            else
            {
                rayDir = normalize(xformVectorT(I.w2o, wi));
                rayOrigin = spawnRayOrigin(posWS, normalWS, rayDir);
            }
            prevDelta = sDelta;
        }
        // the last vertex reached (BDPTTraceLightPath.comp:335-352)
        out[stored] = nodes[stored & 1];
        B.counts[t] = stored + 1;
    }
}

// per sample index, the light paths that stored vertices in ascending index order (the headers)
__global__ void __launch_bounds__(1024) bdptHeaders(BdptParams B)
{
    const uint32_t f = blockIdx.x;
    const uint32_t* cnt = B.counts + (size_t)f * B.lightPaths;
    uint32_t* out = B.valid + (size_t)f * B.lightPaths;
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t c0 = 0; c0 < B.lightPaths; c0 += blockDim.x)
    {
        uint32_t i = c0 + threadIdx.x;
        uint32_t v = (i < B.lightPaths && cnt[i] > 0) ? 1u : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) warpSums[w] = x;
        __syncthreads();
        if (w == 0)
        {
            uint32_t s = lane < nw ? warpSums[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1)
            {
                uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= (uint32_t)o) s += y;
            }
            warpSums[lane] = s;
        }
        __syncthreads();
        uint32_t excl = base + (w ? warpSums[w - 1] : 0u) + x - v;
        if (v) out[excl] = i;
        uint32_t blockTotal = warpSums[nw - 1];
        __syncthreads();
        if (threadIdx.x == 0) base += blockTotal;
        __syncthreads();
    }
    if (threadIdx.x == 0) B.validCount[f] = base;
}

// ------------------------------------------------------------------ camera subpaths + connections
// ExtractedLightPathNodeData (BDPTCommon.hlsl:69-74) with the spectral surface and the forward
// shading frame of the vertex, which depend only on the light path
struct SharedNode
{
    LightNode n;
    Surface s;
    SurfaceCtx c;
    float4 w2o[3];
    float3 prevPos, prevNormal; // the previous vertex (the entry point of a subsurface exit)
    float3 woOS;
    uint32_t material;
    float emissionFocus;
    uint32_t twoSided;
    // the light subpath's MIS context of a connection to this vertex (LightVertexContext of
    // traceCameraRays, which depends on the light path only): the ratio sum of the vertices
    // before the previous one, the previous vertex, and the flags of the path's origin
    float lvRiSum, lvPrevPdfFwd;
    float3 lvPrevPos, lvPrevNormal;
    uint32_t lvPrevFlags, lvOriginFlags;
};

YG_DEV void prepareSharedNode(const SceneView& S, const LaunchParams& P, const Spectral& sp, const LightNode& src,
                              float3 prevPos, float3 prevNormal, uint32_t index, SharedNode& d)
{
    d.n = src;
    d.prevPos = prevPos;
    d.prevNormal = prevNormal;
    if (src.flags & (NF_ENV | NF_PUNCTUAL)) return; // light origins without a surface
    const GpuInstance& I = S.instances[src.instance];
    d.w2o[0] = I.w2o[0];
    d.w2o[1] = I.w2o[1];
    d.w2o[2] = I.w2o[2];
    d.material = I.material;
    const GpuMaterial& M = S.materials[I.material];
    d.emissionFocus = M.emissionFocus;
    d.twoSided = M.mask & 1u;
    if (index == 0) return;
    // fillSurfaceDefRGB + regularizeMaterial + convertSurfaceDefinitionFromRGB, no two-sided
    // orientation (BDPTCommon.hlsl:845-869); a subsurface exit is oriented to wo, its stored
    // outward normal (BDPTCommon.hlsl:800-823)
    Hit h;
    h.instance = src.instance;
    h.prim = src.prim;
    h.b1 = src.bary.x;
    h.b2 = src.bary.y;
    h.front = (src.flags & NF_FRONT) != 0;
    h.t = 0.0f;
    PathState st;
    initState(st);
    if (src.flags & NF_REGULARIZED) st.flags |= kFlagRegularize;
    LaunchParams Pn = P;
    Pn.regularizeAfter = 0xffffffffu;
    HitSurface hs;
    const bool exitNode = (src.flags & NF_SSS_EXIT) != 0;
    setupSurface(S, Pn, sp, h, I, exitNode ? -src.normal : src.normal, st, hs, exitNode);
    d.s = hs.s;
    if (exitNode)
    {
        d.woOS = normalize(xformVector(I.w2o, src.normal));
    }
    else
    {
        float3 lpos = xformPoint(I.w2o, src.pos);
        float3 ppos = xformPoint(I.w2o, prevPos);
        d.woOS = normalize(ppos - lpos);
    }
    makeSurfaceCtx(d.s, src.iorCur, src.iorPrev, d.woOS, h.front, d.c);
}

// calculateConnectingLightNodeWeightsAndPDFs (BDPTCommon.hlsl:725-876) for the light end of a
// connection to nextPos; returns false when the connection carries nothing
YG_DEV bool lightEndOfConnection(const SceneView& S, const BdptParams& B, const Luts& Lt, const Spectral& sp,
                                 const SharedNode& sn, uint32_t index, float3 nextPos, bool alreadyTerminated,
                                 ScatterEval& ev, float& pdfFwdMIS)
{
    const LightNode& n = sn.n;
    ev.weight = splat4(0.0f);
    ev.pdfFwd = 0.0f;
    ev.pdfBwd = 0.0f;
    ev.transmission = 0;
    if (index == 0 && (n.flags & NF_PUNCTUAL))
    {
        // node radiance is intensity (point, spot) or irradiance (directional): no area density
        const GpuLight& L = S.lights[n.prim];
        const float pick = (1.0f - envSelectionPdf(S)) * L.selectionPdf;
        if (L.type == kLightDirectional)
        {
            ev.pdfFwd = pick;
            ev.weight = splat4(1.0f / pick);
            pdfFwdMIS = pdfEnvPosition(B); // planar density; the cosine at the next vertex is the caller's
        }
        else
        {
            float3 fl = nextPos - n.pos;
            float d2 = fmaxf(dot(fl, fl), 1e-10f);
            float3 fd = fl * (1.0f / sqrtf(d2));
            float fall = punctualFalloff(L, fd);
            if (fall <= 0.0f)
            {
                pdfFwdMIS = 0.0f;
                return false;
            }
            ev.pdfFwd = pick * d2;
            ev.weight = splat4(fall / ev.pdfFwd);
            // pdfPunctualLightEmissionDirection (lightSampling.hlsl:280-288)
            if (L.type == kLightSpot)
                pdfFwdMIS = dot(fd, mk3(L.directionCosOuter.x, L.directionCosOuter.y, L.directionCosOuter.z)) >= L.directionCosOuter.w
                                ? pdfUniformCone(L.directionCosOuter.w)
                                : 0.0f;
            else
                pdfFwdMIS = 1.0f / (4.0f * kPI);
        }
        ev.pdfBwd = 0.0f;
        return true;
    }
    if (index == 0 && (n.flags & NF_ENV))
    {
        float pdfDir = envSelectionPdf(S) * pdfEnvDirection(n.normal);
        if (pdfDir <= 0.0f)
        {
            pdfFwdMIS = 0.0f;
            return false;
        }
        ev.pdfFwd = pdfDir;
        ev.weight = splat4(1.0f / pdfDir);
        pdfFwdMIS = pdfEnvPosition(B);
        return true;
    }
    if (index == 0)
    {
        float3 fromLight = nextPos - n.pos;
        if (dot(fromLight, n.normal) <= 0.0f && !sn.twoSided)
        {
            pdfFwdMIS = 0.0f;
            return false;
        }
        ev.pdfFwd = n.pdfFwd * (1.0f / solidAngleToArea(-fromLight, n.normal));
        float cosE = dot(n.normal, normalize(fromLight));
        ev.weight = splat4(safeDiv(evaluateEmissionProfile(cosE, sn.emissionFocus), ev.pdfFwd));
        pdfFwdMIS = sn.twoSided ? pdfCosPowSphere(cosE, sn.emissionFocus)
                                : (cosE >= 0.0f ? pdfCosPowHemi(cosE, sn.emissionFocus) : 0.0f);
        return true;
    }
    float3 lpos = xformPoint(sn.w2o, n.pos);
    float3 cpos = xformPoint(sn.w2o, nextPos);
    float3 wi = normalize(cpos - lpos);
    bool front = (n.flags & NF_FRONT) != 0;
    if (n.flags & NF_SSS_EXIT)
    {
        // the exit lobe; the backward density is an area density over the subsurface edge
        ev = evaluateExitBoth(sn.s, sn.c, n.iorCur, n.iorPrev, sn.woOS, wi, front, true, n.pos, n.normal, sn.prevPos,
                              sn.prevNormal);
        pdfFwdMIS = ev.pdfFwd;
        return !(ev.pdfBwd == 0.0f || allEqual4(ev.weight, 0.0f));
    }
    ev = evaluateBoth(Lt, sp, sn.s, sn.c, n.iorCur, n.iorPrev, sn.woOS, wi, front, true, false);
    bool terminated = alreadyTerminated || (n.flags & NF_TERMINATED);
    if ((ev.transmission & kTransDispersed) && !terminated) terminateSecondary(ev.weight);
    pdfFwdMIS = ev.pdfFwd;
    return !(ev.pdfBwd == 0.0f || allEqual4(ev.weight, 0.0f));
}

struct CamVertex
{
    float3 pos, normal, prevPos, prevNormal;
    float pdfRatioSum, prevPdfFwd, curPdfFwd;
    bool isExit, prevIsExit; // reached through the subsurface (no ray led to the vertex)
};
struct LightVertexCtx
{
    float3 prevPos, prevNormal;
    float prevPdfFwd, riSum;
    uint32_t originFlags, prevFlags;
};

// calculateMISWeight (BDPTCommon.hlsl:918-1006)
YG_DEV float misWeight(const SceneView& S, uint32_t camIndex, const CamVertex& cv, uint32_t lightIndex,
                       const LightVertexCtx& lv, const LightNode& ln, float fwdCam, float bwdCam, float fwdLight, float bwdLight)
{
    float riCam = cv.pdfRatioSum;
    if (camIndex > 0)
    {
        // from a subsurface exit the backward density is an area density already
        float bwd = cv.isExit ? bwdCam : bwdCam * solidAngleToArea(cv.prevPos - cv.pos, cv.prevNormal);
        riCam = accumulateRISum(riCam, bwd, cv.prevPdfFwd, !cv.prevIsExit);
    }
    const bool env0 = lightIndex == 0 && (ln.flags & NF_ENV);
    const bool inf0 = lightIndex == 0 && (ln.flags & NF_INFINITE);
    float toCamArea = inf0 ? fwdLight * fabsf(dot(cv.normal, ln.normal)) : fwdLight * solidAngleToArea(cv.pos - ln.pos, cv.normal);
    riCam = accumulateRISum(riCam, toCamArea, cv.curPdfFwd, !cv.isExit);
    float riLight = lv.riSum;
    if (lightIndex == 0)
    {
        float pick, posPdf, dirPdf, toLight;
        if (ln.flags & NF_PUNCTUAL)
        {
            // a camera path never hits a delta light
            pick = 1.0f;
            posPdf = 1.0f;
            toLight = 0.0f;
        }
        else if (env0)
        {
            pick = envSelectionPdf(S);
            posPdf = pdfEnvDirection(ln.normal);
            toLight = fwdCam;
        }
        else
        {
            float3 camToLight = ln.pos - cv.pos;
            float len = length(camToLight);
            pdfForSamplingLight(S, ln.instance, ln.prim, ln.normal, -camToLight / len, pick, posPdf, dirPdf);
            toLight = fwdCam * solidAngleToArea(camToLight, ln.normal);
        }
        riLight = pdfRatio(toLight, pick * posPdf);
    }
    else
    {
        float bwdPrev = bwdLight;
        const bool lnExit = (ln.flags & NF_SSS_EXIT) != 0;
        const bool prevExit = (lv.prevFlags & NF_SSS_EXIT) != 0;
        bool prevEnv = lightIndex == 1 && (lv.originFlags & NF_ENV);
        bool prevPunctual = lightIndex == 1 && (lv.originFlags & NF_PUNCTUAL);
        if (prevPunctual) bwdPrev = 0.0f;
        else if (!prevEnv && !lnExit) bwdPrev *= solidAngleToArea(lv.prevPos - ln.pos, lv.prevNormal);
        riLight = accumulateRISum(riLight, bwdPrev, lv.prevPdfFwd, !prevExit);
        riLight = accumulateRISum(riLight, fwdCam * solidAngleToArea(ln.pos - cv.pos, ln.normal), ln.pdfFwd, !lnExit);
    }
    return 1.0f / (1.0f + riCam + riLight);
}

// ------------------------------------------------------------------ camera subpaths as a wavefront
// traceCameraRays (BDPTTraceCameraPath.comp:40-432) split into stages over a wave of camera
// paths, one bounce at a time: trace the camera rays; shade each vertex (emitter or
// environment term, or one connection record per light vertex with its contribution and
// visibility ray, then the scattered continuation); trace the visibility rays; add each
// path's visible connections in light-vertex order. The sums are formed in the same order as
// the one-thread-per-path loop of the reference (vertex by vertex, light vertex by light
// vertex), so a sample does not depend on the staging.
//
// A camera group is 64 consecutive entries of the pixel permutation; its light path is
// picked per (sample index, group) as in the reference. The light vertices' spectral surfaces
// and forward frames are prepared once per wave in global memory (they depend only on the
// light path and its hero wavelength, which the group shares).
// a connecting camera vertex as its connections read it (calculateLightPathRadiance's camera
// side: CameraVertexContext and the ray state at the vertex)
struct alignas(16) ConnVertex
{
    float4 thr;       // throughput at the vertex
    float4 absNone;   // absorption along a connection that stays in the current medium
    float4 absExited; // and along one whose camera end leaves it
    float3 pos;
    uint32_t flags; // path flags at the vertex, kWbAtExit / kWbPrevExit
    float3 normal;
    float curPdfFwd;
    float3 prevPos;
    float pdfRatioSum;
    float3 prevNormal;
    float prevPdfFwd;
    float3 wo; // object space
    float hero;
    float curIOR, prevIOR;
    uint32_t instance, front;
};

struct BdptWave
{
    uint64_t c0;         // first camera path (frame * cropPixels + permutation slot) of the wave
    uint32_t n;          // paths in the wave
    uint32_t fBase;      // first frame the wave touches (prepared nodes start there)
    uint32_t capacity;
    SharedNode* prep;    // [(frame - fBase) * lightPaths + path] * maxLightVerts + vertex
    float4* thr;         // path throughput
    float4* tot;         // camera-path radiance so far
    float4* cv0;         // previous vertex position, pdf ratio sum
    float4* cv1;         // previous vertex normal, its forward area pdf
    float4* cv2;         // deferred ratio sum, forward pdf of the current ray, hero wavelength
    uint4* misc;         // flags | volumes << 16, sampler dimension, sampler seed, frame
    uint4* misc2;        // permutation slot pixel, light path, light vertex count
    uint2* conn;         // this bounce's connection records: first, count
    float4* exitHit;     // a pending subsurface exit: barycentrics, instance, primitive | front << 31
    Surface* camSurf;    // a connecting camera vertex: its surface and frames,
    SurfaceCtx* camCtx;
    struct ConnVertex* cvx; // and the rest of its state the connections read
    uint2* connSlot;     // per connection record: camera path slot, light vertex
    float4* volIOR;
    uint4* volMat;
    float4* volAbs;      // [k * capacity + slot]
    float4* fhAlb;
    float4* fhNrm;
    ShadowQueue C;       // connection records (o.w = path slot, d.w = tmax, < 0: no ray)
    uint8_t* vis;        // visibility of each record
    uint32_t* connCount;
};

constexpr uint32_t kNoLightPath = 0xffffffffu;

__device__ __forceinline__ void wbLoadVolumes(const BdptWave& W, uint32_t s, PathState& st)
{
    if (!st.nVol) return;
    float4 vi = W.volIOR[s];
    uint4 vm = W.volMat[s];
    st.volIOR[0] = vi.x, st.volIOR[1] = vi.y, st.volIOR[2] = vi.z, st.volIOR[3] = vi.w;
    st.volMat[0] = vm.x, st.volMat[1] = vm.y, st.volMat[2] = vm.z, st.volMat[3] = vm.w;
    for (int k = 0; k < kMaxVolumes; ++k) st.volAbs[k] = W.volAbs[(size_t)k * W.capacity + s];
}
__device__ __forceinline__ void wbStoreVolumes(const BdptWave& W, uint32_t s, const PathState& st)
{
    W.volIOR[s] = mk4(st.volIOR[0], st.volIOR[1], st.volIOR[2], st.volIOR[3]);
    W.volMat[s] = make_uint4(st.volMat[0], st.volMat[1], st.volMat[2], st.volMat[3]);
    for (int k = 0; k < kMaxVolumes; ++k) W.volAbs[(size_t)k * W.capacity + s] = st.volAbs[k];
}

// consecutive records for every lane of the warp: n per lane, one atomic per warp
__device__ __forceinline__ uint32_t warpReserve(uint32_t* counter, uint32_t n)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t inc = n;
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += u;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + inc - n;
}

// the light vertices of every light path the wave's frames can pick
__global__ void __launch_bounds__(128) wbPrepare(const SceneView S, const LaunchParams P, BdptParams B, BdptWave W,
                                                uint32_t frames)
{
    const uint64_t total = (uint64_t)frames * B.lightPaths * B.maxLightVerts;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t k = (uint32_t)(i % B.maxLightVerts);
        const uint64_t fl = i / B.maxLightVerts;
        const uint32_t l = (uint32_t)(fl % B.lightPaths), fi = (uint32_t)(fl / B.lightPaths);
        const uint32_t f = W.fBase + fi;
        const size_t pl = (size_t)f * B.lightPaths + l;
        if (k >= B.counts[pl]) continue;
        Spectral sp;
        spectralOf(S, B.heroes[pl], sp);
        const LightNode* src = B.nodes + pl * B.maxLightVerts;
        SharedNode& d = W.prep[i];
        prepareSharedNode(S, P, sp, src[k], k ? src[k - 1].pos : src[0].pos, k ? src[k - 1].normal : src[0].normal, k, d);
        float ri = 0.0f;
        for (uint32_t j = 0; j + 1 < k; ++j) ri = accumulateRISum(ri, src[j].pdfBwd, src[j].pdfFwd, !(src[j].flags & NF_SSS_EXIT));
        d.lvRiSum = ri;
        d.lvPrevPos = k ? src[k - 1].pos : mk3(0.f, 0.f, 0.f);
        d.lvPrevNormal = k ? src[k - 1].normal : mk3(0.f, 0.f, 0.f);
        d.lvPrevPdfFwd = k ? src[k - 1].pdfFwd : 0.0f;
        d.lvPrevFlags = k ? src[k - 1].flags : 0u;
        d.lvOriginFlags = k ? src[0].flags : 0u;
    }
}

__global__ void __launch_bounds__(128) wbGenerate(const SceneView S, const LaunchParams P, BdptParams B, BdptWave W, RayQueue Q)
{
    const uint64_t cropPix = (uint64_t)P.cropW * P.cropH;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < W.n; s += gridDim.x * blockDim.x)
    {
        const uint64_t c = W.c0 + s;
        const uint32_t f = (uint32_t)(c / cropPix);
        const uint32_t slotInFrame = (uint32_t)(c % cropPix);
        const uint32_t pix = B.perm[slotInFrame];
        const uint32_t px = P.cropX + pix % P.cropW, py = P.cropY + pix / P.cropW;
        const uint32_t* point = S.sobol + (size_t)f * kSobolDims;
        const uint32_t seed = (py * P.width + px) ^ (P.seed * 0x9E3779B9u);
        RandomSampler rs{point, B.camDimOffset + 2u, seed};
        const float2 lensR = rs.r2();
        const uint32_t g = slotInFrame / kGroupSize, j = slotInFrame % kGroupSize;
        const uint32_t hc = B.validCount[f];
        uint32_t path = kNoLightPath, count = 0;
        float hero;
        if (hc == 0)
        {
            // the group's first pixel draws the wavelength with its next dimension
            const uint32_t pix0 = B.perm[(size_t)g * kGroupSize];
            const uint32_t px0 = P.cropX + pix0 % P.cropW, py0 = P.cropY + pix0 / P.cropW;
            RandomSampler r0{point, B.camDimOffset + 4u, (py0 * P.width + px0) ^ (P.seed * 0x9E3779B9u)};
            hero = S.lambdaMin + r0.r1() * (S.lambdaMax - S.lambdaMin);
            if (j == 0) rs.r1();
        }
        else
        {
            RandomSampler rt{point, 2u, g ^ (P.seed * 0x9E3779B9u)};
            uint32_t h = (uint32_t)fminf(floorf(rt.r1() * (float)hc), (float)(hc - 1u));
            // the headers are in light-path order, so header h would be the path whose hero
            // wavelength was drawn from the same Sobol dimension with the seed h: a per-sample
            // rotation (a hash of the sample index) keeps the chosen wavelength uniform, as the
            // reference's atomically ordered headers do
            h = (h + hash2(P.sppStart + f, P.seed ^ 0x2545F491u) % hc) % hc;
            path = B.valid[(size_t)f * B.lightPaths + h];
            count = B.counts[(size_t)f * B.lightPaths + path];
            hero = B.heroes[(size_t)f * B.lightPaths + path];
        }
        // generateCameraRay (raytraceCommonResources.hlsl:113-137) with the group's wavelength
        float invW = 1.0f / (float)P.width, invH = 1.0f / (float)P.height;
        float2 uv = make_float2((float)px * invW + 0.5f * invW, (float)py * invH + 0.5f * invH);
        float2 texel = make_float2(sampleDim(point, 0, seed), sampleDim(point, 1, seed));
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
        float3 rayOrigin = mk3(ow.x, ow.y, ow.z);
        float3 rayDir = normalize(mk3(dw.x, dw.y, dw.z));
        W.thr[s] = splat4(1.0f);
        W.tot[s] = splat4(0.0f);
        W.cv0[s] = splat4(0.0f);
        W.cv1[s] = splat4(0.0f);
        W.cv2[s] = mk4(0.0f, cameraDirectionalPdf(S, P, rayDir), hero, 0.0f);
        W.misc[s] = make_uint4(0u, rs.dim, rs.seed, f);
        W.misc2[s] = make_uint4(pix, path, count, 0u);
        if (P.featAlbedo)
        {
            W.fhAlb[s] = splat4(0.0f);
            W.fhNrm[s] = splat4(0.0f);
        }
        Q.o[s] = mk4(rayOrigin.x, rayOrigin.y, rayOrigin.z, __uint_as_float(s));
        Q.d[s] = mk4(rayDir.x, rayDir.y, rayDir.z, 0.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *Q.count = W.n;
}

// closest hits of the queued camera rays; a queued subsurface exit (d.w = 1) is not traced, its
// hit is the exit point stored by the vertex that took the subsurface event
__global__ void __launch_bounds__(128, YG_TRACE_MIN_BLOCKS) wbTrace(const SceneView S, RayQueue Q, HitQueue H, const float4* exitHit)
{
    TraversalCount tc{0, 0};
    uint32_t rays = 0;
    traceGrid<false>(
        *Q.count,
        [&](TraceState& t, uint32_t i) {
            const float4 o = Q.o[i], d = Q.d[i];
            traceBegin(t, S, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), kRayMinT, d.w != 0.0f ? 0.0f : __int_as_float(0x7f800000));
        },
        [&](const TraceState& t, uint32_t i) {
            if (Q.d[i].w != 0.0f)
            {
                const float4 e = exitHit[__float_as_uint(Q.o[i].w)];
                H.a[i] = mk4(0.0f, e.x, e.y, e.z);
                H.b[i] = __float_as_uint(e.w);
                return;
            }
            H.a[i] = mk4(t.h.t, t.h.b1, t.h.b2, __uint_as_float(t.h.instance));
            H.b[i] = t.found ? (t.h.prim | (t.h.front ? 0x80000000u : 0u)) : 0xffffffffu;
        },
        tc, rays);
}

// one camera vertex per queued path (the body of the bounce loop of traceCameraRays)
#ifndef YG_WBSHADE_MIN_BLOCKS
#define YG_WBSHADE_MIN_BLOCKS 1
#endif
__global__ void __launch_bounds__(128, YG_WBSHADE_MIN_BLOCKS) wbShade(const SceneView S, const LaunchParams P, BdptParams B, BdptWave W,
                                              RayQueue Qin, HitQueue H, RayQueue Qout, uint32_t ci)
{
    const Luts Lt = bdptLuts(S);
    const uint32_t n = *Qin.count;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r)
    {
        const uint32_t i = first + r * stride;
        const bool active = i < n;
        uint32_t s = 0, count = 0, f = 0;
        bool connect = false, alive = false;
        PathState st;
        RandomSampler rs;
        Spectral sp;
        CamVertex cv;
        float deferredRI = 0.0f, pdfFwdCam = 0.0f;
        float3 rayOrigin = mk3(0.f, 0.f, 0.f), rayDir = mk3(0.f, 0.f, 1.f);
        Hit hit;
        HitSurface hs;
        SurfaceCtx c;
        const GpuInstance* I = nullptr;
        bool delta = true;
        float4 total = splat4(0.0f);
        float4 rv = splat4(0.0f);
        if (active)
        {
            const float4 qo = Qin.o[i], qd = Qin.d[i];
            s = __float_as_uint(qo.w);
            rayOrigin = mk3(qo.x, qo.y, qo.z);
            rayDir = mk3(qd.x, qd.y, qd.z);
            const uint4 m = W.misc[s], m2 = W.misc2[s];
            f = m.w;
            count = m2.z;
            initState(st);
            st.throughput = W.thr[s];
            st.flags = m.x & 0x0fffu;
            st.nVol = m.x >> 16;
            cv.isExit = (m.x & kWbAtExit) != 0;
            cv.prevIsExit = (m.x & kWbPrevExit) != 0;
            wbLoadVolumes(W, s, st);
            rs = RandomSampler{S.sobol + (size_t)f * kSobolDims, m.y, m.z};
            const float4 a = W.cv0[s], b = W.cv1[s], e = W.cv2[s];
            cv.prevPos = mk3(a.x, a.y, a.z);
            cv.pdfRatioSum = a.w;
            cv.prevNormal = mk3(b.x, b.y, b.z);
            cv.prevPdfFwd = b.w;
            deferredRI = e.x;
            pdfFwdCam = e.y;
            spectralOf(S, e.z, sp);
            total = W.tot[s];
            const float4 ha = H.a[i];
            const uint32_t hb = H.b[i];
            const bool found = hb != 0xffffffffu;
            hit.t = ha.x;
            hit.b1 = ha.y;
            hit.b2 = ha.z;
            hit.instance = __float_as_uint(ha.w);
            hit.prim = hb & 0x7fffffffu;
            hit.front = (hb & 0x80000000u) != 0;
            rv = rs.r4();
            if (!found)
            {
                // calculateMISWeightOnCameraPathMissing (BDPTCommon.hlsl:1039-1059)
                cv.curPdfFwd = pdfFwdCam;
                float mis = 1.0f;
                if (ci > 0)
                {
                    float ri = accumulateRISum(cv.pdfRatioSum, pdfEnvPosition(B) * fabsf(dot(cv.prevNormal, rayDir)), cv.prevPdfFwd,
                                               !cv.prevIsExit);
                    ri = accumulateRISum(ri, envSelectionPdf(S) * pdfEnvDirection(-rayDir), cv.curPdfFwd);
                    mis = 1.0f / (1.0f + ri);
                }
                total = total + st.throughput * skyRadiance(S, P, sp, rayDir) * mis;
            }
            else
            {
                I = &S.instances[hit.instance];
                if (P.regularizeEnable && ci >= P.regularizeAfter) st.flags |= kFlagRegularize;
                vertexSurface(S, P, sp, hit, *I, rayDir, st, hs, c);
                const Surface& sf = hs.s;
                cv.pos = rayOrigin + rayDir * hit.t;
                cv.normal = normalize(xformVectorT(I->w2o, sf.geometryNormal));
                if (ci == 0 && P.featAlbedo)
                {
                    float3 nn = normalize(xformVectorT(I->w2o, sf.baseLayerNormal));
                    float4 vp = mul44(S.cam.worldToView, mk4(cv.pos.x, cv.pos.y, cv.pos.z, 1.0f));
                    W.fhAlb[s] = mk4(hs.albedoRGB.x, hs.albedoRGB.y, hs.albedoRGB.z, 0.0f);
                    W.fhNrm[s] = mk4(nn.x, nn.y, nn.z, vp.z * S.cam.forwardZSign);
                }
                // a subsurface exit has only the exit lobe, and the density of reaching it is an
                // area density already; its emission was accounted for at the entry point
                delta = !cv.isExit && isDeltaDistribution(c.a2, sf);
                if (cv.isExit)
                {
                    cv.curPdfFwd = pdfFwdCam;
                }
                else
                {
                    cv.curPdfFwd = pdfFwdCam < 0.0f ? -1.0f : pdfFwdCam * solidAngleToArea(cv.pos - rayOrigin, cv.normal);
                    float4 ab = st.nVol ? st.volAbs[st.nVol - 1] : splat4(0.0f);
                    if (!allEqual4(ab, 0.0f)) st.throughput = st.throughput * transmittance(ab, hit.t);
                }
                if (!cv.isExit && !allEqual4(sf.emissive, 0.0f))
                {
                    // calculateMISWeightOnCameraPathHittingLight (BDPTCommon.hlsl:1008-1035)
                    float mis = 1.0f;
                    if (ci > 0)
                    {
                        float3 towards = cv.prevPos - cv.pos;
                        float pick, posPdf, dirPdf;
                        pdfForSamplingLight(S, hit.instance, hit.prim, cv.normal, normalize(towards), pick, posPdf, dirPdf);
                        float ri = accumulateRISum(cv.pdfRatioSum, dirPdf * solidAngleToArea(towards, cv.prevNormal), cv.prevPdfFwd,
                                                   !cv.prevIsExit);
                        ri = accumulateRISum(ri, pick * posPdf, cv.curPdfFwd);
                        mis = 1.0f / (1.0f + ri);
                    }
                    if (isTwoSided(sf.flags) || dot(sf.geometryNormal, -hs.rayDirOS) > 0.0f)
                    {
                        float profile = evaluateEmissionProfile(dot(cv.normal, -rayDir), sf.emissionFocus);
                        total = total + st.throughput * sf.emissive * mis * profile;
                    }
                }
                else
                {
                    connect = !delta && !allEqual4(st.throughput, 0.0f) && count > 0;
                    alive = true;
                }
            }
            if (!alive) W.tot[s] = total; // the path ends at this vertex
        }
        // connection records: count per connecting path, consecutive per path (neighbouring
        // threads of wbConnect then read the same camera vertex); the connections themselves
        // are evaluated by wbConnect, one thread per record
        const uint32_t base = warpReserve(W.connCount, connect ? count : 0u);
        if (active) W.conn[s] = make_uint2(base, connect ? count : 0u);
        if (connect)
        {
            W.camSurf[s] = hs.s;
            W.camCtx[s] = c;
            ConnVertex v;
            v.thr = st.throughput;
            v.absNone = st.nVol ? st.volAbs[st.nVol - 1] : splat4(0.0f);
            v.absExited = absorptionAfter(st, kTransExited, hs.s, hs.material);
            v.pos = cv.pos;
            v.flags = st.flags | (cv.isExit ? kWbAtExit : 0u) | (cv.prevIsExit ? kWbPrevExit : 0u);
            v.normal = cv.normal;
            v.curPdfFwd = cv.curPdfFwd;
            v.prevPos = cv.prevPos;
            v.pdfRatioSum = cv.pdfRatioSum;
            v.prevNormal = cv.prevNormal;
            v.prevPdfFwd = cv.prevPdfFwd;
            v.wo = -hs.rayDirOS;
            v.hero = sp.hero;
            v.curIOR = currentIOR(st);
            v.prevIOR = previousIOR(st);
            v.instance = hit.instance;
            v.front = hit.front ? 1u : 0u;
            W.cvx[s] = v;
            for (uint32_t li = 0; li < count; ++li) W.connSlot[base + li] = make_uint2(s, li);
        }
        bool cont = false, toExit = false;
        if (alive)
        {
            // the scattered continuation (rv was drawn right after the trace)
            const Surface& sf = hs.s;
            const float3 wo = -hs.rayDirOS;
            bool isDiffuse, sDelta;
            float3 wiS;
            SubsurfaceExit ex;
            const uint32_t event = sampleEvent(S, Lt, sp, sf, c, wo, rv, cv.isExit, vertexPoint(cv.pos, cv.normal, -rayDir, hit), wiS,
                                               ex, isDiffuse, sDelta);
            if (event != kEventNone)
            {
                if (isDiffuse) st.flags |= kFlagRegularize;
                ScatterEval ev;
                if (event == kEventEntry) ev = evaluateEntry(Lt, sp, sf, c, wo, ex);
                else if (event == kEventExitLobe)
                    ev = evaluateExitBoth(sf, c, currentIOR(st), previousIOR(st), wo, wiS, hit.front, false, cv.pos, cv.normal,
                                          cv.prevPos, cv.prevNormal);
                else ev = evaluateBoth(Lt, sp, sf, c, currentIOR(st), previousIOR(st), wo, wiS, hit.front, false, sDelta);
                bool dispersed = applyTransmission(st, ev.transmission, sf, hs.material);
                float4 w = ev.weight * safeDiv(1.0f, ev.pdfFwd);
                if (dispersed) terminateSecondary(st.throughput);
                if (!russianRoulette(st.throughput, rs.r1()))
                {
                    if (ci > 0)
                    {
                        float bwdPrev = sDelta ? -1.0f
                                               : (event == kEventExitLobe ? ev.pdfBwd
                                                                          : ev.pdfBwd * solidAngleToArea(rayOrigin - cv.pos, cv.prevNormal));
                        deferredRI = accumulateRISum(deferredRI, bwdPrev, cv.prevPdfFwd, !cv.prevIsExit);
                        cv.pdfRatioSum = deferredRI;
                    }
                    cv.prevNormal = cv.normal;
                    cv.prevPos = cv.pos;
                    cv.prevPdfFwd = cv.curPdfFwd;
                    pdfFwdCam = sDelta ? -1.0f : ev.pdfFwd;
                    st.throughput = st.throughput * w;
                    if (event == kEventEntry)
                    {
                        // the next vertex is the exit point: queued without a ray to trace
                        toExit = true;
                        rayOrigin = ex.exit.pos;
                        rayDir = -ex.exit.normal;
                        W.exitHit[s] = mk4(ex.exit.b1, ex.exit.b2, __uint_as_float(ex.exit.instance),
                                           __uint_as_float(ex.exit.prim | (ex.exit.front ? 0x80000000u : 0u)));
                    }
                    else
                    {
                        rayDir = normalize(xformVectorT(I->w2o, wiS));
                        rayOrigin = spawnRayOrigin(cv.pos, cv.normal, rayDir);
                    }
                    cont = ci + 1 < P.maxDepth;
                }
            }
            W.tot[s] = total;
            if (cont)
            {
                W.thr[s] = st.throughput;
                W.cv0[s] = mk4(cv.prevPos.x, cv.prevPos.y, cv.prevPos.z, cv.pdfRatioSum);
                W.cv1[s] = mk4(cv.prevNormal.x, cv.prevNormal.y, cv.prevNormal.z, cv.prevPdfFwd);
                W.cv2[s] = mk4(deferredRI, pdfFwdCam, sp.hero, 0.0f);
                W.misc[s] = make_uint4(st.flags | (toExit ? kWbAtExit : 0u) | (cv.isExit ? kWbPrevExit : 0u) | (st.nVol << 16),
                                       rs.dim, rs.seed, f);
                wbStoreVolumes(W, s, st);
            }
        }
        const uint32_t o = warpAppend(Qout.count, cont);
        if (cont)
        {
            Qout.o[o] = mk4(rayOrigin.x, rayOrigin.y, rayOrigin.z, __uint_as_float(s));
            Qout.d[o] = mk4(rayDir.x, rayDir.y, rayDir.z, toExit ? 1.0f : 0.0f);
        }
    }
}

// the connections of this bounce's camera vertices, one thread per (camera vertex, light
// vertex) record (getLightNodeConnection + calculateLightPathRadiance, BDPTCommon.hlsl:622-635,
// 1062-1215): the contribution and the visibility ray of each, summed later in light-vertex
// order. The light side's MIS context comes prepared with the light vertex.
#ifndef YG_CONNECT_MIN_BLOCKS
#define YG_CONNECT_MIN_BLOCKS 16
#endif
__global__ void __launch_bounds__(128, YG_CONNECT_MIN_BLOCKS) wbConnect(const SceneView S, BdptParams B, BdptWave W, uint32_t ci)
{
    const Luts Lt = bdptLuts(S);
    const uint32_t n = *W.connCount;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    {
        const uint2 sl = W.connSlot[e];
        const uint32_t s = sl.x, li = sl.y;
        const uint32_t f = W.misc[s].w, path = W.misc2[s].y;
        const SharedNode& sn = W.prep[(((size_t)(f - W.fBase)) * B.lightPaths + path) * B.maxLightVerts + li];
        const LightNode& ln = sn.n;
        float4 ro = mk4(0.f, 0.f, 0.f, __uint_as_float(s)), rd = mk4(0.f, 0.f, 0.f, -1.0f), contrib = splat4(0.0f);
        uint2 target = make_uint2(0u, 0u);
        if (!(ln.flags & NF_DELTA))
        {
            const ConnVertex v = W.cvx[s];
            const Surface sf = W.camSurf[s];
            const SurfaceCtx c = W.camCtx[s];
            const GpuInstance& I = S.instances[v.instance];
            Spectral sp;
            spectralOf(S, v.hero, sp);
            CamVertex cv;
            cv.pos = v.pos;
            cv.normal = v.normal;
            cv.prevPos = v.prevPos;
            cv.prevNormal = v.prevNormal;
            cv.pdfRatioSum = v.pdfRatioSum;
            cv.prevPdfFwd = v.prevPdfFwd;
            cv.curPdfFwd = v.curPdfFwd;
            cv.isExit = (v.flags & kWbAtExit) != 0;
            cv.prevIsExit = (v.flags & kWbPrevExit) != 0;
            LightVertexCtx lv;
            lv.riSum = sn.lvRiSum;
            lv.prevPos = sn.lvPrevPos;
            lv.prevNormal = sn.lvPrevNormal;
            lv.prevPdfFwd = sn.lvPrevPdfFwd;
            lv.prevFlags = sn.lvPrevFlags;
            lv.originFlags = sn.lvOriginFlags;
            const bool front = v.front != 0;
            const bool camTerminated = (v.flags & kFlagSecondaryTerminated) != 0;
            const bool atInfinity = li == 0 && (ln.flags & NF_INFINITE);
            const bool noGeometry = li == 0 && (ln.flags & (NF_ENV | NF_PUNCTUAL));
            float3 toLightDir;
            float dist;
            if (atInfinity)
            {
                toLightDir = -ln.normal;
                dist = __int_as_float(0x7f800000);
            }
            else
            {
                float3 toLight = ln.pos - cv.pos;
                dist = length(toLight);
                toLightDir = toLight / dist;
            }
            const float3 wi = normalize(xformVector(I.w2o, toLightDir));
            const bool lightTerminated = (ln.flags & NF_TERMINATED) != 0;
            const bool terminatedBefore = camTerminated || lightTerminated;
            ScatterEval ce = cv.isExit ? evaluateExitBoth(sf, c, v.curIOR, v.prevIOR, v.wo, wi, front, false, cv.pos, cv.normal,
                                                          cv.prevPos, cv.prevNormal)
                                       : evaluateBoth(Lt, sp, sf, c, v.curIOR, v.prevIOR, v.wo, wi, front, false, false);
            if ((ce.transmission & kTransDispersed) && !terminatedBefore) terminateSecondary(ce.weight);
            if (ce.pdfFwd != 0.0f && !allEqual4(ce.weight, 0.0f))
            {
                const bool terminatedNow = terminatedBefore || (ce.transmission & kTransDispersed);
                ScatterEval le;
                float fwdLight;
                if (lightEndOfConnection(S, B, Lt, sp, sn, li, cv.pos, terminatedNow, le, fwdLight))
                {
                    float mis = misWeight(S, ci, cv, li, lv, ln, ce.pdfFwd, ce.pdfBwd, fwdLight, le.pdfBwd);
                    float G = li > 0 ? 1.0f / (dist * dist) : 1.0f;
                    float4 wc = ce.weight;
                    if (!atInfinity)
                    {
                        // absorptionAfter: the medium the connection runs through
                        float4 cab = (ce.transmission & kTransExited)    ? v.absExited
                                     : (ce.transmission & kTransEntered) ? sf.absorption
                                                                          : v.absNone;
                        if (!allEqual4(cab, 0.0f)) wc = wc * transmittance(cab, dist);
                    }
                    contrib = le.weight * wc * v.thr * ln.radiance * G * mis;
                    if (camTerminated && lightTerminated) contrib.x *= 0.25f; // undoSecondaryWavelengthRescale
                    const float3 start = spawnRayOrigin(cv.pos, cv.normal, toLightDir);
                    ro = mk4(start.x, start.y, start.z, __uint_as_float(s));
                    rd = mk4(toLightDir.x, toLightDir.y, toLightDir.z,
                             atInfinity ? __int_as_float(0x7f800000)
                                        : (noGeometry ? dist - kRayMinT : kRayMinT + dist + kVisibilityEps));
                    target = noGeometry ? make_uint2(0xffffffffu, 0xffffffffu) : make_uint2(ln.instance, ln.prim);
                }
            }
        }
        W.C.o[e] = ro;
        W.C.d[e] = rd;
        W.C.target[e] = target;
        W.C.contrib[e] = contrib;
    }
}

// visibility of the connection records (checkVisibility: the segment must reach the light
// vertex's own triangle first; toward the environment nothing may be hit)
__global__ void __launch_bounds__(128, YG_SHADOW_MIN_BLOCKS) wbVisibility(const SceneView S, BdptWave W,
                                                                         unsigned long long* travCtr)
{
    TraversalCount tc{0, 0};
    uint32_t rays = 0;
    uint2 tg = make_uint2(0u, 0u);
    bool early = false, none = false;
    traceGridStop<false>(
        *W.connCount,
        [&](TraceState& t, uint32_t e) {
            const float4 d = W.C.d[e];
            // a record without a connection (d.w < 0) has no ray: its traversal is empty
            none = d.w < 0.0f;
            if (none)
            {
                t.gHits = 0;
                t.sp = 0;
                return;
            }
            const float4 o = W.C.o[e];
            // the light vertex's own triangle must be the first hit; toward a target without
            // geometry (kPunctualShadow) nothing may be hit
            tg = W.C.target[e];
            early = shadowBegin(t, S, mk3(o.x, o.y, o.z), mk3(d.x, d.y, d.z), kRayMinT, d.w, tg.x, tg.y);
        },
        [&](const TraceState& t, uint32_t e) { W.vis[e] = !none && shadowVisible(t.found, t.h, tg.x, tg.y); },
        [&](const TraceState& t) { return shadowStopped(t, early, tg.x, tg.y); }, tc, rays);
    countRays(travCtr ? travCtr + 5 : nullptr, rays);
}

// adds each path's visible connections of this bounce, in light-vertex order
__global__ void __launch_bounds__(256) wbAccumulate(BdptWave W, RayQueue Qin)
{
    const uint32_t n = *Qin.count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t s = __float_as_uint(Qin.o[i].w);
        const uint2 cr = W.conn[s];
        if (cr.y == 0) continue;
        float4 total = W.tot[s];
        for (uint32_t j = 0; j < cr.y; ++j)
            if (W.vis[cr.x + j]) total = total + W.C.contrib[cr.x + j];
        W.tot[s] = total;
    }
}

__global__ void __launch_bounds__(256) wbFinalize(const SceneView S, const LaunchParams P, BdptWave W)
{
    const uint64_t cropPix = (uint64_t)P.cropW * P.cropH;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < W.n; s += gridDim.x * blockDim.x)
    {
        const uint4 m = W.misc[s], m2 = W.misc2[s];
        const uint64_t idx = (uint64_t)m.w * cropPix + m2.x;
        Spectral sp;
        spectralOf(S, W.cv2[s].z, sp);
        const float4 total = W.tot[s];
        float3 X = toXYZ(S, sp, total);
        P.sampleXYZ[idx] = mk4(X.x, X.y, X.z, 1.0f);
        if (P.dump)
        {
            float* d = P.dump + idx * 8;
            d[0] = sp.hero;
            d[1] = total.x;
            d[2] = total.y;
            d[3] = total.z;
            d[4] = total.w;
            d[5] = X.x;
            d[6] = X.y;
            d[7] = X.z;
        }
        if (P.featAlbedo)
        {
            P.featAlbedo[idx] = W.fhAlb[s];
            P.featNormalDepth[idx] = W.fhNrm[s];
        }
    }
}

// ------------------------------------------------------------------ light tracing to the lens (t = 1)
// calculatePureLightPaths (BDPTCalculatePureLightPaths.comp:107-206): one thread per header
__global__ void __launch_bounds__(128) bdptLightTrace(const SceneView S, const LaunchParams P, BdptParams B)
{
    const Luts Lt = bdptLuts(S);
    const uint32_t total = B.frames * B.lightPaths;
    const uint64_t cropPix = (uint64_t)P.cropW * P.cropH;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        const uint32_t f = t / B.lightPaths, h = t - f * B.lightPaths;
        const uint32_t hc = B.validCount[f];
        if (h >= hc) continue;
        const uint32_t l = B.valid[(size_t)f * B.lightPaths + h];
        const uint32_t vCount = B.counts[(size_t)f * B.lightPaths + l];
        if (vCount <= 1) continue;
        Spectral sp;
        spectralOf(S, B.heroes[(size_t)f * B.lightPaths + l], sp);
        const LightNode* nodes = B.nodes + ((size_t)f * B.lightPaths + l) * B.maxLightVerts;
        RandomSampler lr{S.sobol + (size_t)f * kSobolDims, B.lensDimOffset + 2u, h ^ (P.seed * 0x9E3779B9u)};
        float2 disk = sampleConcentricDisk(lr.r2());
        float3 lensVS = mk3(disk.x * S.cam.apertureRadius, disk.y * S.cam.apertureRadius, 0.0f);
        float4 lw = mul44(S.cam.viewToWorld, mk4(lensVS.x, lensVS.y, lensVS.z, 1.0f));
        float3 lensWS = mk3(lw.x, lw.y, lw.z);
        LightNode n0 = nodes[0];
        float3 prevPos = n0.pos, prevNormal = n0.normal;
        float prevPdfFwd = n0.pdfFwd;
        const uint32_t originFlags = n0.flags;
        uint32_t prevFlags = n0.flags;
        float riSum = 0.0f;
        float deferred = accumulateRISum(0.0f, n0.pdfBwd, n0.pdfFwd);
        for (uint32_t i = 1; i < vCount; ++i)
        {
            LightNode n = nodes[i];
            // projectThroughLensToUV (raytraceCommonResources.hlsl:140-160)
            float4 pv = mul44(S.cam.worldToView, mk4(n.pos.x, n.pos.y, n.pos.z, 1.0f));
            float3 lensToPos = mk3(pv.x, pv.y, pv.z) - lensVS;
            float fwd = lensToPos.z * S.cam.forwardZSign;
            bool onScreen = false;
            uint32_t tx = 0, ty = 0;
            if (fwd > 0.0f)
            {
                float3 fp = lensVS + lensToPos * (S.cam.focusDistance / fwd);
                float4 us = mul44(S.cam.viewToUV, mk4(fp.x, fp.y, fp.z, 1.0f));
                float u = us.x / us.w, v = us.y / us.w;
                onScreen = u >= 0.0f && v >= 0.0f && u <= 1.0f && v <= 1.0f;
                tx = (uint32_t)floorf(fminf(saturate(u) * (float)P.width, (float)P.width - 1.0f));
                ty = (uint32_t)floorf(fminf(saturate(v) * (float)P.height, (float)P.height - 1.0f));
            }
            bool inCrop = tx >= P.cropX && tx < P.cropX + P.cropW && ty >= P.cropY && ty < P.cropY + P.cropH;
            if (onScreen && inCrop && !(n.flags & NF_DELTA))
            {
                SharedNode sn;
                prepareSharedNode(S, P, sp, n, prevPos, prevNormal, i, sn);
                ScatterEval ev;
                float unused;
                if (lightEndOfConnection(S, B, Lt, sp, sn, i, lensWS, false, ev, unused) && !isZero4(ev.weight))
                {
                    float3 toLens = lensWS - n.pos;
                    float len = length(toLens);
                    bool visible = true;
                    if (len >= 0.0001f)
                    {
                        Hit vh;
                        visible = !traceClosest<false>(S, n.pos, toLens / len, 0.01f, len, vh, nullptr);
                    }
                    if (visible)
                    {
                        bool prevEnv = i == 1 && (originFlags & NF_ENV);
                        const bool nodeExit = (n.flags & NF_SSS_EXIT) != 0;
                        // from a subsurface exit the backward density is an area density already
                        float bwdPrev = ev.pdfBwd * ((prevEnv || nodeExit) ? 1.0f : solidAngleToArea(prevPos - n.pos, prevNormal));
                        if (i == 1 && (originFlags & NF_PUNCTUAL)) bwdPrev = 0.0f; // a camera path never hits a delta light
                        float3 camToNode = n.pos - lensWS;
                        float pdfCam = cameraDirectionalPdf(S, P, camToNode);
                        float ri = accumulateRISum(riSum, bwdPrev, prevPdfFwd, !(prevFlags & NF_SSS_EXIT));
                        ri = accumulateRISum(ri, pdfCam * solidAngleToArea(camToNode, n.normal), n.pdfFwd, !nodeExit);
                        float mis = 1.0f / (1.0f + ri);
                        float G = 1.0f / fmaxf(0.0001f, dot(camToNode, camToNode));
                        float importance = safeDiv(pdfCam, (float)hc);
                        float4 contrib = n.radiance * ev.weight * mis * G * importance;
                        float3 X = toXYZ(S, sp, contrib);
                        unsigned long long* dst =
                            B.splat + 3 * ((uint64_t)f * cropPix + (uint64_t)(ty - P.cropY) * P.cropW + (tx - P.cropX));
                        const float xs[3] = {X.x, X.y, X.z};
                        for (int k = 0; k < 3; ++k)
                        {
                            // splat XYZ is non-negative; the fixed-point sum holds 2^39 per pixel
                            double q = (double)xs[k] * kSplatScale;
                            if (q > 0.0 && q < 9.0e18) atomicAdd(dst + k, (unsigned long long)llrint(q));
                        }
                    }
                }
            }
            riSum = deferred;
            deferred = accumulateRISum(deferred, n.pdfBwd, n.pdfFwd, !(n.flags & NF_SSS_EXIT));
            prevFlags = n.flags;
            prevPos = n.pos;
            prevNormal = n.normal;
            prevPdfFwd = n.pdfFwd;
        }
    }
}

// accumulatePureLightPaths (BDPTAccumulatePureLightPaths.comp:7-31): adds the splats of each
// sample index to its sample image
__global__ void bdptResolveSplats(const LaunchParams P, BdptParams B)
{
    const uint64_t n = (uint64_t)B.frames * P.cropW * P.cropH;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const unsigned long long* s = B.splat + 3 * i;
        unsigned long long a = s[0], b = s[1], c = s[2];
        if ((a | b | c) == 0ull) continue;
        float4 v = P.sampleXYZ[i];
        v.x += (float)((double)a / kSplatScale);
        v.y += (float)((double)b / kSplatScale);
        v.z += (float)((double)c / kSplatScale);
        P.sampleXYZ[i] = v;
        if (P.dump)
        {
            P.dump[i * 8 + 5] = v.x;
            P.dump[i * 8 + 6] = v.y;
            P.dump[i * 8 + 7] = v.z;
        }
    }
}

// ------------------------------------------------------------------ host side
namespace
{
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
} // namespace

constexpr uint32_t kBdptWave = 1u << 20; // camera paths per wave

namespace
{
struct WaveShape
{
    uint32_t capacity;   // camera paths per wave
    uint32_t spanFrames; // frames one wave can touch
};
WaveShape waveShape(uint32_t frames, uint64_t cropPixels)
{
    const uint64_t total = (uint64_t)frames * cropPixels;
    WaveShape w;
    w.capacity = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(total, kBdptWave));
    w.spanFrames = (uint32_t)std::min<uint64_t>(frames, w.capacity / std::max<uint64_t>(cropPixels, 1) + 2);
    return w;
}
// per path: state (5 x 16 + 2 x 16 + 8 + volumes 96 + features 32), two ray queues (64), hits
// (20), the regrouped ray and hit queues (52) and the class key (1)
size_t waveSlotBytes()
{
    return 5 * 16 + 2 * 16 + 8 + 16 + 16 + 16 + 64 + 2 * 16 + 2 * 32 + 20 + 52 + 1 + sizeof(Surface) + sizeof(SurfaceCtx) +
           sizeof(ConnVertex);
}
} // namespace

size_t bdptArenaBytes(uint32_t frames, uint32_t lightPaths, uint32_t maxLightVerts, uint64_t cropPixels)
{
    size_t b = align256((size_t)frames * lightPaths * maxLightVerts * sizeof(LightNode));
    b += 3 * align256((size_t)frames * lightPaths * 4);
    b += align256((size_t)frames * 4);
    b += align256((size_t)frames * cropPixels * 24);
    const WaveShape w = waveShape(frames, cropPixels);
    b += align256((size_t)w.spanFrames * lightPaths * maxLightVerts * sizeof(SharedNode));
    b += (size_t)w.capacity * waveSlotBytes() + 40 * 256;
    b += (size_t)w.capacity * maxLightVerts * (56 + 1 + 8) + 8 * 256;
    b += 256;
    return b;
}

uint32_t bdptConnectionRecordBytes()
{
    return (uint32_t)(sizeof(uint2) + sizeof(Surface) + sizeof(SurfaceCtx) + sizeof(ConnVertex) + sizeof(SharedNode) +
                      16 + 16 + 8 + 16);
}

int launchBdpt(const SceneView& S, const LaunchParams& P, void* arena, const uint32_t* perm, uint32_t lightPaths,
               uint32_t maxLightVerts, float3 worldCenter, float worldRadiusSqr, int smCount, cudaStream_t stream,
               KernelTimer* T)
{
    BdptParams B;
    const uint64_t cropPix = (uint64_t)P.cropW * P.cropH;
    B.frames = P.sppCount;
    B.lightPaths = lightPaths;
    B.maxLightVerts = maxLightVerts;
    B.groups = (uint32_t)((cropPix + kGroupSize - 1) / kGroupSize);
    B.camDimOffset = maxLightVerts * 5 + 12;
    B.lensDimOffset = maxLightVerts * 5 + 9;
    B.perm = perm;
    B.worldCenter = worldCenter;
    B.worldRadiusSqr = worldRadiusSqr;
    char* p = static_cast<char*>(arena);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += align256(bytes);
        return r;
    };
    B.nodes = reinterpret_cast<LightNode*>(take((size_t)B.frames * lightPaths * maxLightVerts * sizeof(LightNode)));
    B.counts = reinterpret_cast<uint32_t*>(take((size_t)B.frames * lightPaths * 4));
    B.heroes = reinterpret_cast<float*>(take((size_t)B.frames * lightPaths * 4));
    B.valid = reinterpret_cast<uint32_t*>(take((size_t)B.frames * lightPaths * 4));
    B.validCount = reinterpret_cast<uint32_t*>(take((size_t)B.frames * 4));
    B.splat = reinterpret_cast<unsigned long long*>(take((size_t)B.frames * cropPix * 24));
    // the camera wave
    const WaveShape ws = waveShape(B.frames, cropPix);
    const size_t C = ws.capacity;
    BdptWave W;
    W.capacity = ws.capacity;
    W.prep = reinterpret_cast<SharedNode*>(take((size_t)ws.spanFrames * lightPaths * maxLightVerts * sizeof(SharedNode)));
    W.thr = reinterpret_cast<float4*>(take(C * 16));
    W.tot = reinterpret_cast<float4*>(take(C * 16));
    W.cv0 = reinterpret_cast<float4*>(take(C * 16));
    W.cv1 = reinterpret_cast<float4*>(take(C * 16));
    W.cv2 = reinterpret_cast<float4*>(take(C * 16));
    W.misc = reinterpret_cast<uint4*>(take(C * 16));
    W.misc2 = reinterpret_cast<uint4*>(take(C * 16));
    W.conn = reinterpret_cast<uint2*>(take(C * 8));
    W.exitHit = reinterpret_cast<float4*>(take(C * 16));
    W.camSurf = reinterpret_cast<Surface*>(take(C * sizeof(Surface)));
    W.camCtx = reinterpret_cast<SurfaceCtx*>(take(C * sizeof(SurfaceCtx)));
    W.cvx = reinterpret_cast<ConnVertex*>(take(C * sizeof(ConnVertex)));
    W.volIOR = reinterpret_cast<float4*>(take(C * 16));
    W.volMat = reinterpret_cast<uint4*>(take(C * 16));
    W.volAbs = reinterpret_cast<float4*>(take(C * 64));
    W.fhAlb = reinterpret_cast<float4*>(take(C * 16));
    W.fhNrm = reinterpret_cast<float4*>(take(C * 16));
    uint32_t* counters = reinterpret_cast<uint32_t*>(take(256));
    RayQueue QA{reinterpret_cast<float4*>(take(C * 16)), reinterpret_cast<float4*>(take(C * 16)), counters + 0};
    RayQueue QB{reinterpret_cast<float4*>(take(C * 16)), reinterpret_cast<float4*>(take(C * 16)), counters + 1};
    HitQueue H{reinterpret_cast<float4*>(take(C * 16)), reinterpret_cast<uint32_t*>(take(C * 4))};
    RayQueue QS{reinterpret_cast<float4*>(take(C * 16)), reinterpret_cast<float4*>(take(C * 16)), counters + 3};
    HitQueue HS{reinterpret_cast<float4*>(take(C * 16)), reinterpret_cast<uint32_t*>(take(C * 4))};
    uint8_t* keys = reinterpret_cast<uint8_t*>(take(C));
    uint32_t* classCounts = counters + 8; // [kShadeClasses] counts, then [kShadeClasses] cursors
    const size_t CR = C * maxLightVerts;
    W.C = ShadowQueue{reinterpret_cast<float4*>(take(CR * 16)), reinterpret_cast<float4*>(take(CR * 16)),
                      reinterpret_cast<uint2*>(take(CR * 8)), reinterpret_cast<float4*>(take(CR * 16)), counters + 2};
    W.vis = reinterpret_cast<uint8_t*>(take(CR));
    W.connSlot = reinterpret_cast<uint2*>(take(CR * 8));
    W.connCount = counters + 2;

    cudaMemsetAsync(B.splat, 0, (size_t)B.frames * cropPix * 24, stream);
    const uint32_t lp = B.frames * lightPaths;
    int lb = (int)std::min<uint64_t>((lp + 127) / 128, (uint64_t)smCount * 16);
    int launches = 0;
    bdptLightPaths<<<lb, 128, 0, stream>>>(S, P, B);
    bdptHeaders<<<B.frames, 1024, 0, stream>>>(B);
    launches += 2;
    const uint64_t total = (uint64_t)B.frames * cropPix;
    const int traceBlocks = smCount * 16, shadeBlocks = smCount * 8;
    for (uint64_t c0 = 0; c0 < total; c0 += C)
    {
        W.c0 = c0;
        W.n = (uint32_t)std::min<uint64_t>(C, total - c0);
        W.fBase = (uint32_t)(c0 / cropPix);
        const uint32_t waveFrames = (uint32_t)((c0 + W.n - 1) / cropPix) - W.fBase + 1;
        const uint64_t prepItems = (uint64_t)waveFrames * lightPaths * maxLightVerts;
        int pb = (int)std::min<uint64_t>((prepItems + 127) / 128, (uint64_t)smCount * 16);
        wbPrepare<<<pb, 128, 0, stream>>>(S, P, B, W, waveFrames);
        int gb = (int)std::min<uint64_t>((W.n + 127) / 128, (uint64_t)smCount * 16);
        wbGenerate<<<gb, 128, 0, stream>>>(S, P, B, W, QA);
        launches += 2;
        RayQueue* cur = &QA;
        RayQueue* nxt = &QB;
        for (uint32_t ci = 0; ci < P.maxDepth; ++ci)
        {
            if (T) T->begin(stream);
            wbTrace<<<traceBlocks, 128, 0, stream>>>(S, *cur, H, W.exitHit);
            if (T) T->end(kKernelTrace, stream);
            cudaMemsetAsync(nxt->count, 0, 4, stream);
            cudaMemsetAsync(W.connCount, 0, 4, stream);
            // shading coherence: hits grouped by material class before the vertex pass
            cudaMemsetAsync(classCounts, 0, 2 * kShadeClasses * 4, stream);
            if (T) T->begin(stream);
            wfClassify<kShadeClasses><<<smCount * 4, 256, 0, stream>>>(S, *cur, H, keys, classCounts);
            wfRegroup<kShadeClasses><<<smCount * 4, 256, 0, stream>>>(*cur, H, keys, classCounts, classCounts + kShadeClasses, QS, HS);
            if (T) T->end(kKernelRegroup, stream);
            if (T) T->begin(stream);
            wbShade<<<shadeBlocks, 128, 0, stream>>>(S, P, B, W, QS, HS, *nxt, ci);
            if (T) T->end(kKernelShade, stream);
            if (T) T->begin(stream);
            wbConnect<<<traceBlocks, 128, 0, stream>>>(S, B, W, ci);
            if (T) T->end(kKernelConnect, stream);
            if (T) T->begin(stream);
            wbVisibility<<<traceBlocks, 128, 0, stream>>>(S, W, P.traversalCounter);
            wbAccumulate<<<smCount * 4, 256, 0, stream>>>(W, QS);
            if (T) T->end(kKernelShadow, stream);
            launches += 7;
            RayQueue* t = cur;
            cur = nxt;
            nxt = t;
        }
        int fb = (int)std::min<uint64_t>((W.n + 255) / 256, (uint64_t)smCount * 8);
        wbFinalize<<<fb, 256, 0, stream>>>(S, P, W);
        ++launches;
    }
    bdptLightTrace<<<lb, 128, 0, stream>>>(S, P, B);
    int rb = (int)std::min<uint64_t>((B.frames * cropPix + 255) / 256, (uint64_t)smCount * 8);
    bdptResolveSplats<<<rb, 256, 0, stream>>>(P, B);
    launches += 2;
    return launches;
}

} // namespace yg
