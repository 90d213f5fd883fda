// The reference's edge-stopping a-trous denoiser, rebuilt as the baseline that the learned
// denoiser is measured against. Three stages, all on the device:
//  * gather (with each render that asks for it): per pixel, the features of the first camera
//    vertex of every sample are summed as four moment layers (first and second moments of
//    albedo, normal, material vector, IOR and view depth), and the XYZ of the odd-indexed
//    samples is summed apart, so that the film splits into two interleaved half films whose
//    difference estimates the per-pixel variance (mergeNewSamples.comp: two accumulation
//    targets, variance of log(1 + Y));
//  * resolve + prefilter: moments -> feature means and variances, smoothed over 5x5 with the
//    variance-normalised edge-stopping weights (prefilterFeatures.comp:72-149) and packed to
//    half precision as the reference's two RGBA32_UINT feature textures
//    (denoiseFeatures.hlsl:108-127); the same kernel forms the input colour and variance;
//  * five a-trous passes with the 5x5 B3 kernel at steps 1, 2, 4, 8, 16, weighted by plane
//    distance, normal, albedo, material and luminance (denoise.comp:153-275).
// Data layout (W x H film, row major): moments 4 planes of float4 sums, odd sums one float4
// plane (XYZ, count), packed features 2 planes of uint4 (32 B a pixel), colour and variance
// ping-pong planes. Every stage is one thread per pixel in 32x8 blocks, so the 5x5 footprint
// of a warp stays within a few cache lines of each row.
#include "yg_kernels.h"
#include "yg_path.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace yg
{

namespace
{

constexpr float kFeatureIorScale = 0.5f;   // FEATURE_IOR_SCALE
constexpr float kFeatureHalfMax = 65000.f; // FEATURE_HALF_MAX
constexpr float kEpsMin = 1e-6f;

struct Features
{
    float3 albedo, normal;
    float depth, roughness, metalness, transparency, anisotropy, ior;
    float varAlbedo, varDepth, varMaterial;
};

// 4x4 row-major times (x, y, z, w), summed left to right
__device__ __forceinline__ float4 xform(const float* m, float x, float y, float z, float w)
{
    return mk4(m[0] * x + m[1] * y + m[2] * z + m[3] * w, m[4] * x + m[5] * y + m[6] * z + m[7] * w,
               m[8] * x + m[9] * y + m[10] * z + m[11] * w, m[12] * x + m[13] * y + m[14] * z + m[15] * w);
}

__device__ __forceinline__ bool finite3(float3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

// ---------------------------------------------------------------- gather
// writeMaterialParamsForFirstBounce (hitShadersCommon.hlsl:94-128) for one camera sample and
// featureSampleToMoments (denoiseFeatures.hlsl:27-43); a non-finite feature counts as a miss
// (mergeNewSamples.comp:96-103). Returns false for a miss.
__device__ bool firstVertexMoments(const SceneView& S, const LaunchParams& P, const Spectral& sp, const Hit& hit,
                                   PathState& ps, float4 m[4])
{
    const GpuInstance& I = S.instances[hit.instance];
    HitSurface hs;
    setupSurface(S, P, sp, hit, I, ps.dir, ps, hs);
    const Surface& s = hs.s;
    const GpuMaterial& M = S.materials[hs.material];
    float coatW = s.clearCoatAmount, sheenW = s.sheenAmount, baseW = s.specularAmount;
    float wsum = coatW + sheenW + baseW;
    if (wsum == 0.0f) wsum = 1.0f;
    coatW = coatW / wsum;
    sheenW = sheenW / wsum;
    baseW = baseW / wsum;
    float3 n = xformVectorT(I.w2o, s.baseLayerNormal);
    if (s.clearCoatAmount > 0.0f) n = n + xformVectorT(I.w2o, s.coatingLayerNormal);
    n = normalize(n);
    const float4 e = M.emissive_roughness, sh = M.sheenColor_roughness;
    float3 a = mk3(e.x / (1.0f + e.x) + hs.albedoRGB.x + sh.x * s.sheenAmount,
                   e.y / (1.0f + e.y) + hs.albedoRGB.y + sh.y * s.sheenAmount,
                   e.z / (1.0f + e.z) + hs.albedoRGB.z + sh.z * s.sheenAmount);
    float rough = s.roughness * baseW + s.clearCoatRoughness * coatW + s.sheenRoughness * sheenW;
    float ior = s.dielectricIOR * s.specularAmount + s.clearCoatIOR * s.clearCoatAmount;
    float3 hp = ps.origin + ps.dir * hit.t;
    float4 vp = mul44(S.cam.worldToView, mk4(hp.x, hp.y, hp.z, 1.0f));
    float depth = vp.z * S.cam.forwardZSign;
    if (!finite3(a) || !finite3(n) || !isfinite(depth) || !isfinite(rough) || !isfinite(s.metalness) ||
        !isfinite(s.transparency) || !isfinite(s.anisotropy) || !isfinite(ior))
        return false;
    float iorS = ior * kFeatureIorScale;
    float matSq = rough * rough + s.metalness * s.metalness + s.transparency * s.transparency + s.anisotropy * s.anisotropy;
    m[0] = mk4(a.x, a.y, a.z, dot(a, a));
    m[1] = mk4(n.x, n.y, n.z, 1.0f);
    m[2] = mk4(rough, s.metalness, s.transparency, s.anisotropy);
    m[3] = mk4(iorS, matSq + iorS * iorS, depth, depth * depth);
    return true;
}

// One thread per pixel of the crop; samples in index order, so the sums do not depend on
// scheduling. The camera ray of each sample is the uni/NEE integrators' own (same Sobol
// point, pixel seed and dimensions).
__global__ void __launch_bounds__(128) atrousGather(const SceneView S, const LaunchParams P, float4* __restrict__ mom,
                                                     float4* __restrict__ odd, const float4* __restrict__ samples,
                                                     uint32_t nspp)
{
    const uint32_t npix = P.cropW * P.cropH;
    const size_t plane = (size_t)P.width * P.height;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x)
    {
        const uint32_t cx = P.cropX + p % P.cropW, cy = P.cropY + p / P.cropW;
        const size_t fi = (size_t)cy * P.width + cx;
        float4 acc[4] = {mom[fi], mom[plane + fi], mom[2 * plane + fi], mom[3 * plane + fi]};
        float4 od = odd[fi];
        const uint32_t seed = (cy * P.width + cx) ^ (P.seed * 0x9E3779B9u);
        for (uint32_t k = 0; k < nspp; ++k)
        {
            if ((P.sppStart + k) & 1u)
            {
                float4 v = samples[(size_t)k * npix + p];
                od = od + mk4(v.x, v.y, v.z, 1.0f);
            }
            RandomSampler rs{S.sobol + (size_t)k * kSobolDims, 2u, seed};
            Spectral sp;
            PathState ps;
            beginPath(S, P, cx, cy, rs, sp, ps);
            Hit hit;
            if (!traceClosest<false>(S, ps.origin, ps.dir, kRayMinT, __int_as_float(0x7f800000), hit, nullptr)) continue;
            float4 m[4];
            if (!firstVertexMoments(S, P, sp, hit, ps, m)) continue;
            for (int l = 0; l < 4; ++l) acc[l] = acc[l] + m[l];
        }
        for (int l = 0; l < 4; ++l) mom[l * plane + fi] = acc[l];
        odd[fi] = od;
    }
}

// ---------------------------------------------------------------- weights
// calculateVarianceNormalizedWeight (denoiseFeatures.hlsl:145-150)
__device__ __forceinline__ float vnWeight(float distSqr, float sigma, float varSum, float k)
{
    return ygm_expf(-distSqr / (sigma * sigma + k * varSum + 1e-8f));
}

__device__ __forceinline__ float normalVariance(const Features& f) { return saturate(1.0f - length(f.normal)); }

// calculateFeatureWeight (denoiseFeatures.hlsl:152-166)
__device__ float featureWeight(const Features& a, const Features& b, const AtrousSettings& A, float k)
{
    float3 dn = a.normal - b.normal;
    float wN = vnWeight(dot(dn, dn), A.normalSigma, normalVariance(a) + normalVariance(b), k);
    float3 da = a.albedo - b.albedo;
    float wA = vnWeight(dot(da, da), A.materialSigma, a.varAlbedo + b.varAlbedo, k);
    float d0 = a.roughness - b.roughness, d1 = a.metalness - b.metalness, d2 = a.transparency - b.transparency,
          d3 = a.anisotropy - b.anisotropy, di = a.ior - b.ior;
    float matSq = d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
    float wM = vnWeight(matSq + di * di, A.materialSigma, a.varMaterial + b.varMaterial, k);
    return wN * wA * wM;
}

// ---------------------------------------------------------------- resolve + prefilter
// featuresFromMoments (denoiseFeatures.hlsl:61-88) of the running means sum / n
__device__ Features loadMoments(const float4* __restrict__ mom, const float4* __restrict__ film, size_t plane, size_t fi)
{
    float n = film[fi].w;
    float inv = n > 0.0f ? 1.0f / n : 0.0f;
    float4 m0 = mom[fi] * inv, m1 = mom[plane + fi] * inv, m2 = mom[2 * plane + fi] * inv, m3 = mom[3 * plane + fi] * inv;
    Features f;
    f.albedo = mk3(m0.x, m0.y, m0.z);
    f.varAlbedo = fmaxf(m0.w - dot(f.albedo, f.albedo), 0.0f);
    f.normal = mk3(m1.x, m1.y, m1.z);
    float coverage = m1.w;
    f.roughness = m2.x;
    f.metalness = m2.y;
    f.transparency = m2.z;
    f.anisotropy = m2.w;
    f.ior = m3.x;
    float matSq = m2.x * m2.x + m2.y * m2.y + m2.z * m2.z + m2.w * m2.w;
    f.varMaterial = fmaxf(m3.y - matSq - f.ior * f.ior, 0.0f);
    if (coverage > 0.0f)
    {
        f.depth = m3.z / coverage;
        f.varDepth = fmaxf(m3.w / coverage - f.depth * f.depth, 0.0f);
    }
    else
    {
        f.depth = 0.0f;
        f.varDepth = 0.0f;
    }
    return f;
}

// calculateRelativeDepthWeight (prefilterFeatures.comp:50-58)
__device__ float relativeDepthWeight(const Features& c, const Features& s, const AtrousSettings& A, float k)
{
    if (c.depth <= 0.0f || s.depth <= 0.0f) return 1.0f;
    float d = c.depth - s.depth;
    return vnWeight(d * d, c.depth * A.depthSigmaScale, c.varDepth + s.varDepth, k);
}

__device__ __forceinline__ uint32_t packHalf2(float a, float b)
{
    return (uint32_t)__half_as_ushort(__float2half_rn(a)) | ((uint32_t)__half_as_ushort(__float2half_rn(b)) << 16);
}
__device__ __forceinline__ float halfLo(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v & 0xFFFFu))); }
__device__ __forceinline__ float halfHi(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v >> 16))); }

// writeDenoiseFeatures (denoiseFeatures.hlsl:108-127)
__device__ void packFeatures(const Features& f, uint4& v0, uint4& v1)
{
    float relVarDepth = f.depth > 0.0f ? fminf(f.varDepth / (f.depth * f.depth), kFeatureHalfMax) : 0.0f;
    v0 = make_uint4(packHalf2(f.albedo.x, f.albedo.y), packHalf2(f.albedo.z, relVarDepth), packHalf2(f.normal.x, f.normal.y),
                    packHalf2(f.normal.z, f.roughness));
    v1 = make_uint4(__float_as_uint(f.depth), packHalf2(f.metalness, f.anisotropy), packHalf2(f.transparency, f.ior),
                    packHalf2(fminf(f.varAlbedo, kFeatureHalfMax), fminf(f.varMaterial, kFeatureHalfMax)));
}

// readDenoiseFeatures (denoiseFeatures.hlsl:129-141)
__device__ Features unpackFeatures(uint4 v0, uint4 v1)
{
    Features f;
    f.albedo = mk3(halfLo(v0.x), halfHi(v0.x), halfLo(v0.y));
    float relVarDepth = halfHi(v0.y);
    f.normal = mk3(halfLo(v0.z), halfHi(v0.z), halfLo(v0.w));
    f.roughness = halfHi(v0.w);
    f.depth = __uint_as_float(v1.x);
    f.metalness = halfLo(v1.y);
    f.anisotropy = halfHi(v1.y);
    f.transparency = halfLo(v1.z);
    f.ior = halfHi(v1.z);
    f.varAlbedo = halfLo(v1.w);
    f.varMaterial = halfHi(v1.w);
    f.varDepth = relVarDepth * f.depth * f.depth;
    return f;
}

__global__ void __launch_bounds__(256) atrousPrefilter(AtrousBuffers B, const AtrousSettings A)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = (int)B.width, H = (int)B.height;
    if (x >= W || y >= H) return;
    const size_t plane = (size_t)W * H, fi = (size_t)y * W + x;
    const Features c = loadMoments(B.moments, B.film, plane, fi);
    Features r = c;
    if (A.prefilter)
    {
        const float g3[3] = {3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
        const float g33[3] = {1.0f / 4.0f, 1.0f / 8.0f, 1.0f / 16.0f};
        float3 sumAlbedo = mk3(0.f, 0.f, 0.f), sumNormal = mk3(0.f, 0.f, 0.f);
        float4 sumMat = splat4(0.0f);
        float sumIor = 0.f, sumW = 0.f, sumDepth = 0.f, sumDepthW = 0.f;
        float sumVarAlbedo = 0.f, sumVarDepth = 0.f, sumVarMaterial = 0.f, sumVarW = 0.f;
        for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx)
            {
                const int sx = x + dx, sy = y + dy;
                if (sx < 0 || sx > W - 1 || sy < 0 || sy > H - 1) continue;
                const Features s = loadMoments(B.moments, B.film, plane, (size_t)sy * W + sx);
                float kw = g3[abs(dx)] * g3[abs(dy)];
                float w = kw * featureWeight(c, s, A, A.featureVarianceScale) * relativeDepthWeight(c, s, A, A.featureVarianceScale);
                sumAlbedo = sumAlbedo + s.albedo * w;
                sumNormal = sumNormal + s.normal * w;
                sumMat = sumMat + mk4(s.roughness, s.metalness, s.transparency, s.anisotropy) * w;
                sumIor = sumIor + s.ior * w;
                sumW = sumW + w;
                if (s.depth > 0.0f)
                {
                    sumDepth = sumDepth + s.depth * w;
                    sumDepthW = sumDepthW + w;
                }
                if (abs(dx) <= 1 && abs(dy) <= 1)
                {
                    float wv = g33[abs(dx) + abs(dy)] * featureWeight(c, s, A, 0.0f) * relativeDepthWeight(c, s, A, 0.0f);
                    sumVarAlbedo = sumVarAlbedo + s.varAlbedo * wv;
                    sumVarMaterial = sumVarMaterial + s.varMaterial * wv;
                    sumVarDepth = sumVarDepth + (s.depth > 0.0f ? s.varDepth : c.varDepth) * wv;
                    sumVarW = sumVarW + wv;
                }
            }
        float inv = 1.0f / fmaxf(sumW, kEpsMin);
        r.albedo = sumAlbedo * inv;
        r.normal = sumNormal * inv;
        float4 mat = sumMat * inv;
        r.roughness = mat.x;
        r.metalness = mat.y;
        r.transparency = mat.z;
        r.anisotropy = mat.w;
        r.ior = sumIor * inv;
        if (c.depth > 0.0f && sumDepthW > 0.0f) r.depth = sumDepth / sumDepthW;
        float invV = 1.0f / fmaxf(sumVarW, kEpsMin);
        r.varAlbedo = sumVarAlbedo * invV;
        r.varMaterial = sumVarMaterial * invV;
        r.varDepth = sumVarDepth * invV;
    }
    uint4 v0, v1;
    packFeatures(r, v0, v1);
    B.feat0[fi] = v0;
    B.feat1[fi] = v1;
    // the merged colour and its variance (mergeNewSamples.comp:254-285): the mean of the even
    // and odd half films, and the squared difference of their log(1 + Y) over two
    const float4 f = B.film[fi], o = B.odd[fi];
    const float n = f.w, no = o.w, ne = n - no;
    float4 col = splat4(0.0f);
    float var = 0.0f;
    if (ne > 0.0f && no > 0.0f)
    {
        float ie = 1.0f / ne, io = 1.0f / no;
        float3 ev = mk3((f.x - o.x) * ie, (f.y - o.y) * ie, (f.z - o.z) * ie);
        float3 ov = mk3(o.x * io, o.y * io, o.z * io);
        col = mk4((ev.x + ov.x) * 0.5f, (ev.y + ov.y) * 0.5f, (ev.z + ov.z) * 0.5f, 1.0f);
        float d = fabsf(ygm_logf(1.0f + ev.y) - ygm_logf(1.0f + ov.y));
        var = d * d / 2.0f;
    }
    else if (n > 0.0f)
    {
        float in = 1.0f / n;
        col = mk4(f.x * in, f.y * in, f.z * in, 1.0f);
    }
    B.colour[0][fi] = col;
    B.variance[0][fi] = var;
}

// ---------------------------------------------------------------- a-trous pass
// reconstructWorldPosition (denoise.comp:108-118): planar view depth along the pixel's pinhole ray
__device__ float3 worldPosition(const AtrousBuffers& B, int x, int y, float depth)
{
    float u = ((float)x + 0.5f) * B.invW, v = ((float)y + 0.5f) * B.invH;
    float4 p = xform(B.uvToView, u, v, 0.0f, 1.0f);
    p = mk4(p.x / p.w, p.y / p.w, p.z / p.w, p.w / p.w);
    float s = depth / fmaxf(fabsf(p.z), 1e-8f);
    float4 w = xform(B.viewToWorld, p.x * s, p.y * s, p.z * s, 1.0f);
    return mk3(w.x, w.y, w.z);
}

// calculatePlaneDistanceWeight (denoise.comp:120-139)
__device__ float planeDistanceWeight(float3 cp, const Features& c, float3 sp, const Features& s, const AtrousSettings& A)
{
    if (s.depth <= 0.0f) return 1.0f;
    float dist;
    float nl = length(c.normal);
    if (nl > 1e-3f)
    {
        float3 n = mk3(c.normal.x / nl, c.normal.y / nl, c.normal.z / nl);
        dist = dot(n, sp - cp);
    }
    else
        dist = c.depth - s.depth;
    return vnWeight(dist * dist, c.depth * A.depthSigmaScale, c.varDepth + s.varDepth, A.featureVarianceScale);
}

// denoiseAtrous (denoise.comp:157-275) at step 2^pass, reading colour/variance plane `src`
__global__ void __launch_bounds__(256) atrousPass(AtrousBuffers B, const AtrousSettings A, uint32_t pass, uint32_t src,
                                                  float4* __restrict__ outColour, float* __restrict__ outVar)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = (int)B.width, H = (int)B.height;
    if (x >= W || y >= H) return;
    const size_t fi = (size_t)y * W + x;
    const float4* __restrict__ colour = B.colour[src];
    const float* __restrict__ variance = B.variance[src];
    const float g33[3][3] = {{1.0f / 16, 1.0f / 8, 1.0f / 16}, {1.0f / 8, 1.0f / 4, 1.0f / 8}, {1.0f / 16, 1.0f / 8, 1.0f / 16}};
    float vs = 0.f, vw = 0.f;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx)
        {
            const int sx = x + dx, sy = y + dy;
            if (sx < 0 || sx > W - 1 || sy < 0 || sy > H - 1) continue;
            float w = g33[dx + 1][dy + 1];
            vs = vs + __ldg(variance + (size_t)sy * W + sx) * w;
            vw = vw + w;
        }
    const float centreStd = sqrtf(fmaxf(vs / fmaxf(vw, kEpsMin), kEpsMin));
    const Features c = unpackFeatures(__ldg(B.feat0 + fi), __ldg(B.feat1 + fi));
    const float4 cc = __ldg(colour + fi);
    if (c.depth <= 0.0f)
    {
        outColour[fi] = cc;
        outVar[fi] = 0.0f;
        return;
    }
    const float3 cp = worldPosition(B, x, y, c.depth);
    const float g3[3] = {3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
    const int step = 1 << pass;
    float4 sumC = splat4(0.0f);
    float sumV = 0.f, sumW = 0.f;
    for (int dy = -2; dy <= 2; ++dy)
        for (int dx = -2; dx <= 2; ++dx)
        {
            const int sx = x + dx * step, sy = y + dy * step;
            if (sx < 0 || sx > W - 1 || sy < 0 || sy > H - 1) continue;
            const size_t si = (size_t)sy * W + sx;
            float kw = g3[abs(dx)] * g3[abs(dy)];
            const Features s = unpackFeatures(__ldg(B.feat0 + si), __ldg(B.feat1 + si));
            const float4 sc = __ldg(colour + si);
            const float sv = __ldg(variance + si);
            float wD = 1.0f;
            if (s.depth > 0.0f) wD = planeDistanceWeight(cp, c, worldPosition(B, sx, sy, s.depth), s, A);
            float wM = featureWeight(c, s, A, A.featureVarianceScale);
            float cd = fabsf(sc.y - cc.y);
            float wC = ygm_expf(-cd / (A.colorSigma * centreStd + kEpsMin));
            float w = kw * wD * wM * wC;
            sumC = sumC + sc * w;
            sumV = sumV + w * w * sv;
            sumW = sumW + w;
        }
    const float inv = 1.0f / fmaxf(sumW, kEpsMin);
    outColour[fi] = sumC * inv;
    outVar[fi] = sumV * inv * inv;
}

} // namespace

int launchAtrousGather(const SceneView& S, const LaunchParams& P, float4* moments, float4* odd, const float4* samples,
                       uint32_t nspp, int smCount, cudaStream_t stream)
{
    uint32_t npix = P.cropW * P.cropH;
    int threads = 128;
    int blocks = (int)std::min<uint64_t>((npix + threads - 1) / threads, (uint64_t)smCount * 16);
    if (blocks < 1) blocks = 1;
    atrousGather<<<blocks, threads, 0, stream>>>(S, P, moments, odd, samples, nspp);
    return 1;
}

// Prefilter, then `passes` a-trous passes ping-ponging between the two colour/variance
// planes; the last pass writes outColour/outVar. Returns the number of launches.
int launchAtrous(const AtrousBuffers& B, const AtrousSettings& A, float4* outColour, float* outVar, cudaStream_t stream)
{
    dim3 block(32, 8), grid((B.width + 31) / 32, (B.height + 7) / 8);
    atrousPrefilter<<<grid, block, 0, stream>>>(B, A);
    int launches = 1;
    uint32_t src = 0;
    for (uint32_t pass = 0; pass < A.passes; ++pass)
    {
        const bool last = pass + 1 == A.passes;
        float4* oc = last ? outColour : B.colour[src ^ 1u];
        float* ov = last ? outVar : B.variance[src ^ 1u];
        atrousPass<<<grid, block, 0, stream>>>(B, A, pass, src, oc, ov);
        ++launches;
        src ^= 1u;
    }
    if (A.passes == 0)
    {
        cudaMemcpyAsync(outColour, B.colour[0], (size_t)B.width * B.height * sizeof(float4), cudaMemcpyDeviceToDevice, stream);
        cudaMemcpyAsync(outVar, B.variance[0], (size_t)B.width * B.height * sizeof(float), cudaMemcpyDeviceToDevice, stream);
    }
    return launches;
}

} // namespace yg
