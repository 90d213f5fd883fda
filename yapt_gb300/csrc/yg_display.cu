// The display path of the reference's tonemap stage (TonemapStage.cpp with
// gatherLuminanceHistogram.comp, analyzeLuminanceHistogram.comp, prepareTonemapData.comp and
// tonemap.frag with TONEMAP_ACES), into a headless RGBA8 image:
//  * the source (the film mean, or the a-trous output) in linear sRGB, gamut clamped as the
//    denoiser's RGB conversion does (denoise.comp:279-336);
//  * a 128-bucket histogram of EV = log2(Y_perceived x 100 / 12.5) from EV -12, one shared-memory
//    histogram per 16x16 block folded into the global one;
//  * the weighted mean EV (one block of 128 threads);
//  * the exposure: manual, or the key 0.18 over the mean luminance with exposure compensation,
//    approached with 1 - exp(-dt x speed) per frame (the state lives on the device);
//  * exposure x colour, the ACES fitted curve (if enabled), clamped, encoded with the sRGB
//    transfer function to 8 bits (the swapchain's sRGB format).
#include "yg_kernels.h"
#include "yg_vec.cuh"

#include <algorithm>

namespace yg
{
namespace
{

constexpr int kBuckets = 128;   // HISTOGRAM_BUCKETS_COUNT
constexpr float kMinEV = -12.f; // TonemapStage.cpp:344
constexpr float kIsoCalib = 100.f / 12.5f;

__device__ __forceinline__ float3 sourceRGB(const DisplayArgs& A, size_t i)
{
    float3 xyz;
    if (A.atrous)
    {
        const float4 c = A.atrous[i];
        xyz = mk3(c.x, c.y, c.z);
    }
    else
    {
        const float4 s = A.film[i];
        const float inv = s.w > 0.0f ? 1.0f / s.w : 0.0f;
        xyz = mk3(s.x * inv, s.y * inv, s.z * inv);
    }
    // c_srgbXYZToRGB (colorSpaces.hlsl:18-23), then gamutClamp (denoise.comp:274-284)
    float3 c = mk3(3.2406f * xyz.x - 1.5372f * xyz.y - 0.4986f * xyz.z, -0.9689f * xyz.x + 1.8758f * xyz.y + 0.0415f * xyz.z,
                   0.0557f * xyz.x - 0.2040f * xyz.y + 1.0570f * xyz.z);
    const float lum = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
    const float m = fminf(fminf(c.x, c.y), c.z);
    if (m < 0.0f)
    {
        const float t = safeDiv(lum, lum - m);
        c = mk3(lum + (c.x - lum) * t, lum + (c.y - lum) * t, lum + (c.z - lum) * t);
    }
    return c;
}

__global__ void __launch_bounds__(256) gatherHistogram(DisplayArgs A)
{
    __shared__ uint32_t local[kBuckets];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid < kBuckets) local[tid] = 0;
    __syncthreads();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < A.width && y < A.height)
    {
        const float3 c = sourceRGB(A, (size_t)y * A.width + x);
        const float lum = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
        const float ev = log2f(lum * kIsoCalib);
        float b = ev - kMinEV;
        b = fminf(fmaxf(b, 0.0f), (float)(kBuckets - 1)); // NaN-free: log2(0) = -inf clamps to 0
        atomicAdd(&local[(uint32_t)floorf(b + 0.5f)], 1u);
    }
    __syncthreads();
    if (tid < kBuckets && local[tid]) atomicAdd(&A.histogram[tid], local[tid]);
}

// analyzeLuminanceHistogram + prepareTonemapData in one block
__global__ void __launch_bounds__(kBuckets) exposureFromHistogram(DisplayArgs A)
{
    __shared__ float sw[kBuckets], swe[kBuckets];
    const int i = threadIdx.x;
    const float w = (float)A.histogram[i];
    sw[i] = w;
    swe[i] = w * (kMinEV + (float)i);
    __syncthreads();
    for (int s = kBuckets / 2; s > 0; s >>= 1)
    {
        if (i < s)
        {
            sw[i] += sw[i + s];
            swe[i] += swe[i + s];
        }
        __syncthreads();
    }
    if (i == 0)
    {
        const float avgLum = exp2f(swe[0] / sw[0]) / kIsoCalib;
        float e;
        if (A.init || !A.autoExposure)
            e = A.exposureParam;
        else
        {
            const float prev = *A.exposure;
            const float ev = log2f(avgLum * kIsoCalib) + A.exposureParam;
            const float target = 0.18f / (exp2f(ev) / kIsoCalib);
            e = prev + (target - prev) * (1.0f - expf(-A.deltaTime * A.adaptSpeed));
        }
        *A.exposure = e;
        A.stats[0] = avgLum;
    }
}

// ACESFitted (tonemapUtils.hlsl:1-38)
__device__ float3 acesFitted(float3 c)
{
    float3 v = mk3(0.59719f * c.x + 0.35458f * c.y + 0.04823f * c.z, 0.07600f * c.x + 0.90834f * c.y + 0.01566f * c.z,
                   0.02840f * c.x + 0.13383f * c.y + 0.83777f * c.z);
    float3 a = mk3(v.x * (v.x + 0.0245786f) - 0.000090537f, v.y * (v.y + 0.0245786f) - 0.000090537f,
                   v.z * (v.z + 0.0245786f) - 0.000090537f);
    float3 b = mk3(v.x * (0.983729f * v.x + 0.4329510f) + 0.238081f, v.y * (0.983729f * v.y + 0.4329510f) + 0.238081f,
                   v.z * (0.983729f * v.z + 0.4329510f) + 0.238081f);
    v = mk3(a.x / b.x, a.y / b.y, a.z / b.z);
    return mk3(saturate(1.60475f * v.x - 0.53108f * v.y - 0.07367f * v.z),
               saturate(-0.10208f * v.x + 1.10813f * v.y - 0.00605f * v.z),
               saturate(-0.00327f * v.x - 0.07276f * v.y + 1.07602f * v.z));
}

__device__ __forceinline__ uint32_t srgb8(float v)
{
    v = saturate(v);
    const float e = v <= 0.0031308f ? 12.92f * v : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
    return (uint32_t)__float2int_rn(saturate(e) * 255.0f);
}

__global__ void __launch_bounds__(256) applyTonemap(DisplayArgs A)
{
    const size_t n = (size_t)A.width * A.height;
    const float e = *A.exposure;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    {
        float3 c = sourceRGB(A, i);
        c = mk3(c.x * e, c.y * e, c.z * e);
        if (A.tonemap) c = acesFitted(c);
        A.out[i] = srgb8(c.x) | (srgb8(c.y) << 8) | (srgb8(c.z) << 16) | (255u << 24);
    }
}

} // namespace

int launchDisplay(const DisplayArgs& A, int smCount, cudaStream_t stream)
{
    cudaMemsetAsync(A.histogram, 0, kBuckets * sizeof(uint32_t), stream);
    dim3 b(16, 16), g((A.width + 15) / 16, (A.height + 15) / 16);
    gatherHistogram<<<g, b, 0, stream>>>(A);
    exposureFromHistogram<<<1, kBuckets, 0, stream>>>(A);
    const size_t n = (size_t)A.width * A.height;
    int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)smCount * 8);
    applyTonemap<<<blocks < 1 ? 1 : blocks, 256, 0, stream>>>(A);
    return 3;
}

} // namespace yg
