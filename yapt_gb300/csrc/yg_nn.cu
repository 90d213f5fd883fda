// Denoiser network operators: BF16 tensor-core convolutions with FP32 accumulation for the
// U-Net's forward and backward passes, and the small operators around them.
//
// Tensors are NHWC (channels innermost) in BF16, each addressed with a channel stride and a
// channel offset so that a U-Net skip concatenation is just two writers into one buffer.
// Channel counts are multiples of 16.
//
// conv3x3: implicit GEMM, M = pixels, N = output channels, K = 9 taps x input channels, on the
// tcgen05 tensor cores with the accumulator in tensor memory: one CTA per 128 pixels of an
// image row and up to 256 output channels; the input halo of each channel chunk is staged once
// and every tap reads it through a shifted matrix descriptor. The default (conv3x3Tma) loads
// the operands with TMA boxes tracked by mbarrier transaction counts, one producer thread and
// one MMA thread; conv3x3Tc stages them with cp.async by all threads; a warp-level mma.sync
// m16n8k16 version (conv3x3Kernel: 128 x 64 tiles, cp.async + ldmatrix) is kept for
// comparison. The path is selectable (yg_nn_set_conv_impl). Both epilogues add the bias, apply ReLU or a
// ReLU-derivative mask, optionally accumulate into the destination, and store BF16. The data
// gradient is the same kernel on spatially flipped, transposed weights; the weight gradient is
// a split-K GEMM over pixels (mma.sync) with a deterministic reduction.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/yapt_gpu.h"

namespace ygnn
{
typedef __nv_bfloat16 bf16;

__device__ __forceinline__ void cpAsync16(void* smem, const void* gmem, bool valid)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    int n = valid ? 16 : 0; // src-size 0 zero-fills the 16 bytes
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cpAsyncWait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
__device__ __forceinline__ void ldmatrixX4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(s));
}
__device__ __forceinline__ void ldmatrixX4T(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(s));
}
__device__ __forceinline__ void mma16816(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct Act
{
    bf16* p;          // element (pixel q, channel c) at p[q * stride + off + c]
    uint32_t stride;  // channels per pixel in the buffer
    uint32_t off;     // first channel of this tensor
    uint32_t ch;      // channels of this tensor
};

// ------------------------------------------------------------------ 3x3 convolution (forward / data gradient)
constexpr int CM = 128, CN = 64, CSTAGES = 3;

template <int KC>
__global__ void __launch_bounds__(256) conv3x3Kernel(Act x, const bf16* __restrict__ w, const float* __restrict__ bias,
                                                     Act y, Act mask, int relu, int accumulate, int nImg, int H, int W)
{
    constexpr int RS = KC + 8; // shared row stride (elements): 16-byte aligned, ldmatrix conflict free
    __shared__ __align__(16) bf16 sA[CSTAGES][CM * RS];
    __shared__ __align__(16) bf16 sB[CSTAGES][CN * RS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp & 3, wn = warp >> 2;
    const long P = (long)nImg * H * W;
    const long m0 = (long)blockIdx.x * CM;
    const int n0 = blockIdx.y * CN;
    const int Cin = (int)x.ch, Cout = (int)y.ch;
    const int chunks = Cin / KC;
    const int kTiles = 9 * chunks;
    constexpr int SEGS = KC / 8; // 16-byte segments per row

    auto loadTile = [&](int kt, int stage) {
        const int tap = kt / chunks, c0 = (kt % chunks) * KC;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        for (int i = tid; i < CM * SEGS; i += 256)
        {
            int r = i / SEGS, sg = i % SEGS;
            long q = m0 + r;
            bool ok = q < P;
            const bf16* src = x.p;
            if (ok)
            {
                int img = (int)(q / ((long)H * W));
                int rem = (int)(q - (long)img * H * W);
                int yy = rem / W + dy, xx = rem % W + dx;
                ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
                if (ok) src = x.p + ((long)(img * H + yy) * W + xx) * x.stride + x.off + c0 + sg * 8;
            }
            cpAsync16(&sA[stage][r * RS + sg * 8], src, ok);
        }
        for (int i = tid; i < CN * SEGS; i += 256)
        {
            int r = i / SEGS, sg = i % SEGS;
            int co = n0 + r;
            bool ok = co < Cout;
            const bf16* src = ok ? w + ((long)co * 9 + tap) * Cin + c0 + sg * 8 : w;
            cpAsync16(&sB[stage][r * RS + sg * 8], src, ok);
        }
    };

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;

#pragma unroll
    for (int s = 0; s < CSTAGES - 1; ++s)
    {
        if (s < kTiles) loadTile(s, s);
        cpAsyncCommit();
    }
    for (int kt = 0; kt < kTiles; ++kt)
    {
        cpAsyncWait<CSTAGES - 2>();
        __syncthreads();
        const int nk = kt + CSTAGES - 1;
        if (nk < kTiles) loadTile(nk, nk % CSTAGES);
        cpAsyncCommit();
        const bf16* A = sA[kt % CSTAGES];
        const bf16* B = sB[kt % CSTAGES];
#pragma unroll
        for (int kk = 0; kk < KC; kk += 16)
        {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i)
            {
                int mi = lane >> 3, r = lane & 7;
                int row = wm * 32 + i * 16 + r + (mi & 1) * 8;
                int col = kk + (mi >> 1) * 8;
                ldmatrixX4(a[i][0], a[i][1], a[i][2], a[i][3], A + row * RS + col);
            }
#pragma unroll
            for (int j = 0; j < 4; j += 2)
            {
                int mi = lane >> 3, r = lane & 7;
                int row = wn * 32 + j * 8 + r + (mi >> 1) * 8;
                int col = kk + (mi & 1) * 8;
                ldmatrixX4(b[j][0], b[j][1], b[j + 1][0], b[j + 1][1], B + row * RS + col);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma16816(acc[i][j], a[i][0], a[i][1], a[i][2], a[i][3], b[j][0], b[j][1]);
        }
    }
    cpAsyncWait<0>();
    // epilogue
    const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            long q = m0 + wm * 32 + i * 16 + g + h * 8;
            if (q >= P) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                int co = n0 + wn * 32 + j * 8 + t4 * 2;
                if (co >= Cout) continue;
                float v0 = acc[i][j][h * 2], v1 = acc[i][j][h * 2 + 1];
                if (bias)
                {
                    v0 += bias[co];
                    v1 += bias[co + 1];
                }
                if (relu)
                {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                if (mask.p)
                {
                    __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask.p + q * mask.stride + mask.off + co);
                    if (!(__bfloat162float(mk.x) > 0.0f)) v0 = 0.0f;
                    if (!(__bfloat162float(mk.y) > 0.0f)) v1 = 0.0f;
                }
                __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(y.p + q * y.stride + y.off + co);
                if (accumulate)
                {
                    __nv_bfloat162 old = *dst;
                    v0 += __bfloat162float(old.x);
                    v1 += __bfloat162float(old.y);
                }
                *dst = __floats2bfloat162_rn(v0, v1);
            }
        }
}

// ------------------------------------------------------------------ 3x3 convolution on tcgen05
// The same implicit GEMM on the 5th-generation tensor cores: one CTA of 128 threads per 128
// output pixels and up to 256 output channels (N). The FP32 accumulator [128 x N] lives in
// tensor memory (TMEM, one column per output channel, one lane per pixel). Per K block (one
// tap, KC input channels) all threads stage the im2col A tile [128 x KC] and the weight tile
// B [N x KC] in shared memory with cp.async (zero fill outside the image), in the no-swizzle
// K-major layout of 8-row x 16-byte core matrices (core (g, k) at g * SBO + k * 128 bytes).
// One thread issues the tcgen05.mma instructions (kind::f16, BF16 x BF16 -> FP32, K = 16
// each) and commits them to the stage's mbarrier. Two stages: a stage is reloaded once the
// MMAs that read it have completed. The epilogue reads TMEM with tcgen05.ld (warp w owns
// lanes 32w..32w+31), adds the bias, applies ReLU / mask / accumulation and stores BF16.
// Every mbarrier wait is bounded; on a timeout the kernel records it, waits (bounded) for
// its MMAs, frees its TMEM and returns.
namespace tc
{
__device__ uint32_t g_timeouts; // waits that ran out (read by yg_nn_tc_timeouts)
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading (K) and stride (M/N) byte offsets in
// 16-byte units, descriptor version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5), BF16 A (bits 7-9) and B
// (bits 10-12), both K-major, N >> 3 (bits 17-22), M >> 4 (bits 24-28)
__host__ __device__ constexpr uint32_t idescBf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbarInit(uint32_t addr, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbarWait(uint32_t addr, uint32_t parity)
{
    for (uint32_t i = 0; i < kSpinLimit; ++i)
    {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok)
                     : "r"(addr), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

template <int KC, int NT>
struct TcShape
{
    static constexpr int HALO = 130;                          // input pixels per halo row (128 + 2)
    static constexpr uint32_t A_LBO = 3u * HALO * 16u;        // bytes between 8-channel groups of the halo
    static constexpr int A_BYTES = (int)A_LBO * (KC / 8);     // one channel chunk of the 3 halo rows
    static constexpr int TAP_BYTES = NT * KC * 2;             // one tap's weights for the chunk
    // taps per K block (9, 3 or 1): as many as fit beside the two halo buffers, so that one
    // synchronisation round issues enough MMAs
    static constexpr int FREE = 200704 - 2 * A_BYTES;
    static constexpr int TB = 2 * 9 * TAP_BYTES <= FREE ? 9 : (3 * 3 * TAP_BYTES <= FREE ? 3 : 1);
    static constexpr int B_BYTES = TB * TAP_BYTES;
    static constexpr int B_STAGES = TB == 9 ? 2 : 3;
    static constexpr int SMEM = 2 * A_BYTES + B_STAGES * B_BYTES;
    static constexpr uint32_t TCOLS = NT < 32 ? 32 : NT;
};

// One CTA computes 128 consecutive output pixels of one image row (x0..x0+127 of row y) for NT
// output channels. The three input rows y-1..y+1, columns x0-1..x0+128, of one chunk of KC
// input channels are staged once: 8-channel group g of halo pixel (r, c) at
// g * A_LBO + (r * 130 + c) * 16. Rows then sit 16 bytes apart within a group, so the A
// operand of tap (dy, dx) is the same buffer with its start shifted by
// ((1 + dy) * 130 + 1 + dx) * 16 bytes (SBO 128, LBO A_LBO): the nine taps read one copy of the
// input. B (the tap's NT x KC weights) goes through a three-deep ring; the MMAs of one K block
// (a chunk and a tap) are committed to that B stage's mbarrier.
template <int KC, int NT>
__global__ void __launch_bounds__(128) conv3x3Tc(Act x, const bf16* __restrict__ w, const float* __restrict__ bias, Act y,
                                                 Act mask, int relu, int accumulate, int nImg, int H, int W)
{
    using T = TcShape<KC, NT>;
    constexpr uint32_t IDESC = idescBf16(128, NT);
    constexpr uint32_t SBO_B = (KC / 8) * 128;
    constexpr int SEGS = KC / 8;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[T::B_STAGES];
    __shared__ uint32_t tmemSlot;
    __shared__ int abortFlag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tilesPerRow = (W + 127) / 128;
    const int rowTile = blockIdx.x % tilesPerRow;
    const int rowIdx = blockIdx.x / tilesPerRow; // image * H + y
    const int img = rowIdx / H, yy0 = rowIdx % H;
    const int x0 = rowTile * 128;
    const int n0 = blockIdx.y * NT;
    const int Cin = (int)x.ch;
    constexpr int GROUPS = 9 / T::TB; // K blocks per chunk
    const int chunks = Cin / KC, kBlocks = GROUPS * chunks;
    uint8_t* sA[2] = {smem, smem + T::A_BYTES};
    uint8_t* sBring = smem + 2 * T::A_BYTES;

    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(&tmemSlot)),
                     "r"(T::TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0)
    {
        for (int k = 0; k < T::B_STAGES; ++k) mbarInit(smemAddr(&mbar[k]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abortFlag = 0;
    }
    fenceBeforeSync();
    __syncthreads();
    fenceAfterSync();
    const uint32_t tmem = tmemSlot;

    auto loadA = [&](int c) {
        uint8_t* dst = sA[c & 1];
        const int c0 = c * KC;
        for (int i = tid; i < 3 * T::HALO * SEGS; i += 128)
        {
            const int sg = i % SEGS, px = i / SEGS;
            const int r = px / T::HALO, cc = px % T::HALO;
            const int yy = yy0 + r - 1, xx = x0 + cc - 1;
            const bool ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
            const bf16* src = ok ? x.p + ((long)(img * H + yy) * W + xx) * x.stride + x.off + c0 + sg * 8 : x.p;
            cpAsync16(dst + sg * T::A_LBO + px * 16, src, ok);
        }
    };
    auto loadB = [&](int kb) {
        uint8_t* dst = sBring + (kb % T::B_STAGES) * T::B_BYTES;
        const int c0 = (kb / GROUPS) * KC, tap0 = (kb % GROUPS) * T::TB;
        for (int i = tid; i < T::TB * NT * SEGS; i += 128)
        {
            const int t = i / (NT * SEGS), rs = i % (NT * SEGS);
            const int r = rs / SEGS, sg = rs % SEGS;
            const bf16* src = w + ((long)(n0 + r) * 9 + tap0 + t) * Cin + c0 + sg * 8;
            cpAsync16(dst + t * T::TAP_BYTES + (r >> 3) * SBO_B + sg * 128 + (r & 7) * 16, src, true);
        }
    };
    uint32_t parity[T::B_STAGES] = {};
    // waits for the MMAs of K block kb (its B stage's mbarrier); in order, so earlier blocks are done too
    auto waitBlock = [&](int kb) {
        const int stg = kb % T::B_STAGES;
        if (!mbarWait(smemAddr(&mbar[stg]), parity[stg])) abortFlag = 1;
        parity[stg] ^= 1u;
    };

    // prologue: A of chunk 0 and B of block 0
    loadA(0);
    loadB(0);
    cpAsyncCommit();
    int waitedUpTo = -1; // highest K block whose MMAs are known complete
    for (int kb = 0; kb < kBlocks; ++kb)
    {
        const int c = kb / GROUPS, grp = kb % GROUPS;
        // prefetch B of kb + 1 (its stage last served kb + 1 - B_STAGES) and, in the middle of
        // a chunk, A of the next chunk (its buffer last served chunk c - 1, done by then)
        const int nb = kb + 1;
        if (nb < kBlocks)
        {
            const int reuse = nb - T::B_STAGES;
            while (waitedUpTo < reuse) waitBlock(++waitedUpTo);
            loadB(nb);
        }
        if (grp == GROUPS / 2 && c + 1 < chunks)
        {
            const int lastOfPrev = GROUPS * c - 1;
            while (waitedUpTo < lastOfPrev) waitBlock(++waitedUpTo);
            loadA(c + 1);
        }
        cpAsyncCommit();
        if (__syncthreads_or(abortFlag)) break;
        cpAsyncWait<1>(); // everything but the group just issued
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0)
        {
            fenceAfterSync();
            const uint32_t aBase = smemAddr(sA[c & 1]);
            const uint32_t bBase = smemAddr(sBring + (kb % T::B_STAGES) * T::B_BYTES);
#pragma unroll
            for (int t = 0; t < T::TB; ++t)
            {
                const int tap = grp * T::TB + t;
                const int dy = tap / 3 - 1, dx = tap % 3 - 1;
                const uint32_t a0 = aBase + (uint32_t)(((1 + dy) * T::HALO + 1 + dx) * 16);
                const uint32_t b0 = bBase + t * T::TAP_BYTES;
#pragma unroll
                for (int kk = 0; kk < KC / 16; ++kk)
                {
                    const uint64_t ad = smemDesc(a0 + kk * 2 * T::A_LBO, T::A_LBO, 128);
                    const uint64_t bd = smemDesc(b0 + kk * 2 * 128, 128, SBO_B);
                    const uint32_t acc = (kb | t | kk) != 0 ? 1u : 0u;
                    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                                 "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                                 : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smemAddr(&mbar[kb % T::B_STAGES]))
                         : "memory");
        }
    }
    cpAsyncWait<0>();
    bool ok = !abortFlag;
    if (ok)
    {
        while (waitedUpTo < kBlocks - 1) waitBlock(++waitedUpTo);
        ok = !abortFlag;
    }
    else
    {
        // a wait ran out: drain what may still be in flight (bounded) before TMEM is freed
        for (int k = 0; k < T::B_STAGES; ++k) mbarWait(smemAddr(&mbar[k]), parity[k]);
    }
    if (__syncthreads_or(!ok))
    {
        if (tid == 0) atomicAdd(&g_timeouts, 1u);
    }
    else
    {
        fenceAfterSync();
        const int xo = x0 + warp * 32 + lane;
        const long q = ((long)(img * H + yy0)) * W + xo;
#pragma unroll 1
        for (int cc = 0; cc < NT; cc += 16)
        {
            uint32_t r[16];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                         : "r"(ta)
                         : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (xo >= W) continue;
#pragma unroll
            for (int j = 0; j < 16; j += 2)
            {
                const int co = n0 + cc + j;
                float v0 = __uint_as_float(r[j]), v1 = __uint_as_float(r[j + 1]);
                if (bias)
                {
                    v0 += bias[co];
                    v1 += bias[co + 1];
                }
                if (relu)
                {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                if (mask.p)
                {
                    __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask.p + q * mask.stride + mask.off + co);
                    if (!(__bfloat162float(mk.x) > 0.0f)) v0 = 0.0f;
                    if (!(__bfloat162float(mk.y) > 0.0f)) v1 = 0.0f;
                }
                __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(y.p + q * y.stride + y.off + co);
                if (accumulate)
                {
                    __nv_bfloat162 old = *dst;
                    v0 += __bfloat162float(old.x);
                    v1 += __bfloat162float(old.y);
                }
                *dst = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
    fenceBeforeSync();
    __syncthreads();
    if (warp == 0)
    {
        fenceAfterSync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(T::TCOLS) : "memory");
    }
}

// ------------------------------------------------------------------ the same convolution fed by TMA
// Operands arrive by the Tensor Memory Accelerator: one thread (warp 0) is the producer, one
// (warp 1) issues the MMAs, and the four warps share the epilogue. For every 8-channel group the
// producer loads the 3 x 130 halo as one 4-D box (channels, x, y, image; out-of-image pixels
// read as zero) into that group's block of the A buffer, and each tap's weights as one 3-D box
// (channels, tap, output channel) of NT rows; the stage's "full" mbarrier expects the bytes.
// The MMA thread waits for "full", issues the block's MMAs and commits them to the stage's
// "empty" mbarrier, which the producer waits for before reloading the stage. No thread
// barrier in the main loop. Layouts: A as in conv3x3Tc (groups padded to 128-byte
// multiples); B group-major, 8-channel group g of a tap at g * NT * 16 bytes (SBO 128,
// LBO NT * 16).
template <int KC, int NT>
struct TmaShape
{
    static constexpr int HALO = 130;
    static constexpr uint32_t A_GROUP = 3u * HALO * 16u;               // bytes the box writes
    static constexpr uint32_t A_LBO = (A_GROUP + 127u) / 128u * 128u;   // group pitch
    static constexpr int A_BYTES = (int)A_LBO * (KC / 8);
    static constexpr int TAP_BYTES = NT * KC * 2;
    static constexpr int FREE = 200704 - 2 * A_BYTES;
    static constexpr int TB = 2 * 9 * TAP_BYTES <= FREE ? 9 : (3 * 3 * TAP_BYTES <= FREE ? 3 : 1);
    static constexpr int B_BYTES = TB * TAP_BYTES;
    static constexpr int B_STAGES = TB == 9 ? 2 : 3;
    static constexpr int SMEM = 2 * A_BYTES + B_STAGES * B_BYTES;
    static constexpr uint32_t TCOLS = NT < 32 ? 32 : NT;
};

__device__ __forceinline__ void expectTx(uint32_t mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tmaLoad4(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, uint32_t mbar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(
                     dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void tmaLoad3(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t mbar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
                     dst),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
                 : "memory");
}

template <int KC, int NT>
__global__ void __launch_bounds__(128) conv3x3Tma(const __grid_constant__ CUtensorMap mapX, const __grid_constant__ CUtensorMap mapW,
                                                  const float* __restrict__ bias, Act x, Act y, Act mask, int relu,
                                                  int accumulate, int nImg, int H, int W)
{
    using T = TmaShape<KC, NT>;
    constexpr uint32_t IDESC = idescBf16(128, NT);
    constexpr int G = KC / 8;                 // 8-channel groups per chunk
    constexpr int GROUPS = 9 / T::TB;         // K blocks per chunk
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[T::B_STAGES], empty[T::B_STAGES], done;
    __shared__ uint32_t tmemSlot;
    __shared__ int abortFlag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tilesPerRow = (W + 127) / 128;
    const int rowTile = blockIdx.x % tilesPerRow;
    const int rowIdx = blockIdx.x / tilesPerRow;
    const int img = rowIdx / H, yy0 = rowIdx % H;
    const int x0 = rowTile * 128;
    const int n0 = blockIdx.y * NT;
    const int chunks = (int)x.ch / KC, kBlocks = GROUPS * chunks;
    const uint32_t sBase = smemAddr(smem);
    const uint32_t aBuf[2] = {sBase, sBase + T::A_BYTES};
    const uint32_t bRing = sBase + 2 * T::A_BYTES;

    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(&tmemSlot)),
                     "r"(T::TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0)
    {
        for (int k = 0; k < T::B_STAGES; ++k)
        {
            mbarInit(smemAddr(&full[k]), 1);
            mbarInit(smemAddr(&empty[k]), 1);
        }
        mbarInit(smemAddr(&done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abortFlag = 0;
    }
    fenceBeforeSync();
    __syncthreads();
    fenceAfterSync();
    const uint32_t tmem = tmemSlot;

    if (warp == 0 && lane == 0)
    {
        // producer
        int last = -1;
        for (int kb = 0; kb < kBlocks && !abortFlag; ++kb)
        {
            const int st = kb % T::B_STAGES, use = kb / T::B_STAGES;
            if (!mbarWait(smemAddr(&empty[st]), (uint32_t)(use & 1) ^ 1u))
            {
                abortFlag = 1;
                break;
            }
            const int c = kb / GROUPS, grp = kb % GROUPS;
            const uint32_t fb = smemAddr(&full[st]);
            expectTx(fb, (uint32_t)(T::TB * G * NT * 16) + (grp == 0 ? (uint32_t)(G * T::A_GROUP) : 0u));
            if (grp == 0)
                for (int g = 0; g < G; ++g)
                    tmaLoad4(aBuf[c & 1] + g * T::A_LBO, &mapX, (int)x.off + c * KC + 8 * g, x0 - 1, yy0 - 1, img, fb);
            const uint32_t sb = bRing + st * T::B_BYTES;
            for (int t = 0; t < T::TB; ++t)
                for (int g = 0; g < G; ++g)
                    tmaLoad3(sb + (t * G + g) * NT * 16, &mapW, c * KC + 8 * g, grp * T::TB + t, n0, fb);
            last = kb;
        }
        // on an abort, let the loads already issued land before the CTA can exit
        if (abortFlag && last >= 0) mbarWait(smemAddr(&full[last % T::B_STAGES]), (uint32_t)((last / T::B_STAGES) & 1));
    }
    else if (warp == 1 && lane == 0)
    {
        // MMA issue
        for (int kb = 0; kb < kBlocks && !abortFlag; ++kb)
        {
            const int st = kb % T::B_STAGES, use = kb / T::B_STAGES;
            if (!mbarWait(smemAddr(&full[st]), (uint32_t)(use & 1)))
            {
                abortFlag = 1;
                break;
            }
            fenceAfterSync();
            const int c = kb / GROUPS, grp = kb % GROUPS;
            const uint32_t sb = bRing + st * T::B_BYTES;
#pragma unroll
            for (int t = 0; t < T::TB; ++t)
            {
                const int tap = grp * T::TB + t;
                const int dy = tap / 3 - 1, dx = tap % 3 - 1;
                const uint32_t a0 = aBuf[c & 1] + (uint32_t)(((1 + dy) * T::HALO + 1 + dx) * 16);
                const uint32_t b0 = sb + t * G * NT * 16;
#pragma unroll
                for (int kk = 0; kk < KC / 16; ++kk)
                {
                    const uint64_t ad = smemDesc(a0 + kk * 2 * T::A_LBO, T::A_LBO, 128);
                    const uint64_t bd = smemDesc(b0 + kk * 2 * NT * 16, NT * 16, 128);
                    const uint32_t acc = (kb | t | kk) != 0 ? 1u : 0u;
                    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                                 "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                                 : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smemAddr(&empty[st]))
                         : "memory");
        }
        // completes when every MMA issued above has
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smemAddr(&done))
                     : "memory");
    }
    __syncwarp();
    const bool ok = mbarWait(smemAddr(&done), 0u);
    if (__syncthreads_or(!ok || abortFlag))
    {
        if (tid == 0) atomicAdd(&g_timeouts, 1u);
    }
    else
    {
        fenceAfterSync();
        const int xo = x0 + warp * 32 + lane;
        const long q = ((long)(img * H + yy0)) * W + xo;
#pragma unroll 1
        for (int cc = 0; cc < NT; cc += 16)
        {
            uint32_t r[16];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                         : "r"(ta)
                         : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (xo >= W) continue;
#pragma unroll
            for (int j = 0; j < 16; j += 2)
            {
                const int co = n0 + cc + j;
                float v0 = __uint_as_float(r[j]), v1 = __uint_as_float(r[j + 1]);
                if (bias)
                {
                    v0 += bias[co];
                    v1 += bias[co + 1];
                }
                if (relu)
                {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                if (mask.p)
                {
                    __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask.p + q * mask.stride + mask.off + co);
                    if (!(__bfloat162float(mk.x) > 0.0f)) v0 = 0.0f;
                    if (!(__bfloat162float(mk.y) > 0.0f)) v1 = 0.0f;
                }
                __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(y.p + q * y.stride + y.off + co);
                if (accumulate)
                {
                    __nv_bfloat162 old = *dst;
                    v0 += __bfloat162float(old.x);
                    v1 += __bfloat162float(old.y);
                }
                *dst = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
    fenceBeforeSync();
    __syncthreads();
    if (warp == 0)
    {
        fenceAfterSync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(T::TCOLS) : "memory");
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                  const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiled()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried)
    {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

template <int KC, int NT>
int launchTma(const Act& x, const bf16* w, const float* bias, const Act& y, const Act& m, int relu, int accumulate, int n,
              int h, int wd, cudaStream_t st)
{
    using T = TmaShape<KC, NT>;
    EncodeTiledFn enc = encodeTiled();
    if (!enc) return YG_ERR_CUDA;
    alignas(64) CUtensorMap mapX, mapW;
    // activations: (channels of the buffer, x, y, image); boxes of 8 channels x 130 x 3 x 1
    const cuuint64_t dimX[4] = {x.stride, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strideX[3] = {(cuuint64_t)x.stride * 2, (cuuint64_t)x.stride * 2 * wd, (cuuint64_t)x.stride * 2 * wd * h};
    const cuuint32_t boxX[4] = {8, (cuuint32_t)T::HALO, 3, 1};
    const cuuint32_t ones[4] = {1, 1, 1, 1};
    if (enc(&mapX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)x.p, dimX, strideX, boxX, ones, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return YG_ERR_CUDA;
    // weights [Cout][3][3][Cin]: (input channel, tap, output channel); boxes of 8 x 1 x NT
    const cuuint64_t dimW[3] = {x.ch, 9, y.ch};
    const cuuint64_t strideW[2] = {(cuuint64_t)x.ch * 2, (cuuint64_t)x.ch * 2 * 9};
    const cuuint32_t boxW[3] = {8, 1, (cuuint32_t)NT};
    if (enc(&mapW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)w, dimW, strideW, boxW, ones, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return YG_ERR_CUDA;
    constexpr int floorBytes = 233472 / (512 / (int)T::TCOLS) - 2047;
    constexpr int smemBytes = T::SMEM > floorBytes ? T::SMEM : floorBytes;
    static_assert(smemBytes <= 232448, "shared memory");
    static bool configured = false;
    if (!configured)
    {
        if (cudaFuncSetAttribute(conv3x3Tma<KC, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes) != cudaSuccess)
            return YG_ERR_CUDA;
        configured = true;
    }
    dim3 grid((unsigned)(n * h * ((wd + 127) / 128)), (unsigned)(y.ch / NT));
    conv3x3Tma<KC, NT><<<grid, 128, smemBytes, st>>>(mapX, mapW, bias, x, y, m, relu, accumulate, n, h, wd);
    return YG_OK;
}

template <int KC>
int launchTmaN(const Act& x, const bf16* w, const float* bias, const Act& y, const Act& m, int relu, int accumulate, int n,
               int h, int wd, cudaStream_t st)
{
    const int c = (int)y.ch;
    if (c % 256 == 0) return launchTma<KC, 256>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    if (c % 128 == 0) return launchTma<KC, 128>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    if (c % 64 == 0) return launchTma<KC, 64>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    if (c % 32 == 0) return launchTma<KC, 32>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    return YG_ERR_INVALID_ARGUMENT;
}

// ------------------------------------------------------------------ persistent TMA + tcgen05 convolution
// For layers whose whole input window (all Cin channels of a 3 x 130-pixel halo, twice) and all
// nine taps of weights fit in shared memory: Cin <= 96 and N <= 64, the full- and half-resolution
// layers. Their few MMAs per 128-pixel tile left conv3x3Tma waiting on loads and set-up, so here a
// persistent CTA walks a strided sequence of row tiles: the weights load once, the halo of the next
// tile loads while the current one multiplies (two A buffers), and the accumulator alternates
// between two TMEM buffers so that the epilogue of one tile overlaps the MMAs of the next.
// Warps 0-3 run the epilogue (warp w reads TMEM lanes 32w..32w+31), warp 4 lane 0 issues the TMA
// loads, warp 5 lane 0 the MMAs. Barriers: wFull (weights), aFull/aEmpty (A buffers), accFull
// (MMAs of a tile complete) and accEmpty (its epilogue has read TMEM, one arrival per epilogue
// warp). Every wait is bounded; a time-out stops every role, the producer waits for its issued
// loads and every thread for the issued MMAs before TMEM is freed, and the time-out is counted.
template <int CIN, int NT>
struct PersistShape
{
    static constexpr int HALO = 130;
    static constexpr int G = CIN / 8;
    static constexpr uint32_t A_GROUP = 3u * HALO * 16u;
    static constexpr uint32_t A_LBO = (A_GROUP + 127u) / 128u * 128u;
    static constexpr int A_BYTES = (int)A_LBO * G;
    static constexpr int W_BYTES = 9 * G * NT * 16;
    static constexpr int SMEM = 2 * A_BYTES + W_BYTES;
    static constexpr uint32_t TCOLS = 2 * NT;
};

__device__ __forceinline__ void mbarArrive(uint32_t addr)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(addr) : "memory");
}

template <int CIN, int NT>
__global__ void __launch_bounds__(192) conv3x3Persist(const __grid_constant__ CUtensorMap mapX,
                                                      const __grid_constant__ CUtensorMap mapW, const float* __restrict__ bias,
                                                      Act x, Act y, Act mask, int relu, int accumulate, int nImg, int H, int W)
{
    using T = PersistShape<CIN, NT>;
    constexpr uint32_t IDESC = idescBf16(128, NT);
    constexpr int G = T::G;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t wFull, aFull[2], aEmpty[2], accFull[2], accEmpty[2], done;
    __shared__ uint32_t tmemSlot;
    __shared__ volatile int abortFlag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tilesPerRow = (W + 127) / 128;
    const int nTiles = nImg * H * tilesPerRow;
    const int n0 = blockIdx.y * NT;
    const uint32_t sBase = smemAddr(smem);
    const uint32_t aBuf[2] = {sBase, sBase + T::A_BYTES};
    const uint32_t wBuf = sBase + 2 * T::A_BYTES;

    if (warp == 4)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(&tmemSlot)),
                     "r"(T::TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0)
    {
        mbarInit(smemAddr(&wFull), 1);
        for (int k = 0; k < 2; ++k)
        {
            mbarInit(smemAddr(&aFull[k]), 1);
            mbarInit(smemAddr(&aEmpty[k]), 1);
            mbarInit(smemAddr(&accFull[k]), 1);
            mbarInit(smemAddr(&accEmpty[k]), 4);
        }
        mbarInit(smemAddr(&done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abortFlag = 0;
    }
    fenceBeforeSync();
    __syncthreads();
    fenceAfterSync();
    const uint32_t tmem = tmemSlot;

    if (warp == 4)
    {
        if (lane == 0)
        {
            // producer: the weights once, then the halo of every tile of this CTA
            const uint32_t wf = smemAddr(&wFull);
            expectTx(wf, (uint32_t)T::W_BYTES);
            for (int t = 0; t < 9; ++t)
                for (int g = 0; g < G; ++g) tmaLoad3(wBuf + (t * G + g) * NT * 16, &mapW, 8 * g, t, n0, wf);
            int issued = 0;
            for (int tile = blockIdx.x; tile < nTiles && !abortFlag; tile += gridDim.x, ++issued)
            {
                const int b = issued & 1, use = issued >> 1;
                if (!mbarWait(smemAddr(&aEmpty[b]), (uint32_t)(use & 1) ^ 1u))
                {
                    abortFlag = 1;
                    break;
                }
                const int rowIdx = tile / tilesPerRow, x0 = (tile % tilesPerRow) * 128;
                const int img = rowIdx / H, yy0 = rowIdx % H;
                const uint32_t fb = smemAddr(&aFull[b]);
                expectTx(fb, (uint32_t)(G * T::A_GROUP));
                for (int g = 0; g < G; ++g)
                    tmaLoad4(aBuf[b] + g * T::A_LBO, &mapX, (int)x.off + 8 * g, x0 - 1, yy0 - 1, img, fb);
            }
            // the CTA may not exit before its loads have landed
            mbarWait(wf, 0u);
            if (issued > 0) mbarWait(smemAddr(&aFull[(issued - 1) & 1]), (uint32_t)(((issued - 1) >> 1) & 1));
        }
    }
    else if (warp == 5)
    {
        if (lane == 0)
        {
            // MMA issue: nine taps x Cin / 16 MMAs per tile into the tile's TMEM buffer
            if (!mbarWait(smemAddr(&wFull), 0u)) abortFlag = 1;
            int it = 0;
            for (int tile = blockIdx.x; tile < nTiles && !abortFlag; tile += gridDim.x, ++it)
            {
                const int b = it & 1, use = it >> 1;
                if (!mbarWait(smemAddr(&aFull[b]), (uint32_t)(use & 1)) ||
                    !mbarWait(smemAddr(&accEmpty[b]), (uint32_t)(use & 1) ^ 1u))
                {
                    abortFlag = 1;
                    break;
                }
                fenceAfterSync();
                const uint32_t d = tmem + (uint32_t)(b * NT);
#pragma unroll
                for (int t = 0; t < 9; ++t)
                {
                    const int dy = t / 3 - 1, dx = t % 3 - 1;
                    const uint32_t a0 = aBuf[b] + (uint32_t)(((1 + dy) * T::HALO + 1 + dx) * 16);
                    const uint32_t b0 = wBuf + t * G * NT * 16;
#pragma unroll
                    for (int kk = 0; kk < CIN / 16; ++kk)
                    {
                        const uint64_t ad = smemDesc(a0 + kk * 2 * T::A_LBO, T::A_LBO, 128);
                        const uint64_t bd = smemDesc(b0 + kk * 2 * NT * 16, NT * 16, 128);
                        const uint32_t acc = (t | kk) != 0 ? 1u : 0u;
                        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                     " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                                     "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                                     : "memory");
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smemAddr(&aEmpty[b]))
                             : "memory");
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smemAddr(&accFull[b]))
                             : "memory");
            }
            // completes when every MMA issued above has
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smemAddr(&done))
                         : "memory");
        }
    }
    else
    {
        // epilogue: bias, ReLU, mask, accumulation, BF16 stores of the tile's 128 pixels x NT
        int it = 0;
        for (int tile = blockIdx.x; tile < nTiles; tile += gridDim.x, ++it)
        {
            const int b = it & 1, use = it >> 1;
            const bool ready = mbarWait(smemAddr(&accFull[b]), (uint32_t)(use & 1));
            if (!ready || abortFlag)
            {
                abortFlag = 1;
                break;
            }
            fenceAfterSync();
            const int rowIdx = tile / tilesPerRow, x0 = (tile % tilesPerRow) * 128;
            const int img = rowIdx / H, yy0 = rowIdx % H;
            const int xo = x0 + warp * 32 + lane;
            const long q = ((long)(img * H + yy0)) * W + xo;
#pragma unroll 1
            for (int cc = 0; cc < NT; cc += 16)
            {
                uint32_t r[16];
                const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * NT + cc);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                             : "r"(ta)
                             : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (xo >= W) continue;
#pragma unroll
                for (int j = 0; j < 16; j += 2)
                {
                    const int co = n0 + cc + j;
                    float v0 = __uint_as_float(r[j]), v1 = __uint_as_float(r[j + 1]);
                    if (bias)
                    {
                        v0 += bias[co];
                        v1 += bias[co + 1];
                    }
                    if (relu)
                    {
                        v0 = fmaxf(v0, 0.0f);
                        v1 = fmaxf(v1, 0.0f);
                    }
                    if (mask.p)
                    {
                        __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask.p + q * mask.stride + mask.off + co);
                        if (!(__bfloat162float(mk.x) > 0.0f)) v0 = 0.0f;
                        if (!(__bfloat162float(mk.y) > 0.0f)) v1 = 0.0f;
                    }
                    __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(y.p + q * y.stride + y.off + co);
                    if (accumulate)
                    {
                        __nv_bfloat162 old = *dst;
                        v0 += __bfloat162float(old.x);
                        v1 += __bfloat162float(old.y);
                    }
                    *dst = __floats2bfloat162_rn(v0, v1);
                }
            }
            // TMEM buffer b read: the MMAs of the tile after next may overwrite it
            fenceBeforeSync();
            __syncwarp();
            if (lane == 0) mbarArrive(smemAddr(&accEmpty[b]));
        }
    }
    __syncwarp();
    const bool ok = mbarWait(smemAddr(&done), 0u);
    if (__syncthreads_or(!ok || abortFlag))
    {
        if (tid == 0) atomicAdd(&g_timeouts, 1u);
    }
    fenceBeforeSync();
    __syncthreads();
    if (warp == 4)
    {
        fenceAfterSync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(T::TCOLS) : "memory");
    }
}

template <int CIN, int NT>
int launchPersist(const Act& x, const bf16* w, const float* bias, const Act& y, const Act& m, int relu, int accumulate, int n,
                  int h, int wd, int smCount, cudaStream_t st)
{
    using T = PersistShape<CIN, NT>;
    EncodeTiledFn enc = encodeTiled();
    if (!enc) return YG_ERR_CUDA;
    alignas(64) CUtensorMap mapX, mapW;
    const cuuint64_t dimX[4] = {x.stride, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strideX[3] = {(cuuint64_t)x.stride * 2, (cuuint64_t)x.stride * 2 * wd, (cuuint64_t)x.stride * 2 * wd * h};
    const cuuint32_t boxX[4] = {8, (cuuint32_t)T::HALO, 3, 1};
    const cuuint32_t ones[4] = {1, 1, 1, 1};
    if (enc(&mapX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)x.p, dimX, strideX, boxX, ones, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return YG_ERR_CUDA;
    const cuuint64_t dimW[3] = {x.ch, 9, y.ch};
    const cuuint64_t strideW[2] = {(cuuint64_t)x.ch * 2, (cuuint64_t)x.ch * 2 * 9};
    const cuuint32_t boxW[3] = {8, 1, (cuuint32_t)NT};
    if (enc(&mapW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)w, dimW, strideW, boxW, ones, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return YG_ERR_CUDA;
    // at most 512 / TCOLS CTAs per SM may hold tensor memory at once: the shared-memory request
    // is raised until no more CTAs than that fit on an SM, so an allocation never waits
    constexpr int floorBytes = 233472 / (512 / (int)T::TCOLS) - 2047;
    constexpr int smemBytes = T::SMEM > floorBytes ? T::SMEM : floorBytes;
    static_assert(smemBytes <= 232448, "shared memory");
    static bool configured = false;
    if (!configured)
    {
        if (cudaFuncSetAttribute(conv3x3Persist<CIN, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes) != cudaSuccess)
            return YG_ERR_CUDA;
        configured = true;
    }
    int perSm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, conv3x3Persist<CIN, NT>, 192, smemBytes) != cudaSuccess || perSm < 1)
        return YG_ERR_CUDA;
    const int nCols = (int)(y.ch / NT);
    const long tiles = (long)n * h * ((wd + 127) / 128);
    const long want = std::max<long>(1, (long)smCount * perSm / nCols);
    dim3 grid((unsigned)std::min<long>(tiles, want), (unsigned)nCols);
    conv3x3Persist<CIN, NT><<<grid, 192, smemBytes, st>>>(mapX, mapW, bias, x, y, m, relu, accumulate, n, h, wd);
    return YG_OK;
}

// the persistent kernel where its shape is built; 1 where the layer takes conv3x3Tma instead
int launchPersistAny(const Act& x, const bf16* w, const float* bias, const Act& y, const Act& m, int relu, int accumulate,
                     int n, int h, int wd, int smCount, cudaStream_t st)
{
    const int ci = (int)x.ch, co = (int)y.ch;
#define YG_PERSIST(CI, N)                                                                                                   \
    if (ci == CI && co % N == 0) return launchPersist<CI, N>(x, w, bias, y, m, relu, accumulate, n, h, wd, smCount, st);
    YG_PERSIST(16, 32)
    YG_PERSIST(32, 64)
    YG_PERSIST(32, 32)
    YG_PERSIST(64, 64)
    YG_PERSIST(96, 32)
#undef YG_PERSIST
    return 1;
}

template <int KC, int NT>
int launchTc(const Act& x, const bf16* w, const float* bias, const Act& y, const Act& m, int relu, int accumulate, int n,
             int h, int wd, cudaStream_t st)
{
    using T = TcShape<KC, NT>;
    // at most 512 / TCOLS CTAs per SM may hold tensor memory at once, so the shared-memory
    // request is raised until no more CTAs than that fit on an SM (228 KB each): an
    // allocation then never waits for another CTA's columns
    constexpr int floorBytes = 233472 / (512 / (int)T::TCOLS) - 2047;
    constexpr int smemBytes = T::SMEM > floorBytes ? T::SMEM : floorBytes;
    static_assert(smemBytes <= 232448, "shared memory");
    static bool configured = false;
    if (!configured)
    {
        if (cudaFuncSetAttribute(conv3x3Tc<KC, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes) != cudaSuccess)
            return YG_ERR_CUDA;
        configured = true;
    }
    dim3 grid((unsigned)(n * h * ((wd + 127) / 128)), (unsigned)(y.ch / NT));
    conv3x3Tc<KC, NT><<<grid, 128, smemBytes, st>>>(x, w, bias, y, m, relu, accumulate, n, h, wd);
    return YG_OK;
}

template <int KC>
int launchTcN(const Act& x, const bf16* w, const float* bias, const Act& y, const Act& m, int relu, int accumulate, int n,
              int h, int wd, cudaStream_t st)
{
    const int c = (int)y.ch;
    if (c % 256 == 0) return launchTc<KC, 256>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    if (c % 128 == 0) return launchTc<KC, 128>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    if (c % 64 == 0) return launchTc<KC, 64>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    if (c % 32 == 0) return launchTc<KC, 32>(x, w, bias, y, m, relu, accumulate, n, h, wd, st);
    return YG_ERR_INVALID_ARGUMENT;
}
} // namespace tc

// ------------------------------------------------------------------ 3x3 weight gradient
// dW[co][tap][ci] = sum_q dY[q][co] * X[q shifted by tap][ci]: M = Cout (64 per block),
// N = Cin (64 per block) for one tap, K = pixels, split over blocks (gridDim.z).
constexpr int WM = 64, WN = 64, WK = 32;

__global__ void __launch_bounds__(256) conv3x3WgradKernel(Act x, Act dy, float* __restrict__ partial, int nImg, int H,
                                                          int W, long pixelsPerSplit)
{
    constexpr int RS = 64 + 8; // rows are pixels (k), 64 channels each, padded
    __shared__ __align__(16) bf16 sY[2][WK * RS]; // [k][m]
    __shared__ __align__(16) bf16 sX[2][WK * RS]; // [k][n]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp & 1, wn = warp >> 1; // 2 x 4 warps: 32 (m) x 16 (n) each
    const int Cin = (int)x.ch, Cout = (int)dy.ch;
    const int nBlocksN = (Cin + WN - 1) / WN;
    const int tap = blockIdx.y / nBlocksN;
    const int c0 = (blockIdx.y % nBlocksN) * WN;
    const int o0 = blockIdx.x * WM;
    const int ddy = tap / 3 - 1, ddx = tap % 3 - 1;
    const long P = (long)nImg * H * W;
    const long q0 = (long)blockIdx.z * pixelsPerSplit;
    const long q1 = min(P, q0 + pixelsPerSplit);

    auto load = [&](long qb, int stage) {
        // 32 pixels x 64 channels for each operand: 256 segments of 16 bytes each
        for (int i = tid; i < WK * 8; i += 256)
        {
            int r = i >> 3, sg = i & 7;
            long q = qb + r;
            bool okq = q < q1;
            int co = o0 + sg * 8;
            bool okY = okq && co < Cout;
            const bf16* srcY = okY ? dy.p + q * dy.stride + dy.off + co : dy.p;
            cpAsync16(&sY[stage][r * RS + sg * 8], srcY, okY);
            int ci = c0 + sg * 8;
            bool okX = okq && ci < Cin;
            const bf16* srcX = x.p;
            if (okX)
            {
                int img = (int)(q / ((long)H * W));
                int rem = (int)(q - (long)img * H * W);
                int yy = rem / W + ddy, xx = rem % W + ddx;
                okX = yy >= 0 && yy < H && xx >= 0 && xx < W;
                if (okX) srcX = x.p + ((long)(img * H + yy) * W + xx) * x.stride + x.off + ci;
            }
            cpAsync16(&sX[stage][r * RS + sg * 8], srcX, okX);
        }
    };
    float acc[2][2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;
    const long nk = (q1 - q0 + WK - 1) / WK;
    if (nk > 0) load(q0, 0);
    cpAsyncCommit();
    for (long kt = 0; kt < nk; ++kt)
    {
        if (kt + 1 < nk) load(q0 + (kt + 1) * WK, (kt + 1) & 1);
        cpAsyncCommit();
        cpAsyncWait<1>();
        __syncthreads();
        const bf16* Ys = sY[kt & 1];
        const bf16* Xs = sX[kt & 1];
#pragma unroll
        for (int kk = 0; kk < WK; kk += 16)
        {
            uint32_t a[2][4], b[2][2];
            // A = dY^T (m = channel, k = pixel) from [k][m] storage: transposed loads
#pragma unroll
            for (int i = 0; i < 2; ++i)
            {
                int mi = lane >> 3, r = lane & 7;
                // matrices: (m0-7,k0-7) (m8-15,k0-7) (m0-7,k8-15) (m8-15,k8-15)
                int krow = kk + r + (mi >> 1) * 8;
                int mcol = wm * 32 + i * 16 + (mi & 1) * 8;
                ldmatrixX4T(a[i][0], a[i][1], a[i][2], a[i][3], Ys + krow * RS + mcol);
            }
            // B = X (k = pixel, n = channel) from [k][n] storage: transposed loads give the col layout
            {
                int mi = lane >> 3, r = lane & 7;
                // matrices: (k0-7,n0-7) (k8-15,n0-7) (k0-7,n8-15) (k8-15,n8-15)
                int krow = kk + r + (mi & 1) * 8;
                int ncol = wn * 16 + (mi >> 1) * 8;
                ldmatrixX4T(b[0][0], b[0][1], b[1][0], b[1][1], Xs + krow * RS + ncol);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) mma16816(acc[i][j], a[i][0], a[i][1], a[i][2], a[i][3], b[j][0], b[j][1]);
        }
        __syncthreads();
    }
    cpAsyncWait<0>();
    const int g = lane >> 2, t4 = lane & 3;
    float* out = partial + (long)blockIdx.z * Cout * 9 * Cin;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            int co = o0 + wm * 32 + i * 16 + g + h * 8;
            if (co >= Cout) continue;
#pragma unroll
            for (int j = 0; j < 2; ++j)
            {
                int ci = c0 + wn * 16 + j * 8 + t4 * 2;
                if (ci >= Cin) continue;
                float* o = out + ((long)co * 9 + tap) * Cin + ci;
                o[0] = acc[i][j][h * 2];
                o[1] = acc[i][j][h * 2 + 1];
            }
        }
}

// sums the split-K partials in split order (deterministic) into dW
__global__ void reduceSplits(const float* __restrict__ partial, int splits, long n, float* __restrict__ out)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        float s = 0.0f;
        for (int k = 0; k < splits; ++k) s += partial[(long)k * n + i];
        out[i] = s;
    }
}

// bias gradient: per channel sum over pixels, one block per channel group, fixed order
__global__ void biasGrad(Act dy, long P, float* __restrict__ db)
{
    const int c = blockIdx.x;
    float s = 0.0f;
    for (long q = threadIdx.x; q < P; q += blockDim.x) s += __bfloat162float(dy.p[q * dy.stride + dy.off + c]);
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1)
    {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = red[0];
}

// Wt[ci][8 - tap][co] = W[co][tap][ci]: the data gradient as a forward convolution
__global__ void flipWeights(const bf16* __restrict__ w, int Cout, int Cin, bf16* __restrict__ wt)
{
    long n = (long)Cout * 9 * Cin;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        int ci = (int)(i % Cin);
        int tap = (int)((i / Cin) % 9);
        int co = (int)(i / ((long)Cin * 9));
        wt[((long)ci * 9 + (8 - tap)) * Cout + co] = w[i];
    }
}

// ------------------------------------------------------------------ pooling / upsampling
// 2x2 average pooling: out (H/2 x W/2) from in
__global__ void avgPool(Act in, Act out, int nImg, int H, int W)
{
    const int Ho = H / 2, Wo = W / 2, C = (int)in.ch;
    long n = (long)nImg * Ho * Wo * C;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        int c = (int)(i % C);
        long q = i / C;
        int xo = (int)(q % Wo), yo = (int)((q / Wo) % Ho), img = (int)(q / ((long)Wo * Ho));
        float s = 0.0f;
        for (int k = 0; k < 4; ++k)
        {
            long qi = ((long)(img * H + 2 * yo + (k >> 1)) * W + 2 * xo + (k & 1));
            s += __bfloat162float(in.p[qi * in.stride + in.off + c]);
        }
        out.p[q * out.stride + out.off + c] = __float2bfloat16_rn(s * 0.25f);
    }
}
// dIn = dOut/4 spread over the 2x2 window (+ add, when add.p), times the ReLU mask of the pooled tensor
__global__ void avgPoolBwd(Act dOut, Act add, Act mask, Act dIn, int nImg, int H, int W)
{
    const int Wo = W / 2, Ho = H / 2, C = (int)dIn.ch;
    long n = (long)nImg * H * W * C;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        int c = (int)(i % C);
        long q = i / C;
        int x = (int)(q % W), y = (int)((q / W) % H), img = (int)(q / ((long)W * H));
        long qo = ((long)(img * Ho + y / 2) * Wo + x / 2);
        float v = 0.25f * __bfloat162float(dOut.p[qo * dOut.stride + dOut.off + c]);
        if (add.p) v += __bfloat162float(add.p[q * add.stride + add.off + c]);
        if (mask.p && !(__bfloat162float(mask.p[q * mask.stride + mask.off + c]) > 0.0f)) v = 0.0f;
        dIn.p[q * dIn.stride + dIn.off + c] = __float2bfloat16_rn(v);
    }
}
// nearest 2x upsampling: out (2H x 2W) from in (H x W)
__global__ void upsample(Act in, Act out, int nImg, int H, int W)
{
    const int Ho = 2 * H, Wo = 2 * W, C = (int)in.ch;
    long n = (long)nImg * Ho * Wo * C;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        int c = (int)(i % C);
        long q = i / C;
        int x = (int)(q % Wo), y = (int)((q / Wo) % Ho), img = (int)(q / ((long)Wo * Ho));
        long qi = ((long)(img * H + y / 2) * W + x / 2);
        out.p[q * out.stride + out.off + c] = in.p[qi * in.stride + in.off + c];
    }
}
// dIn (H x W) = sum of the 2x2 block of dOut (2H x 2W), times the ReLU mask of the upsampled tensor
__global__ void upsampleBwd(Act dOut, Act mask, Act dIn, int nImg, int H, int W)
{
    const int Wo = 2 * W, C = (int)dIn.ch;
    long n = (long)nImg * H * W * C;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        int c = (int)(i % C);
        long q = i / C;
        int x = (int)(q % W), y = (int)((q / W) % H), img = (int)(q / ((long)W * H));
        float s = 0.0f;
        for (int k = 0; k < 4; ++k)
        {
            long qo = ((long)(img * 2 * H + 2 * y + (k >> 1)) * Wo + 2 * x + (k & 1));
            s += __bfloat162float(dOut.p[qo * dOut.stride + dOut.off + c]);
        }
        if (mask.p && !(__bfloat162float(mask.p[q * mask.stride + mask.off + c]) > 0.0f)) s = 0.0f;
        dIn.p[q * dIn.stride + dIn.off + c] = __float2bfloat16_rn(s);
    }
}

// ------------------------------------------------------------------ head, loss and its gradient
// out = expm1(W x + b + skip) (linear RGB; 1x1 convolution from C features in FP32 arithmetic,
// added to the first three channels of `skip`, the log1p radiance of the noisy input, so the
// network predicts a correction in log space and a clean input passes through);
// loss = mean over pixels and 3 channels of (out - t)^2 / (t^2 + eps). With dIn set, writes
// the gradient of the loss wrt x (BF16) and per-block partial gradients of W and b.
constexpr int HEAD_C = 32;
__global__ void __launch_bounds__(256) headKernel(Act in, Act skip, const float* __restrict__ w, const float* __restrict__ b, long P,
                                                  float* __restrict__ out, const float* __restrict__ target, float eps,
                                                  float* __restrict__ lossPartial, Act dIn, float* __restrict__ gwPartial)
{
    __shared__ float sw[3 * HEAD_C + 3];
    __shared__ float red[256];
    for (int i = threadIdx.x; i < 3 * HEAD_C + 3; i += blockDim.x) sw[i] = i < 3 * HEAD_C ? w[i] : b[i - 3 * HEAD_C];
    __syncthreads();
    float lsum = 0.0f;
    float gw[3 * HEAD_C + 3];
    if (dIn.p)
        for (int i = 0; i < 3 * HEAD_C + 3; ++i) gw[i] = 0.0f;
    const long per = (P + gridDim.x - 1) / gridDim.x;
    const long qb = (long)blockIdx.x * per, qe = min(P, qb + per);
    for (long q = qb + threadIdx.x; q < qe; q += blockDim.x)
    {
        float xv[HEAD_C];
        for (int c = 0; c < HEAD_C; ++c) xv[c] = __bfloat162float(in.p[q * in.stride + in.off + c]);
        float dz[3];
        for (int o = 0; o < 3; ++o)
        {
            float z = sw[3 * HEAD_C + o];
            for (int c = 0; c < HEAD_C; ++c) z += sw[o * HEAD_C + c] * xv[c];
            if (skip.p) z += __bfloat162float(skip.p[q * skip.stride + skip.off + o]);
            float e = expf(fminf(z, 20.0f));
            float y = e - 1.0f;
            if (out) out[q * 3 + o] = y;
            dz[o] = 0.0f;
            if (target)
            {
                float t = target[q * 3 + o];
                float den = t * t + eps;
                float d = y - t;
                lsum += d * d / den;
                dz[o] = (2.0f * d / den) * e * (z < 20.0f ? 1.0f : 0.0f) / (float)(P * 3);
            }
        }
        if (dIn.p)
        {
            for (int c = 0; c < HEAD_C; ++c)
            {
                float g = dz[0] * sw[c] + dz[1] * sw[HEAD_C + c] + dz[2] * sw[2 * HEAD_C + c];
                if (!(xv[c] > 0.0f)) g = 0.0f; // ReLU of the features
                dIn.p[q * dIn.stride + dIn.off + c] = __float2bfloat16_rn(g);
            }
            for (int o = 0; o < 3; ++o)
            {
                for (int c = 0; c < HEAD_C; ++c) gw[o * HEAD_C + c] += dz[o] * xv[c];
                gw[3 * HEAD_C + o] += dz[o];
            }
        }
    }
    red[threadIdx.x] = lsum;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1)
    {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0 && lossPartial) lossPartial[blockIdx.x] = red[0];
    if (dIn.p)
    {
        // fixed-order block reduction of the weight gradients
        for (int i = 0; i < 3 * HEAD_C + 3; ++i)
        {
            __syncthreads();
            red[threadIdx.x] = gw[i];
            __syncthreads();
            for (int o = blockDim.x / 2; o > 0; o >>= 1)
            {
                if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
                __syncthreads();
            }
            if (threadIdx.x == 0) gwPartial[(long)blockIdx.x * (3 * HEAD_C + 3) + i] = red[0];
        }
    }
}

// ------------------------------------------------------------------ optimiser and input packing
// Adam (Kingma and Ba, 2015) on FP32 master weights; writes the BF16 copy the convolutions read
__global__ void adamKernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                           bf16* __restrict__ pb, long n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    {
        float gi = g[i];
        float mi = b1 * m[i] + (1.0f - b1) * gi;
        float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        if (pb) pb[i] = __float2bfloat16_rn(pi);
    }
}

// network input (16 channels, BF16) from the film mean XYZ and the feature means:
// log1p(linear sRGB radiance) 3, albedo 3, normal 3, depth / depthScale 1, zeros 6
__global__ void packInput(const float* __restrict__ xyz, const float* __restrict__ albedo, const float* __restrict__ normal,
                          const float* __restrict__ depth, float depthScale, long P, Act out)
{
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < P; q += (long)gridDim.x * blockDim.x)
    {
        float X = xyz[3 * q], Y = xyz[3 * q + 1], Z = xyz[3 * q + 2];
        // c_srgbXYZToRGB (colorSpaces.hlsl:18-23)
        float r = 3.2406f * X - 1.5372f * Y - 0.4986f * Z;
        float gg = -0.9689f * X + 1.8758f * Y + 0.0415f * Z;
        float bb = 0.0557f * X - 0.2040f * Y + 1.0570f * Z;
        float v[16] = {log1pf(fmaxf(r, 0.0f)), log1pf(fmaxf(gg, 0.0f)), log1pf(fmaxf(bb, 0.0f)),
                       albedo[3 * q], albedo[3 * q + 1], albedo[3 * q + 2],
                       normal[3 * q], normal[3 * q + 1], normal[3 * q + 2],
                       depth[q] / depthScale, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int c = 0; c < 16; ++c) out.p[q * out.stride + out.off + c] = __float2bfloat16_rn(v[c]);
    }
}

// per-tile error estimate of a denoised image from the denoised images a and b of two
// independent half renders: mean over the tile's pixels and channels of
// ((a - b)^2 / 4) / (out^2 + eps), one block per tile (FP64 sums); flags tiles above threshold
__global__ void tileError(const float* __restrict__ a, const float* __restrict__ b, const float* __restrict__ out, int H, int W,
                          int tile, float eps, float threshold, float* __restrict__ err, uint32_t* __restrict__ flags)
{
    const int tx = (W + tile - 1) / tile;
    const int t = blockIdx.x;
    const int y0 = (t / tx) * tile, x0 = (t % tx) * tile;
    const int th = min(tile, H - y0), tw = min(tile, W - x0);
    double acc = 0.0;
    for (int k = threadIdx.x; k < th * tw; k += blockDim.x)
    {
        const long q = (long)(y0 + k / tw) * W + (x0 + k % tw);
        for (int c = 0; c < 3; ++c)
        {
            const float d = a[3 * q + c] - b[3 * q + c], o = out[3 * q + c];
            acc += (double)(d * d * 0.25f) / (double)(o * o + eps);
        }
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        const float e = (float)(red[0] / (3.0 * th * tw));
        err[t] = e;
        flags[t] = e > threshold ? 1u : 0u;
    }
}

// flagged tiles of out replaced by the linear sRGB of a film mean (XYZ)
__global__ void tileFallback(float* __restrict__ out, const float* __restrict__ xyz, const uint32_t* __restrict__ flags, int H,
                             int W, int tile)
{
    const int tx = (W + tile - 1) / tile;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < (long)H * W; q += (long)gridDim.x * blockDim.x)
    {
        const int y = (int)(q / W), x = (int)(q % W);
        if (!flags[(y / tile) * tx + x / tile]) continue;
        const float X = xyz[3 * q], Y = xyz[3 * q + 1], Z = xyz[3 * q + 2];
        // c_srgbXYZToRGB (colorSpaces.hlsl:18-23)
        out[3 * q] = 3.2406f * X - 1.5372f * Y - 0.4986f * Z;
        out[3 * q + 1] = -0.9689f * X + 1.8758f * Y + 0.0415f * Z;
        out[3 * q + 2] = 0.0557f * X - 0.2040f * Y + 1.0570f * Z;
    }
}

int gridFor(long n, int threads = 256)
{
    long b = (n + threads - 1) / threads;
    return (int)std::max<long>(1, std::min<long>(b, 152L * 16));
}
} // namespace ygnn

using namespace ygnn;

namespace
{
Act act(const yg_nn_tensor* t)
{
    Act a;
    a.p = t ? reinterpret_cast<bf16*>(t->data) : nullptr;
    a.stride = t ? t->stride : 0;
    a.off = t ? t->offset : 0;
    a.ch = t ? t->channels : 0;
    return a;
}
int g_convImpl = YG_NN_CONV_TCGEN05_TMA;

bool okTensor(const yg_nn_tensor* t)
{
    return t && t->data && t->channels % 16 == 0 && t->stride % 8 == 0 && t->offset % 8 == 0 &&
           t->offset + t->channels <= t->stride && ((uintptr_t)t->data & 15u) == 0;
}
int status(cudaStream_t s)
{
    (void)s;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? YG_OK : YG_ERR_CUDA;
}
} // namespace

extern "C" {

YG_API int yg_nn_set_conv_impl(int impl)
{
    if (impl != YG_NN_CONV_MMA_SYNC && impl != YG_NN_CONV_TCGEN05 && impl != YG_NN_CONV_TCGEN05_TMA) return YG_ERR_INVALID_ARGUMENT;
    g_convImpl = impl;
    return YG_OK;
}

YG_API int yg_nn_tc_timeouts(uint32_t* count)
{
    if (!count) return YG_ERR_INVALID_ARGUMENT;
    return cudaMemcpyFromSymbol(count, tc::g_timeouts, sizeof(uint32_t)) == cudaSuccess ? YG_OK : YG_ERR_CUDA;
}

YG_API int yg_nn_conv3x3(const yg_nn_tensor* x, const void* weights, const float* bias, const yg_nn_tensor* y,
                         const yg_nn_tensor* mask, int relu, int accumulate, int n, int h, int w, void* stream)
{
    if (!okTensor(x) || !okTensor(y) || !weights || n <= 0 || h <= 0 || w <= 0) return YG_ERR_INVALID_ARGUMENT;
    if (mask && mask->data && (mask->channels != y->channels || !okTensor(mask))) return YG_ERR_INVALID_ARGUMENT;
    if (y->channels % 32 != 0 || ((uintptr_t)weights & 15u)) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    long P = (long)n * h * w;
    dim3 grid((unsigned)((P + CM - 1) / CM), (unsigned)((y->channels + CN - 1) / CN));
    Act m = act(mask && mask->data ? mask : nullptr);
    if (g_convImpl == YG_NN_CONV_TCGEN05_TMA)
    {
        int r = 1;
        if (h * w >= (1 << 16))
        {
            int dev = 0, sms = 152;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            r = tc::launchPersistAny(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, sms, st);
        }
        if (r == YG_OK) return status(st);
        if (r != 1) return r;
        if (x->channels % 64 == 0) r = tc::launchTmaN<64>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, st);
        else if (x->channels % 32 == 0) r = tc::launchTmaN<32>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, st);
        else r = tc::launchTmaN<16>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, st);
        return r != YG_OK ? r : status(st);
    }
    if (g_convImpl == YG_NN_CONV_TCGEN05)
    {
        int r;
        if (x->channels % 64 == 0) r = tc::launchTcN<64>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, st);
        else if (x->channels % 32 == 0) r = tc::launchTcN<32>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, st);
        else r = tc::launchTcN<16>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w, st);
        return r != YG_OK ? r : status(st);
    }
    if (x->channels % 32 == 0)
        conv3x3Kernel<32><<<grid, 256, 0, st>>>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w);
    else
        conv3x3Kernel<16><<<grid, 256, 0, st>>>(act(x), (const bf16*)weights, bias, act(y), m, relu, accumulate, n, h, w);
    return status(st);
}

YG_API size_t yg_nn_wgrad_workspace(int cin, int cout, int n, int h, int w)
{
    long P = (long)n * h * w;
    int splits = (int)std::min<long>(64, std::max<long>(1, P / 4096));
    return (size_t)splits * cout * 9 * cin * sizeof(float);
}

YG_API int yg_nn_conv3x3_wgrad(const yg_nn_tensor* x, const yg_nn_tensor* dy, float* dw, float* db, void* workspace,
                               int n, int h, int w, void* stream)
{
    if (!okTensor(x) || !okTensor(dy) || !dw || !workspace || dy->channels % 32 != 0) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    long P = (long)n * h * w;
    int splits = (int)std::min<long>(64, std::max<long>(1, P / 4096));
    long per = (P + splits - 1) / splits;
    per = (per + WK - 1) / WK * WK;
    splits = (int)((P + per - 1) / per);
    const int cin = (int)x->channels, cout = (int)dy->channels;
    dim3 grid((unsigned)((cout + WM - 1) / WM), (unsigned)(9 * ((cin + WN - 1) / WN)), (unsigned)splits);
    float* part = static_cast<float*>(workspace);
    conv3x3WgradKernel<<<grid, 256, 0, st>>>(act(x), act(dy), part, n, h, w, per);
    long nw = (long)cout * 9 * cin;
    reduceSplits<<<gridFor(nw), 256, 0, st>>>(part, splits, nw, dw);
    if (db) biasGrad<<<cout, 256, 0, st>>>(act(dy), P, db);
    return status(st);
}

YG_API int yg_nn_sum_rows(const float* in, int rows, long n, float* out, void* stream)
{
    if (!in || !out || rows <= 0 || n <= 0) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    reduceSplits<<<gridFor(n), 256, 0, st>>>(in, rows, n, out);
    return status(st);
}

YG_API int yg_nn_flip_weights(const void* w, int cout, int cin, void* wt, void* stream)
{
    if (!w || !wt) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    flipWeights<<<gridFor((long)cout * 9 * cin), 256, 0, st>>>((const bf16*)w, cout, cin, (bf16*)wt);
    return status(st);
}

YG_API int yg_nn_avgpool(const yg_nn_tensor* in, const yg_nn_tensor* out, int n, int h, int w, void* stream)
{
    if (!okTensor(in) || !okTensor(out) || in->channels != out->channels || (h | w) & 1) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    avgPool<<<gridFor((long)n * (h / 2) * (w / 2) * in->channels), 256, 0, st>>>(act(in), act(out), n, h, w);
    return status(st);
}

YG_API int yg_nn_avgpool_bwd(const yg_nn_tensor* dout, const yg_nn_tensor* add, const yg_nn_tensor* mask,
                             const yg_nn_tensor* din, int n, int h, int w, void* stream)
{
    if (!okTensor(dout) || !okTensor(din) || (h | w) & 1) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    avgPoolBwd<<<gridFor((long)n * h * w * din->channels), 256, 0, st>>>(act(dout), act(add && add->data ? add : nullptr),
                                                                          act(mask && mask->data ? mask : nullptr), act(din),
                                                                          n, h, w);
    return status(st);
}

YG_API int yg_nn_upsample(const yg_nn_tensor* in, const yg_nn_tensor* out, int n, int h, int w, void* stream)
{
    if (!okTensor(in) || !okTensor(out) || in->channels != out->channels) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    upsample<<<gridFor((long)n * 4 * h * w * in->channels), 256, 0, st>>>(act(in), act(out), n, h, w);
    return status(st);
}

YG_API int yg_nn_upsample_bwd(const yg_nn_tensor* dout, const yg_nn_tensor* mask, const yg_nn_tensor* din, int n, int h,
                              int w, void* stream)
{
    if (!okTensor(dout) || !okTensor(din)) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    upsampleBwd<<<gridFor((long)n * h * w * din->channels), 256, 0, st>>>(act(dout), act(mask && mask->data ? mask : nullptr),
                                                                         act(din), n, h, w);
    return status(st);
}

YG_API int yg_nn_head(const yg_nn_tensor* in, const yg_nn_tensor* skip, const float* w, const float* b, long pixels, float* out,
                      const float* target, float eps, float* loss_partial, const yg_nn_tensor* din, float* gw_partial, int blocks,
                      void* stream)
{
    if (!okTensor(in) || in->channels != HEAD_C || !w || !b || blocks <= 0) return YG_ERR_INVALID_ARGUMENT;
    if (skip && skip->data && !okTensor(skip)) return YG_ERR_INVALID_ARGUMENT;
    if (din && din->data && (!gw_partial || !target)) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    headKernel<<<blocks, 256, 0, st>>>(act(in), act(skip && skip->data ? skip : nullptr), w, b, pixels, out, target, eps,
                                       loss_partial,
                                       act(din && din->data ? din : nullptr), gw_partial);
    return status(st);
}

YG_API int yg_nn_adam(float* params, const float* grads, float* m, float* v, void* params_bf16, long n, float lr, float beta1,
                      float beta2, float eps, int step, void* stream)
{
    if (!params || !grads || !m || !v || n <= 0 || step <= 0) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    adamKernel<<<gridFor(n), 256, 0, st>>>(params, grads, m, v, (bf16*)params_bf16, n, lr, beta1, beta2, eps, c1, c2);
    return status(st);
}

YG_API int yg_nn_tile_error(const float* a, const float* b, const float* out, int height, int width, int tile, float eps,
                            float threshold, float* tile_err, uint32_t* tile_flags, void* stream)
{
    if (!a || !b || !out || !tile_err || !tile_flags || height <= 0 || width <= 0 || tile <= 0) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const int tiles = ((height + tile - 1) / tile) * ((width + tile - 1) / tile);
    tileError<<<tiles, 256, 0, st>>>(a, b, out, height, width, tile, eps, threshold, tile_err, tile_flags);
    return status(st);
}

YG_API int yg_nn_tile_fallback(float* out, const float* film_xyz, const uint32_t* tile_flags, int height, int width, int tile,
                               void* stream)
{
    if (!out || !film_xyz || !tile_flags || height <= 0 || width <= 0 || tile <= 0) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    tileFallback<<<gridFor((long)height * width), 256, 0, st>>>(out, film_xyz, tile_flags, height, width, tile);
    return status(st);
}

YG_API int yg_nn_pack_input(const float* xyz, const float* albedo, const float* normal, const float* depth, float depth_scale,
                            long pixels, const yg_nn_tensor* out, void* stream)
{
    if (!xyz || !albedo || !normal || !depth || !okTensor(out) || out->channels != 16) return YG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    packInput<<<gridFor(pixels), 256, 0, st>>>(xyz, albedo, normal, depth, depth_scale, pixels, act(out));
    return status(st);
}

} // extern "C"
