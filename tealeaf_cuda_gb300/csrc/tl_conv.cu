// tl_conv.cu -- BF16 tensor-core kernels of the learned warm start: a
// residual network of 3x3 convolutions (32 channels, GELU) that predicts
// u^{n+1} - u^n from (u^n, log density, Kx, Ky, dt).  No reference
// counterpart: the reference solve always starts from u^n.
//
// Activations are NHWC BF16 with a one-pixel zero halo: [B][H+2][W+2][C].
// A 3x3 convolution is an implicit GEMM: M = pixels, N = output channels,
// K = 9 taps x input channels.  A warp owns 16 consecutive pixels of one
// row and all output channels; each (tap, 16-channel) step feeds
// mma.sync.m16n8k16 (BF16 inputs, FP32 accumulate) with A fragments loaded
// straight from the NHWC input (two channels per 32-bit load) and B
// fragments from weights stored [tap][cout][cin].  The data gradient is the
// same kernel on the output gradient with the weights flipped and
// transposed ([8 - tap][cin][cout]); the weight gradient is a GEMM over
// pixels (M = cout, N = cin per tap, K = pixels) whose per-CTA partial sums
// are reduced in a fixed order.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "tl_internal.cuh"

namespace tl {
namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const bf16 *p) {
    return *reinterpret_cast<const uint32_t *>(p);
}

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
constexpr float kG0 = 0.7978845608028654f, kG1 = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    const float u = kG0 * (x + kG1 * x * x * x);
    return 0.5f * x * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float u = kG0 * (x + kG1 * x * x * x);
    const float th = tanhf(u);
    const float du = kG0 * (1.f + 3.f * kG1 * x * x);
    return 0.5f * (1.f + th) + 0.5f * x * (1.f - th * th) * du;
}

enum ConvMode { kModeGelu = 0, kModeGeluRes = 1, kModeHead = 2, kModeLinear = 3 };

template <int CIN, int COUTP, int MODE>
__global__ void __launch_bounds__(128) k_conv(const bf16 *__restrict__ in, const bf16 *__restrict__ wt,
                                              const float *__restrict__ bias,
                                              const bf16 *__restrict__ res, bf16 *__restrict__ out,
                                              bf16 *__restrict__ pre, float *__restrict__ outf, int B,
                                              int H, int W) {
    const int lane = threadIdx.x & 31;
    const long long task = (long long)blockIdx.x * 4 + (threadIdx.x >> 5);
    const int wx = W / 16;
    if (task >= (long long)B * H * wx) return;
    const int b = (int)(task / ((long long)H * wx));
    const int rem = (int)(task % ((long long)H * wx));
    const int y = rem / wx, x0 = (rem % wx) * 16;
    const int g = lane >> 2, t = lane & 3;
    constexpr int NT = COUTP / 8;
    float acc[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    const long long Wp = W + 2;
    const bf16 *img = in + (long long)b * (H + 2) * Wp * CIN;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
        const bf16 *r0 = img + ((long long)(y + dy) * Wp + (x0 + dx + g)) * CIN;
        const bf16 *r1 = r0 + 8 * CIN;
#pragma unroll
        for (int kc = 0; kc < CIN / 16; ++kc) {
            const int ch = kc * 16 + 2 * t;
            const uint32_t a0 = ld32(r0 + ch), a1 = ld32(r1 + ch);
            const uint32_t a2 = ld32(r0 + ch + 8), a3 = ld32(r1 + ch + 8);
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
                const bf16 *wr = wt + (long long)(tap * COUTP + nt * 8 + g) * CIN + ch;
                mma16816(acc[nt], a0, a1, a2, a3, ld32(wr), ld32(wr + 8));
            }
        }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int co = nt * 8 + 2 * t;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int px = x0 + g + 8 * half;
            float v0 = acc[nt][2 * half], v1 = acc[nt][2 * half + 1];
            const long long o = ((long long)b * (H + 2) + y + 1) * Wp + px + 1;
            if (MODE == kModeHead) {
                if (co == 0) outf[((long long)b * H + y) * W + px] = v0 + bias[0];
                continue;
            }
            if (MODE == kModeGelu || MODE == kModeGeluRes) {
                v0 += bias[co];
                v1 += bias[co + 1];
                *reinterpret_cast<uint32_t *>(pre + o * COUTP + co) =
                    pack2(__float2bfloat16(v0), __float2bfloat16(v1));
                v0 = gelu(v0);
                v1 = gelu(v1);
            }
            if ((MODE == kModeGeluRes || MODE == kModeLinear) && res) {
                const __nv_bfloat162 rv = *reinterpret_cast<const __nv_bfloat162 *>(res + o * COUTP + co);
                v0 += __bfloat162float(rv.x);
                v1 += __bfloat162float(rv.y);
            }
            *reinterpret_cast<uint32_t *>(out + o * COUTP + co) =
                pack2(__float2bfloat16(v0), __float2bfloat16(v1));
        }
    }
}

// ---------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05): a CTA
// of 4 warps computes a tile of 128 pixels of one row (M = 128) for all
// COUTP output channels (N), accumulating in tensor memory.
//
// Shared memory holds, per kernel row dy, the 130 input pixels the tile's
// three taps dx = 0, 1, 2 read, in the K-major no-swizzle layout of the MMA
// operands: 16-byte core-matrix rows (one pixel, 8 channels), the pixels of
// an 8-channel chunk contiguous (16 bytes apart) and the chunks kChunkA bytes
// apart.  The A operand of tap (dy, dx) and 16-channel step kk is that block
// shifted by dx pixels: start + dx * 16, core matrices 128 bytes apart along
// M (SBO) and kChunkA along K (LBO).  The weights [tap][cout][cin] sit in the
// same layout (cout rows 16 bytes apart, chunks 16 * COUTP apart).  One
// thread issues the 9 * CIN / 16 MMAs (M 128, N COUTP, K 16, BF16 in, FP32
// accumulate) and commits them to an mbarrier; each warp then reads its 32
// TMEM lanes (one pixel a lane, one channel a column) and runs the epilogue
// of k_conv.
constexpr int kTcPix = 128;               // pixels of a tile (MMA M)
constexpr int kTcRow = kTcPix + 2;        // input pixels a kernel row reads
constexpr int kChunkA = kTcRow * 16;      // bytes between 8-channel chunks of A
constexpr int kTmemCols = 32;             // accumulator columns allocated (>= COUTP)
constexpr long long kTcWaitCycles = 2000000000LL;  // ~1 s: the MMA wait gives up after this

// set by a tcgen05 conv whose MMA completion wait ran out (read and cleared
// by tl_nn_conv_status)
__device__ int g_conv_tc_error;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: no swizzle, version 1 (bits 46-47)
__device__ __forceinline__ uint64_t mma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait on phase `parity` of an mbarrier: false if it ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kTcWaitCycles) return false;
    return true;
}

template <int N>
__device__ __forceinline__ void tmem_load(uint32_t taddr, float (&v)[N]);

template <>
__device__ __forceinline__ void tmem_load<32>(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

template <>
__device__ __forceinline__ void tmem_load<16>(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

template <int CIN, int COUTP, int MODE>
__global__ void __launch_bounds__(128) k_conv_tc(const bf16 *__restrict__ in, const bf16 *__restrict__ wt,
                                                 const float *__restrict__ bias,
                                                 const bf16 *__restrict__ res, bf16 *__restrict__ out,
                                                 bf16 *__restrict__ pre, float *__restrict__ outf, int B,
                                                 int H, int W) {
    static_assert(CIN % 16 == 0 && COUTP % 16 == 0 && COUTP <= kTmemCols, "conv shape");
    constexpr int CA = CIN / 8;                    // 8-channel chunks of a pixel
    constexpr int CHUNK_B = COUTP * 16;            // bytes between chunks of the weights
    constexpr int A_BYTES = 3 * CA * kChunkA;      // three kernel rows
    constexpr int B_BYTES = 9 * CA * CHUNK_B;      // nine taps
    __shared__ __align__(1024) unsigned char sa[A_BYTES];
    __shared__ __align__(1024) unsigned char sb[B_BYTES];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (W + kTcPix - 1) / kTcPix;
    const long long task = blockIdx.x;  // (b, y, tile)
    const int b = (int)(task / ((long long)H * tiles_x));
    const int rem = (int)(task % ((long long)H * tiles_x));
    const int y = rem / tiles_x, x0 = (rem % tiles_x) * kTcPix;
    const long long Wp = W + 2;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(&tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar)));
        // the tensor cores arrive on it: make the initialisation visible to them
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // A: padded input rows y + dy, pixels x0 .. x0 + 129, 16 bytes a load;
    // pixels past the padded row read as zero (partial last tile)
    const bf16 *img = in + (long long)b * (H + 2) * Wp * CIN;
    for (int k = tid; k < 3 * kTcRow * CA; k += 128) {
        const int c = k % CA, j = (k / CA) % kTcRow, dy = k / (CA * kTcRow);
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (x0 + j < Wp) v = *reinterpret_cast<const uint4 *>(img + ((long long)(y + dy) * Wp + x0 + j) * CIN + 8 * c);
        *reinterpret_cast<uint4 *>(sa + (dy * CA + c) * kChunkA + j * 16) = v;
    }
    // B: weights [tap][cout][cin]
    for (int k = tid; k < 9 * COUTP * CA; k += 128) {
        const int c = k % CA, co = (k / CA) % COUTP, tap = k / (CA * COUTP);
        const uint4 v = *reinterpret_cast<const uint4 *>(wt + ((long long)tap * COUTP + co) * CIN + 8 * c);
        *reinterpret_cast<uint4 *>(sb + (tap * CA + c) * CHUNK_B + co * 16) = v;
    }
    // the MMAs read shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t bar = smem_addr(&mbar);
    if (tid == 0) {
        constexpr uint32_t idesc = mma_idesc(kTcPix, COUTP);
        const uint32_t a0 = smem_addr(sa), b0 = smem_addr(sb);
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3, dx = tap % 3;
#pragma unroll
            for (int kk = 0; kk < CIN / 16; ++kk) {
                const uint64_t ad = mma_desc(a0 + (dy * CA + 2 * kk) * kChunkA + dx * 16, kChunkA, 128);
                const uint64_t bd = mma_desc(b0 + (tap * CA + 2 * kk) * CHUNK_B, CHUNK_B, 128);
                const uint32_t acc = (tap | kk) != 0 ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                     : "memory");
    }
    // warp-uniform outcome: tcgen05.ld below is executed by whole warps
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(bar, 0));
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) {
        // the accumulator never became ready: flag it, wait once more
        // (bounded) for the MMAs in flight, release the columns and leave
        if (lane == 0) atomicExch(&g_conv_tc_error, 1);
        mbar_wait_bounded(bar, 0);
    } else {
        // warp w holds TMEM lanes 32w..32w+31: pixel m = 32 w + lane
        float acc[COUTP];
        tmem_load<COUTP>(tmem + ((uint32_t)(32 * warp) << 16), acc);
        const int px = x0 + 32 * warp + lane;
        if (px < W) {
            const long long o = ((long long)b * (H + 2) + y + 1) * Wp + px + 1;
            if (MODE == kModeHead) {
                outf[((long long)b * H + y) * W + px] = acc[0] + bias[0];
            } else {
#pragma unroll
                for (int q = 0; q < COUTP / 8; ++q) {
                    float v[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) v[e] = acc[8 * q + e];
                    if (MODE == kModeGelu || MODE == kModeGeluRes) {
                        uint32_t pk[4];
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[e] += bias[8 * q + e];
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            pk[e] = pack2(__float2bfloat16(v[2 * e]), __float2bfloat16(v[2 * e + 1]));
                        *reinterpret_cast<uint4 *>(pre + o * COUTP + 8 * q) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[e] = gelu(v[e]);
                    }
                    if ((MODE == kModeGeluRes || MODE == kModeLinear) && res) {
                        const uint4 rv = *reinterpret_cast<const uint4 *>(res + o * COUTP + 8 * q);
                        const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            v[2 * e] += __bfloat162float(__ushort_as_bfloat16((unsigned short)(rw[e] & 0xFFFFu)));
                            v[2 * e + 1] += __bfloat162float(__ushort_as_bfloat16((unsigned short)(rw[e] >> 16)));
                        }
                    }
                    uint32_t pk[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) pk[e] = pack2(__float2bfloat16(v[2 * e]), __float2bfloat16(v[2 * e + 1]));
                    *reinterpret_cast<uint4 *>(out + o * COUTP + 8 * q) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// dpre = dh * gelu'(pre) over the interior (halo left at zero)
__global__ void k_gelu_back(const bf16 *__restrict__ dh, const bf16 *__restrict__ pre,
                            bf16 *__restrict__ dpre, int C, int B, int H, int W) {
    const long long n = (long long)B * H * W * C;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(k % C);
        const long long px = k / C;
        const int x = (int)(px % W), y = (int)((px / W) % H), b = (int)(px / ((long long)W * H));
        const long long o = (((long long)b * (H + 2) + y + 1) * (W + 2) + x + 1) * C + c;
        dpre[o] = __float2bfloat16(__bfloat162float(dh[o]) * gelu_grad(__bfloat162float(pre[o])));
    }
}

// Weight gradient: warp `tap` of each CTA accumulates
//   dW[tap][co][ci] += sum_p dpre[p][co] * in[p + off(tap)][ci]
// over the CTA's run of 16-pixel groups with mma (M = co, N = ci, K = pixels);
// the CTA writes its partial [9][COUTP][CIN].
template <int CIN, int COUTP>
__global__ void __launch_bounds__(288) k_wgrad(const bf16 *__restrict__ dpre,
                                               const bf16 *__restrict__ in,
                                               float *__restrict__ partial, int B, int H, int W,
                                               int groups_per_cta) {
    const int lane = threadIdx.x & 31, tap = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int dy = tap / 3, dx = tap % 3;
    constexpr int MT = COUTP / 16, NT = CIN / 8;
    float acc[MT][NT][4];
#pragma unroll
    for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
    const int wx = W / 16;
    const long long ngroups = (long long)B * H * wx;
    const long long Wp = W + 2;
    const long long g0 = (long long)blockIdx.x * groups_per_cta;
    for (long long q = g0; q < g0 + groups_per_cta && q < ngroups; ++q) {
        const int b = (int)(q / ((long long)H * wx));
        const int rem = (int)(q % ((long long)H * wx));
        const int y = rem / wx, x0 = (rem % wx) * 16;
        // dpre at interior pixels (y, x0 + k): padded (y + 1, x0 + k + 1)
        const bf16 *dp = dpre + (((long long)b * (H + 2) + y + 1) * Wp + x0 + 1) * COUTP;
        // in at padded (y + dy, x0 + k + dx)
        const bf16 *ip = in + (((long long)b * (H + 2) + y + dy) * Wp + x0 + dx) * CIN;
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
            const int co = mt * 16 + g;
            const uint32_t a0 = pack2(dp[(2 * t) * COUTP + co], dp[(2 * t + 1) * COUTP + co]);
            const uint32_t a1 = pack2(dp[(2 * t) * COUTP + co + 8], dp[(2 * t + 1) * COUTP + co + 8]);
            const uint32_t a2 = pack2(dp[(2 * t + 8) * COUTP + co], dp[(2 * t + 9) * COUTP + co]);
            const uint32_t a3 = pack2(dp[(2 * t + 8) * COUTP + co + 8], dp[(2 * t + 9) * COUTP + co + 8]);
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
                const int ci = nt * 8 + g;
                const uint32_t b0 = pack2(ip[(2 * t) * CIN + ci], ip[(2 * t + 1) * CIN + ci]);
                const uint32_t b1 = pack2(ip[(2 * t + 8) * CIN + ci], ip[(2 * t + 9) * CIN + ci]);
                mma16816(acc[mt][nt], a0, a1, a2, a3, b0, b1);
            }
        }
    }
    float *pp = partial + ((long long)blockIdx.x * 9 + tap) * COUTP * CIN;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int co = mt * 16 + g, ci = nt * 8 + 2 * t;
            pp[co * CIN + ci] = acc[mt][nt][0];
            pp[co * CIN + ci + 1] = acc[mt][nt][1];
            pp[(co + 8) * CIN + ci] = acc[mt][nt][2];
            pp[(co + 8) * CIN + ci + 1] = acc[mt][nt][3];
        }
}

// dW = sum over CTAs of the partials, in CTA order
__global__ void k_wreduce(const float *__restrict__ partial, float *__restrict__ dw, int n, int nparts) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += partial[(long long)p * n + k];
    dw[k] = s;
}

// db[c] = sum over interior pixels of dpre[p][c]; one CTA per channel
__global__ void k_dbias(const bf16 *__restrict__ dpre, float *__restrict__ db, int C, int B, int H, int W) {
    const int c = blockIdx.x;
    const long long n = (long long)B * H * W;
    float s = 0.f;
    for (long long p = threadIdx.x; p < n; p += blockDim.x) {
        const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((long long)W * H));
        s += __bfloat162float(dpre[(((long long)b * (H + 2) + y + 1) * (W + 2) + x + 1) * C + c]);
    }
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = sh[0];
}

// Adam on FP32 master parameters
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float g = gr[k];
    const float mk = b1 * m[k] + (1.f - b1) * g;
    const float vk = b2 * v[k] + (1.f - b2) * g * g;
    m[k] = mk;
    v[k] = vk;
    p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

// FP32 [9][COUTP][CIN] -> BF16 forward layout (same) and the data-gradient
// layout [8 - tap][CIN][COUTP]
__global__ void k_pack(const float *__restrict__ w, bf16 *__restrict__ wf, bf16 *__restrict__ wb,
                       int cin, int coutp) {
    const int n = 9 * cin * coutp;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int ci = k % cin, co = (k / cin) % coutp, tap = k / (cin * coutp);
    const bf16 v = __float2bfloat16(w[k]);
    wf[k] = v;
    if (wb) wb[((8 - tap) * cin + ci) * coutp + co] = v;
}

// MSE over the central region of each [H][W] image (margin cells excluded);
// dy[b][y][x][0] = 2 (y - t) / count there and 0 elsewhere (channel stride C);
// per-CTA partial sums of the squared error
__global__ void k_loss(const float *__restrict__ yv, const float *__restrict__ tv, bf16 *__restrict__ dy,
                       float *__restrict__ partial, int C, int B, int H, int W, int margin, float inv_count) {
    const long long n = (long long)B * H * W;
    float s = 0.f;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(k % W), y = (int)((k / W) % H), b = (int)(k / ((long long)W * H));
        const bool in_region = x >= margin && x < W - margin && y >= margin && y < H - margin;
        const float e = in_region ? yv[k] - tv[k] : 0.f;
        s += e * e;
        dy[(((long long)b * (H + 2) + y + 1) * (W + 2) + x + 1) * C] = __float2bfloat16(2.f * e * inv_count);
    }
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// crops of a stored dataset into a training batch: fields [N][H][W][F]
// (F-1 features then the target), origins (n, y, x) per batch item; writes
// x [B][S+2][S+2][C] (halo and channels >= F-1 zero) and t [B][S][S]
__global__ void k_gather(const float *__restrict__ fields, const int *__restrict__ org, bf16 *__restrict__ x,
                         float *__restrict__ tgt, int F, int C, int Hs, int Ws, int B, int S) {
    const long long n = (long long)B * S * S;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int xx = (int)(k % S), yy = (int)((k / S) % S), b = (int)(k / ((long long)S * S));
        const int sn = org[3 * b], sy = org[3 * b + 1] + yy, sx = org[3 * b + 2] + xx;
        const float *src = fields + (((long long)sn * Hs + sy) * Ws + sx) * F;
        bf16 *dst = x + (((long long)b * (S + 2) + yy + 1) * (S + 2) + xx + 1) * C;
        for (int c = 0; c < C; ++c) dst[c] = __float2bfloat16(c < F - 1 ? src[c] : 0.f);
        tgt[k] = src[F - 1];
    }
}

// which kernel tl_nn_conv runs: the tcgen05 one (default) or mma.sync
bool g_conv_tcgen05 = true;

template <int CIN, int COUTP, int MODE>
int launch_conv(const void *in, const void *w, const float *bias, const void *res, void *out, void *pre,
                float *outf, int B, int H, int W, cudaStream_t s) {
    if (g_conv_tcgen05) {
        const long long tiles = (long long)B * H * ((W + kTcPix - 1) / kTcPix);
        k_conv_tc<CIN, COUTP, MODE><<<(unsigned)tiles, 128, 0, s>>>((const bf16 *)in, (const bf16 *)w, bias,
                                                                    (const bf16 *)res, (bf16 *)out, (bf16 *)pre,
                                                                    outf, B, H, W);
    } else {
        const long long tasks = (long long)B * H * (W / 16);
        const unsigned grid = (unsigned)((tasks + 3) / 4);
        k_conv<CIN, COUTP, MODE><<<grid, 128, 0, s>>>((const bf16 *)in, (const bf16 *)w, bias,
                                                      (const bf16 *)res, (bf16 *)out, (bf16 *)pre, outf, B,
                                                      H, W);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "conv launch");
}

}  // namespace
}  // namespace tl

using namespace tl;

extern "C" {

int tl_nn_conv(int mode, int cin, int coutp, const void *in, const void *w, const float *bias,
               const void *res, void *out, void *pre, float *outf, int B, int H, int W, void *stream) {
    if (W % 16 != 0 || B < 1 || H < 1) {
        set_error("tl_nn_conv: width must be a multiple of 16 (got %d)", W);
        return TL_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
#define TL_CONV_CASE(CI, CO, MD)                                                          \
    if (cin == CI && coutp == CO && mode == MD)                                           \
        return launch_conv<CI, CO, MD>(in, w, bias, res, out, pre, outf, B, H, W, s);
    TL_CONV_CASE(16, 32, kModeGelu)
    TL_CONV_CASE(32, 32, kModeGeluRes)
    TL_CONV_CASE(32, 32, kModeGelu)
    TL_CONV_CASE(32, 16, kModeHead)
    TL_CONV_CASE(32, 32, kModeLinear)
    TL_CONV_CASE(16, 32, kModeLinear)
#undef TL_CONV_CASE
    set_error("tl_nn_conv: unsupported shape cin=%d coutp=%d mode=%d", cin, coutp, mode);
    return TL_ERR_ARG;
}

int tl_nn_set_conv_kernel(int tcgen05) {
    g_conv_tcgen05 = tcgen05 != 0;
    return TL_OK;
}

int tl_nn_conv_status(void) {
    int flag = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&flag, g_conv_tc_error, sizeof flag);
    if (e != cudaSuccess) return cuda_fail(e, "tl_nn_conv_status");
    if (flag) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_conv_tc_error, &zero, sizeof zero);
        if (e != cudaSuccess) return cuda_fail(e, "tl_nn_conv_status");
        set_error("tcgen05 conv: the wait for the tensor-core result ran out");
        return TL_ERR_CUDA;
    }
    return TL_OK;
}

int tl_nn_gelu_backward(const void *dh, const void *pre, void *dpre, int C, int B, int H, int W, void *stream) {
    k_gelu_back<<<1216, 256, 0, (cudaStream_t)stream>>>((const bf16 *)dh, (const bf16 *)pre, (bf16 *)dpre, C, B, H, W);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "gelu backward launch");
}

long long tl_nn_wgrad_partial_floats(int cin, int coutp, int B, int H, int W, int groups_per_cta) {
    const long long groups = (long long)B * H * (W / 16);
    const long long ctas = (groups + groups_per_cta - 1) / groups_per_cta;
    return ctas * 9LL * cin * coutp;
}

int tl_nn_wgrad(const void *dpre, const void *in, int cin, int coutp, float *partial, float *dw, float *db,
                int B, int H, int W, int groups_per_cta, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (W % 16 != 0 || groups_per_cta < 1) {
        set_error("tl_nn_wgrad: bad shape");
        return TL_ERR_ARG;
    }
    const long long groups = (long long)B * H * (W / 16);
    const unsigned ctas = (unsigned)((groups + groups_per_cta - 1) / groups_per_cta);
    if (cin == 16 && coutp == 32)
        k_wgrad<16, 32><<<ctas, 288, 0, s>>>((const bf16 *)dpre, (const bf16 *)in, partial, B, H, W, groups_per_cta);
    else if (cin == 32 && coutp == 32)
        k_wgrad<32, 32><<<ctas, 288, 0, s>>>((const bf16 *)dpre, (const bf16 *)in, partial, B, H, W, groups_per_cta);
    else if (cin == 32 && coutp == 16)
        k_wgrad<32, 16><<<ctas, 288, 0, s>>>((const bf16 *)dpre, (const bf16 *)in, partial, B, H, W, groups_per_cta);
    else {
        set_error("tl_nn_wgrad: unsupported shape cin=%d coutp=%d", cin, coutp);
        return TL_ERR_ARG;
    }
    const int n = 9 * cin * coutp;
    k_wreduce<<<(n + 255) / 256, 256, 0, s>>>(partial, dw, n, (int)ctas);
    if (db) k_dbias<<<coutp, 256, 0, s>>>((const bf16 *)dpre, db, coutp, B, H, W);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "wgrad launch");
}

int tl_nn_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
               int step, void *stream) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "adam launch");
}

int tl_nn_pack(const float *w, void *wf, void *wb, int cin, int coutp, void *stream) {
    const int n = 9 * cin * coutp;
    k_pack<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(w, (bf16 *)wf, (bf16 *)wb, cin, coutp);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "pack launch");
}

int tl_nn_loss(const float *y, const float *t, void *dy, float *partial, int C, int B, int H, int W,
               int margin, void *stream) {
    const long long cnt = (long long)B * (H - 2 * margin) * (W - 2 * margin);
    if (cnt <= 0) {
        set_error("tl_nn_loss: margin too large");
        return TL_ERR_ARG;
    }
    k_loss<<<1216, 256, 0, (cudaStream_t)stream>>>(y, t, (bf16 *)dy, partial, C, B, H, W, margin,
                                                   (float)(1.0 / (double)cnt));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "loss launch");
}

int tl_nn_gather(const float *fields, const int *org, void *x, float *t, int F, int C, int Hs, int Ws, int B,
                 int S, void *stream) {
    k_gather<<<1216, 256, 0, (cudaStream_t)stream>>>(fields, org, (bf16 *)x, t, F, C, Hs, Ws, B, S);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "gather launch");
}

}  // extern "C"
