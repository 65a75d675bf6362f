// k_cnn.cu -- the learned stage: a 5-layer 3x3 BF16 CNN (4 -> 32 -> 32 -> 32 -> 32 -> 4
// channels, ReLU between layers) that reads the demosaiced linear RGB plus a per-pixel noise
// sigma map and predicts a per-pixel denoise strength (channel 0, a logit) and an RGB
// residual in units of that sigma (channels 1..3).  No counterpart in the reference: it is inserted after
// interpolateRedBlue (raw_converter.cpp:127 of the reference), where the residual is added
// before transformImage and the strength scales the level-0 denoise.
//
// Every layer is an implicit GEMM on the tensor cores: M = pixels (16 consecutive pixels of
// a row per MMA tile), N = output channels, K = 9 taps x input channels, BF16 operands from
// shared memory through ldmatrix, FP32 accumulation.  Activations are NHWC BF16; borders
// are zero-padded ('same' convolution).  Training runs on the same kernels: the input
// gradient is the forward convolution with the weights flipped and transposed (and the
// ReLU mask of the layer below applied in the epilogue); the weight gradient contracts
// over pixels (ldmatrix.trans turns both pixel-major tiles into MMA fragments), reduced
// over blocks in a fixed order; Adam updates FP32 master weights.
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "gls_internal.h"

namespace gls {
namespace {

constexpr int kLayers = 5;
// the noise sigma enters the network scaled to the range of the image values
constexpr float kSigmaScale = 64.0f;
constexpr int kCin[kLayers] = {4, 32, 32, 32, 32};     // real input channels
constexpr int kCout[kLayers] = {32, 32, 32, 32, 4};    // real output channels

// conv tile: 8 rows x 16 columns of output pixels, 4 warps (2 rows each)
constexpr int TR = 8, TC = 16, CT = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x2(uint32_t addr, uint32_t& r0, uint32_t& r1) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x2_t(uint32_t addr, uint32_t& r0, uint32_t& r1) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}

// D (16x8 f32) += A (16x16 bf16, row) * B (16x8 bf16, col)
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------------------------------
// Activation loader: a (TR + 2) x (TC + 2) halo tile of an NHWC tensor with `csrc` channels
// (bf16, or fp32 for the network input, whose sigma channel 3 is scaled by kSigmaScale) into
// shared memory with CIN channels per pixel
// (zero-filled beyond csrc and outside the image) and a pixel stride of CIN + 8 elements,
// which keeps ldmatrix rows on distinct banks.
// ---------------------------------------------------------------------------------------
template <int CIN, bool F32IN>
__device__ __forceinline__ void load_halo(__nv_bfloat16* s, const void* src, int csrc, int w, int h, int x0, int y0) {
    constexpr int PS = CIN + 8, HW = TC + 2, HH = TR + 2;
    for (int i = threadIdx.x; i < HH * HW * (CIN / 8); i += CT) {
        const int q = i % (CIN / 8), p = i / (CIN / 8);
        const int r = p / HW, c = p - r * HW;
        const int x = x0 - 1 + c, y = y0 - 1 + r;
        __nv_bfloat16 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = __float2bfloat16_rn(0.0f);
        if (x >= 0 && x < w && y >= 0 && y < h) {
            const size_t base = ((size_t)y * w + x) * csrc;
            if (F32IN) {
                const float* f = static_cast<const float*>(src) + base;
#pragma unroll
                for (int k = 0; k < 8; k++)
                    if (q * 8 + k < csrc) v[k] = __float2bfloat16_rn(q * 8 + k == 3 ? f[3] * kSigmaScale : f[q * 8 + k]);
            } else {
                const __nv_bfloat16* b = static_cast<const __nv_bfloat16*>(src) + base;
                if (csrc % 8 == 0 && q * 8 + 8 <= csrc) {
                    *reinterpret_cast<uint4*>(v) = *reinterpret_cast<const uint4*>(b + q * 8);
                } else {
#pragma unroll
                    for (int k = 0; k < 8; k++)
                        if (q * 8 + k < csrc) v[k] = b[q * 8 + k];
                }
            }
        }
        *reinterpret_cast<uint4*>(s + (size_t)p * PS + q * 8) = *reinterpret_cast<uint4*>(v);
    }
}

// Weights [NOUT][9 * CIN] (k = tap * CIN + ci) into shared memory, row stride 9 * CIN + 8.
template <int NOUT, int CIN>
__device__ __forceinline__ void load_weights(__nv_bfloat16* s, const __nv_bfloat16* wt) {
    constexpr int K = 9 * CIN, KS = K + 8;
    for (int i = threadIdx.x; i < NOUT * (K / 8); i += CT) {
        const int n = i / (K / 8), q = i - n * (K / 8);
        *reinterpret_cast<uint4*>(s + (size_t)n * KS + q * 8) = *reinterpret_cast<const uint4*>(wt + (size_t)n * K + q * 8);
    }
}

// ---------------------------------------------------------------------------------------
// Forward convolution (also the input-gradient convolution).
//   EPI 0: + bias, ReLU, bf16 out (cout channels)
//   EPI 1: + bias, fp32 out (the network head)
//   EPI 2: no bias, times (mask > 0) of a bf16 tensor with the output's channels, bf16 out
// ---------------------------------------------------------------------------------------
struct ConvArgs {
    const void* in;
    int cin_src;  // channels of `in`
    const __nv_bfloat16* wt;  // [NOUT][9][CIN]
    const float* bias;        // [cout]
    void* out;
    int cout;                 // channels of `out` (<= NOUT)
    const __nv_bfloat16* mask;  // EPI 2
    int w, h;
    size_t in_stride, out_stride, mask_stride;  // elements per image of the batch
};

template <int CIN, int NOUT, int EPI, bool F32IN>
__global__ void __launch_bounds__(CT) conv3x3_kernel(ConvArgs a) {
    constexpr int PS = CIN + 8, HW = TC + 2, HH = TR + 2;
    constexpr int K = 9 * CIN, KS = K + 8;
    constexpr int NT = NOUT / 8;  // n8 tiles
    __shared__ __align__(16) __nv_bfloat16 s_in[HH * HW * PS];
    __shared__ __align__(16) __nv_bfloat16 s_w[NOUT * KS];
    const int x0 = blockIdx.x * TC, y0 = blockIdx.y * TR, img = blockIdx.z;
    const void* in = F32IN ? (const void*)((const float*)a.in + img * a.in_stride)
                           : (const void*)((const __nv_bfloat16*)a.in + img * a.in_stride);
    load_halo<CIN, F32IN>(s_in, in, a.cin_src, a.w, a.h, x0, y0);
    load_weights<NOUT, CIN>(s_w, a.wt);
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][NT][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < NT; n++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[m][n][k] = 0.0f;

    // ldmatrix addressing: lane l supplies row (l & 15) of the A tile, column block l >> 4
    const int arow = lane & 15, acol = (lane >> 4) * 8;
    // B (x4 over two n8 tiles): lane l -> n row (l & 7) + 8 * (l >> 4), k block ((l >> 3) & 1) * 8
    const int brow = (lane & 7) + ((lane >> 4) << 3), bcol = ((lane >> 3) & 1) * 8;
#pragma unroll
    for (int tap = 0; tap < 9; tap++) {
        const int dy = tap / 3, dx = tap % 3;
#pragma unroll
        for (int cb = 0; cb < CIN / 16; cb++) {
            uint32_t af[2][4];
#pragma unroll
            for (int m = 0; m < 2; m++) {
                const int r = 2 * warp + m + dy, c = arow + dx;
                ldsm_x4(smem_u32(s_in + (r * HW + c) * PS + cb * 16 + acol), af[m][0], af[m][1], af[m][2], af[m][3]);
            }
            const int k0 = tap * CIN + cb * 16;
#pragma unroll
            for (int n = 0; n < NT; n += 2) {
                if (n + 1 < NT) {
                    uint32_t b0, b1, b2, b3;
                    ldsm_x4(smem_u32(s_w + (n * 8 + brow) * KS + k0 + bcol), b0, b1, b2, b3);
                    // b0/b1: tile n (k 0-7, 8-15); b2/b3: tile n + 1
#pragma unroll
                    for (int m = 0; m < 2; m++) {
                        mma_bf16(acc[m][n], af[m], b0, b1);
                        mma_bf16(acc[m][n + 1], af[m], b2, b3);
                    }
                } else {
                    uint32_t b0, b1;
                    ldsm_x2(smem_u32(s_w + (n * 8 + (lane & 7)) * KS + k0 + ((lane >> 3) & 1) * 8), b0, b1);
#pragma unroll
                    for (int m = 0; m < 2; m++) mma_bf16(acc[m][n], af[m], b0, b1);
                }
            }
        }
    }

    // epilogue: thread holds rows g, g + 8 (pixels) and columns 2t, 2t + 1 of each n8 tile
#pragma unroll
    for (int m = 0; m < 2; m++) {
        const int y = y0 + 2 * warp + m;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int x = x0 + g + 8 * half;
            if (x >= a.w || y >= a.h) continue;
            const size_t px = (size_t)y * a.w + x;
#pragma unroll
            for (int n = 0; n < NT; n++) {
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const int co = n * 8 + 2 * t + j;
                    if (co >= a.cout) continue;
                    float v = acc[m][n][2 * half + j];
                    if (EPI == 0) {
                        v = fmaxf(v + a.bias[co], 0.0f);
                        ((__nv_bfloat16*)a.out)[img * a.out_stride + px * a.cout + co] = __float2bfloat16_rn(v);
                    } else if (EPI == 1) {
                        ((float*)a.out)[img * a.out_stride + px * a.cout + co] = v + a.bias[co];
                    } else {
                        const float mk = __bfloat162float(a.mask[img * a.mask_stride + px * a.cout + co]);
                        ((__nv_bfloat16*)a.out)[img * a.out_stride + px * a.cout + co] =
                            __float2bfloat16_rn(mk > 0.0f ? v : 0.0f);
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// Forward convolution of a hidden layer (32 -> 32 channels, bias + ReLU, bf16 out) on the
// 5th-generation tensor cores: tcgen05.mma with the accumulator in tensor memory.
//
// One block computes a 16-row x 8-column output tile: M = 128 pixels, N = 32 channels,
// K = 9 taps x 32 channels = 18 MMAs of K = 16.  Shared memory holds the operands in the
// canonical K-major layout without swizzle, as 8-row x 16-byte core matrices:
//   halo   [channel block cb = 0..3][halo row 0..17][halo col 0..9][8 channels]
//   weights [tap 0..8][cb 0..3][output channel 0..31][8 channels]
// An 8-row group of the A operand is one tile row, so a tap (dy, dx) is a shifted start
// address with the same strides: SBO = one halo row (160 B), LBO = one channel block
// (2880 B).  For B, SBO = 8 output channels (128 B), LBO = one channel block (512 B).
// One thread issues the MMAs and commits them to an mbarrier; every thread waits on it
// (bounded: after kWaitLimit polls the block records an error, drains its copies and
// stops), then each warp reads its 32 lanes of the accumulator (tcgen05.ld 32x32b) for the
// epilogue.  Warp 0 allocates the 32 TMEM columns and frees them on every path.
// ---------------------------------------------------------------------------------------
constexpr int TC5_R = 16, TC5_C = 8;  // output tile rows x columns
constexpr int TC5_HR = TC5_R + 2, TC5_HC = TC5_C + 2;
constexpr uint32_t kWaitLimit = 1u << 24;
constexpr int kTc5Stack = 1;         // 16x8 tiles per persistent-block iteration
constexpr int kTc5BlocksPerSm = 5;   // resident blocks per SM (shared memory: 41 KB each; TMEM 64 columns each)

__device__ __forceinline__ int cdiv_d(int a, int b) { return (a + b - 1) / b; }

__device__ __forceinline__ uint64_t tc5_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1, no swizzle
}

// kind::f16, BF16 A and B (K-major), FP32 D, M = 128, N = 32
constexpr uint32_t kIdescBf16M128N32 = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t kIdescBf16M128N16 = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0) : "memory");
}

// Persistent: each block stages the weights once and walks tiles blockIdx.x, + gridDim.x,
// ...; the halo of the next tile streams in (cp.async, zero-filled outside the image) into
// the other of two buffers while the current tile's MMAs and epilogue run.
// MT stacked 16x8 tiles per iteration (MT * 128 threads, MT 32-column accumulators): more
// work per barrier and per wait; dynamic shared memory (two halo buffers + the weights).
// MODE 0: a hidden 32 -> 32 layer (bf16 in and out, bias + ReLU)
// MODE 1: the first layer: fp32 input (R, G, B, sigma scaled), one 8-channel plane per pixel
//         (4 channels + 4 zeros); its K = 16 reads the second core matrix 16 bytes on (the
//         next pixel, finite) against zero weights
// MODE 2: the head: 32 -> 4 channels (N = 16, weight rows 8..15 zero), fp32 out, bias only
template <int MT, int MODE>
struct Tc5 {
    static constexpr int R = 16 * MT, HR = R + 2, HC = TC5_C + 2;
    static constexpr int CB = MODE == 1 ? 1 : 4;    // 8-channel planes of the halo
    static constexpr int WCB = MODE == 1 ? 2 : 4;   // 8-channel blocks of the weights
    static constexpr int NB = MODE == 2 ? 16 : 32;  // MMA N
    static constexpr int KCS = MODE == 1 ? 1 : 2;   // K steps of 16 per tap
    static constexpr int HALO_N = CB * HR * HC, HALO_B = HALO_N * 16, W_B = 9 * WCB * NB * 16;
    static constexpr int THREADS = 128 * MT, COLS = 32 * MT;
    static constexpr int SMEM = 2 * HALO_B + W_B;
};

template <int MT, int MODE>
__global__ void __launch_bounds__(Tc5<MT, MODE>::THREADS) conv3x3_tc05_kernel(ConvArgs a, int nimg, int* err) {
    using K = Tc5<MT, MODE>;
    extern __shared__ __align__(128) unsigned char tc5_smem[];
    unsigned char* s_a0 = tc5_smem;
    unsigned char* s_b = tc5_smem + 2 * K::HALO_B;
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ uint32_t s_taddr;
    __shared__ float s_bias[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar0 = smem_u32(&s_bar[0]);
    const int tiles_x = cdiv_d(a.w, TC5_C), tiles_y = cdiv_d(a.h, K::R);
    if (threadIdx.x < 32) s_bias[threadIdx.x] = threadIdx.x < (MODE == 2 ? 4 : 32) ? a.bias[threadIdx.x] : 0.0f;
    if (MODE == 1) {  // everything the tensor cores may read stays finite
        for (int i = threadIdx.x; i < 2 * K::HALO_B / 16; i += K::THREADS)
            reinterpret_cast<uint4*>(tc5_smem)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();  // before the first halo lands in the same bytes
    }
    const int tiles_img = tiles_x * tiles_y, ntiles = tiles_img * nimg;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_taddr)),
                     "n"(2 * K::COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    // weights [tap][8-channel block][n][8] from the packed [nout_p][9][cin_p]
    for (int i = threadIdx.x; i < 9 * K::WCB * K::NB; i += K::THREADS) {
        const int tap = i / (K::WCB * K::NB), r = i - tap * K::WCB * K::NB, cb = r / K::NB, n = r - cb * K::NB;
        constexpr int CINP = MODE == 1 ? 16 : 32;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (MODE != 2 || n < 8)
            v = *reinterpret_cast<const uint4*>(a.wt + (size_t)n * 9 * CINP + tap * CINP + cb * 8);
        *reinterpret_cast<uint4*>(s_b + (size_t)i * 16) = v;
    }
    auto prefetch = [&](int t, int buf) {
        const int img = t / tiles_img, tt = t - img * tiles_img;
        const int x0 = (tt % tiles_x) * TC5_C, y0 = (tt / tiles_x) * K::R;
        if (MODE == 1) {  // fp32 network input: plain loads, converted to bf16
            const float* in = (const float*)a.in + img * a.in_stride;
            unsigned char* dst = s_a0 + buf * K::HALO_B;
            for (int p = threadIdx.x; p < K::HR * K::HC; p += K::THREADS) {
                const int r = p / K::HC, c = p - r * K::HC;
                const int x = x0 - 1 + c, y = y0 - 1 + r;
                __nv_bfloat16 v[8];
#pragma unroll
                for (int q = 0; q < 8; q++) v[q] = __float2bfloat16_rn(0.0f);
                if (x >= 0 && x < a.w && y >= 0 && y < a.h) {
                    const float4 f = __ldg(reinterpret_cast<const float4*>(in + ((size_t)y * a.w + x) * 4));
                    v[0] = __float2bfloat16_rn(f.x);
                    v[1] = __float2bfloat16_rn(f.y);
                    v[2] = __float2bfloat16_rn(f.z);
                    v[3] = __float2bfloat16_rn(f.w * kSigmaScale);
                }
                *reinterpret_cast<uint4*>(dst + (size_t)p * 16) = *reinterpret_cast<const uint4*>(v);
            }
            return;
        }
        const __nv_bfloat16* in = (const __nv_bfloat16*)a.in + img * a.in_stride;
        const uint32_t base = smem_u32(s_a0 + buf * K::HALO_B);
        for (int i = threadIdx.x; i < K::HALO_N; i += K::THREADS) {
            // consecutive threads take consecutive 16-byte pieces of a pixel's 64 bytes
            const int p = i >> 2, cb = i & 3;
            const int r = p / K::HC, c = p - r * K::HC;
            const int x = x0 - 1 + c, y = y0 - 1 + r;
            const bool ok = x >= 0 && x < a.w && y >= 0 && y < a.h;
            cp_async16(base + (uint32_t)(cb * K::HR * K::HC + p) * 16,
                       ok ? (const void*)(in + ((size_t)y * a.w + x) * 32 + cb * 8) : (const void*)in, ok);
        }
    };
    int t = blockIdx.x;
    if (t < ntiles) prefetch(t, 0);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = s_taddr;
    // bounded wait for MMA group `it` (barrier it & 1, its (it >> 1)-th completion)
    auto wait_mma = [&](int it) -> bool {
        uint32_t done = 0;
        const uint32_t b = bar0 + 8u * (uint32_t)(it & 1), parity = (uint32_t)((it >> 1) & 1);
        for (uint32_t k = 0; k < kWaitLimit && !done; k++) {
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(b), "r"(parity)
                : "memory");
        }
        return __syncthreads_and(done) != 0;
    };
    // the epilogue of tile tp, whose accumulators are TMEM set s
    auto epilogue = [&](int tp, int s) {
        const int mt = warp >> 2, q = warp & 3;  // warp -> (tile, TMEM lane quarter)
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
              "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
              "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
              "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(s * K::COLS) + 32u * mt));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        const int img = tp / tiles_img, tt = tp - img * tiles_img;
        const int m = q * 32 + lane;
        const int x = (tt % tiles_x) * TC5_C + (m & 7), y = (tt / tiles_x) * K::R + 16 * mt + (m >> 3);
        if (MODE == 2 && x < a.w && y < a.h) {
            *reinterpret_cast<float4*>((float*)a.out + img * a.out_stride + ((size_t)y * a.w + x) * 4) =
                make_float4(__uint_as_float(v[0]) + s_bias[0], __uint_as_float(v[1]) + s_bias[1],
                            __uint_as_float(v[2]) + s_bias[2], __uint_as_float(v[3]) + s_bias[3]);
        } else if (MODE != 2 && x < a.w && y < a.h) {
            __nv_bfloat16 o[32];
#pragma unroll
            for (int n = 0; n < 32; n++) o[n] = __float2bfloat16_rn(fmaxf(__uint_as_float(v[n]) + s_bias[n], 0.0f));
            uint4* dst =
                reinterpret_cast<uint4*>((__nv_bfloat16*)a.out + img * a.out_stride + ((size_t)y * a.w + x) * 32);
#pragma unroll
            for (int qq = 0; qq < 4; qq++) dst[qq] = reinterpret_cast<const uint4*>(o)[qq];
        }
    };
    // Tile t's MMAs (accumulator set it & 1) are issued; once tile t - 1's are done, tile
    // t + 1's halo starts into the buffer t - 1 released and t - 1's accumulators are drained
    // while tile t's MMAs run.
    bool ok = true;
    int it = 0, tprev = -1;
    for (; t < ntiles; t += gridDim.x, it++) {
        const int buf = it & 1;
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // this tile's halo has landed
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (threadIdx.x == 0) {
            const uint32_t abase = smem_u32(s_a0 + buf * K::HALO_B), bbase = smem_u32(s_b);
            const uint64_t a0 = tc5_desc(abase, MODE == 1 ? 16 : K::HR * K::HC * 16, K::HC * 16);
            const uint64_t b0 = tc5_desc(bbase, K::NB * 16, 8 * 16);
            constexpr uint32_t idesc = MODE == 2 ? kIdescBf16M128N16 : kIdescBf16M128N32;
            const uint32_t dcol = taddr + (uint32_t)(buf * K::COLS);
#pragma unroll 1
            for (int mt = 0; mt < MT; mt++) {
#pragma unroll
                for (int tap = 0; tap < 9; tap++) {
#pragma unroll
                    for (int kc = 0; kc < K::KCS; kc++) {
                        const uint64_t ad =
                            a0 + (uint64_t)((((2 * kc * K::HR + tap / 3 + 16 * mt) * K::HC + tap % 3) * 16) >> 4);
                        const uint64_t bd = b0 + (uint64_t)(((tap * K::WCB + 2 * kc) * K::NB * 16) >> 4);
                        asm volatile(
                            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol + 32u * mt),
                            "l"(ad), "l"(bd), "r"(idesc), "r"((tap | kc) ? 1u : 0u));
                    }
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             bar0 + 8u * (uint32_t)buf)
                         : "memory");
        }
        if (it > 0 && !(ok = wait_mma(it - 1))) break;
        // the other halo buffer is free once tile t - 1's MMAs are done: start tile t + 1's
        // copy first, then drain tile t - 1's accumulators while tile t's MMAs run
        if (t + (int)gridDim.x < ntiles) prefetch(t + gridDim.x, buf ^ 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        if (it > 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            epilogue(tprev, buf ^ 1);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        tprev = t;
    }
    if (ok && it > 0) {  // the last tile
        if ((ok = wait_mma(it - 1))) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            epilogue(tprev, (it - 1) & 1);
        }
    }
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "n"(2 * K::COLS));
}

// ---------------------------------------------------------------------------------------
// The whole forward pass in one kernel (inference): per 24x24-pixel output tile, the five
// layers run out of shared memory and TMEM; HBM sees only the fp32 input and output.
//   buffers: two 34x34-pixel activation buffers, [8-channel block][row][col][8 channels]
//            bf16 (the canonical no-swizzle K-major layout of the tc05 kernel), ping-pong;
//            the network input (4 channels) is a single 8-channel plane in the second one
//   layers:  each layer computes positions [1, 33) of the buffer (eight 16x8 MMA tiles, one
//            32-column TMEM accumulator each); the valid area shrinks by one pixel per layer
//            from [0, 34) to the tile [5, 29), so what lies outside it never reaches a valid
//            output.  Positions outside the image are stored as zero after every layer (the
//            per-layer zero padding of the layer-by-layer path)
//   layer 1: K = 16 of which 4 input channels; the second K core matrix is read 16 bytes on
//            (the next pixel, always finite) against zero weights
//   head:    N = 16 (4 real outputs), fp32 out for the tile's valid, in-image pixels
// Weights of all layers (72 KB) are staged once per persistent block.  One thread issues
// each layer's 72 (layer 1, head: 72) or 144 MMAs and commits them to an mbarrier; every wait is
// bounded (an error flag, then the block drains and frees TMEM).
// ---------------------------------------------------------------------------------------
constexpr int FU_O = 24, FU_G = FU_O + 10;
constexpr int FU_PLANE = FU_G * FU_G * 16;  // one 8-channel plane, bytes
constexpr int FU_ACT = 4 * FU_PLANE;        // 32 channels
constexpr int FU_W1 = 9 * 2 * 32 * 16, FU_WH = 9 * 4 * 32 * 16, FU_W5 = 9 * 4 * 16 * 16;
constexpr int FU_SMEM = 2 * FU_ACT + FU_W1 + 3 * FU_WH + FU_W5 + 5 * 32 * 4 + 64;  // + 2 mbarriers, TMEM address

struct FusedArgs {
    const float* in;  // [n][h][w][4]
    float* out;       // [n][h][w][4]
    int w, h, nimg;
    const __nv_bfloat16* wt[5];  // packed forward weights [nout_p][9][cin_p]
    const float* bias[5];
};

// bounded wait on phase `parity` of an mbarrier: at most `limit` non-blocking polls
// (test_wait), so the block resumes as soon as the MMAs complete and gives up after the
// limit; the verdict is block-uniform (every thread of the block calls it)
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t limit) {
    uint32_t done = 0;
    for (uint32_t k = 0; k < limit && !done; k++) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
    }
    return __syncthreads_and(done) != 0;
}

__device__ __forceinline__ bool fu_wait(uint32_t bar, uint32_t parity) { return mbar_wait_bounded(bar, parity, 4 * kWaitLimit); }

// The bounded wait of the tensor-core kernels on an mbarrier that nothing arrives at and to
// which no MMA was committed: the wait runs out with nothing in flight, and the block
// records the error as a block whose MMAs never completed does (gls_cnn_wait_probe).
__global__ void __launch_bounds__(128) wait_probe_kernel(int* err, uint32_t limit) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
    __syncthreads();
    const bool ok = mbar_wait_bounded(b, 0u, limit);
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(b) : "memory");
}

__device__ __forceinline__ void fu_sync_for_mma() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// One layer's MMAs (thread 0): tiles 0-3 committed to bar0, tiles 4-7 to bar1, so the
// epilogue of the first half runs while the second half computes.  Descriptors are the
// base descriptors plus the (16-byte unit) offsets of the tap, K step and tile.
template <int KCS, int NB>
__device__ __forceinline__ void fu_issue(uint32_t taddr, uint32_t abase, uint32_t lbo_a, uint32_t wbase,
                                         uint32_t idesc, uint32_t bar0, uint32_t bar1) {
    const uint64_t a0 = tc5_desc(abase, lbo_a, FU_G * 16), b0 = tc5_desc(wbase, NB * 16, 8 * 16);
#pragma unroll 1
    for (int t = 0; t < 8; t++) {
        const int rb = t >> 2, cbk = t & 3;
        const uint64_t at = a0 + (uint64_t)((16 * rb * FU_G + 8 * cbk) * 16 >> 4);
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
#pragma unroll
            for (int kc = 0; kc < KCS; kc++) {
                const uint64_t ad = at + (uint64_t)((2 * kc * FU_PLANE + ((tap / 3) * FU_G + tap % 3) * 16) >> 4);
                const uint64_t bd = b0 + (uint64_t)(((tap * 2 * KCS + 2 * kc) * NB * 16) >> 4);
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr + 32u * t),
                    "l"(ad), "l"(bd), "r"(idesc), "r"((tap | kc) ? 1u : 0u));
            }
        }
        if (t == 3)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar0)
                         : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar1)
                 : "memory");
}

// a 32-lane x 32-column accumulator read (no wait: tcgen05.wait::ld follows the batch)
__device__ __forceinline__ void fu_ld32_nowait(uint32_t addr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
          "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
          "=r"(v[30]), "=r"(v[31])
        : "r"(addr));
}

__device__ __forceinline__ void fu_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ void fu_ld32(uint32_t addr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
          "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
          "=r"(v[30]), "=r"(v[31])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// hidden-layer epilogue of four tiles (t0..t0+3): bias, ReLU, zero outside the image,
// bf16 into the next buffer; the four accumulator reads share one wait
__device__ __forceinline__ void fu_epilogue(uint32_t taddr, unsigned char* obuf, const float* bias, int y0, int x0,
                                            int w, int h, int t0) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, m = warp * 32 + lane;
    uint32_t v[4][32];
    const uint32_t base = taddr + ((uint32_t)(warp * 32) << 16) + 32u * t0;
#pragma unroll
    for (int q = 0; q < 4; q++) fu_ld32_nowait(base + 32u * q, v[q]);
    fu_ld_wait();
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int t = t0 + q;
        const int r = 1 + 16 * (t >> 2) + (m >> 3), c = 1 + 8 * (t & 3) + (m & 7);
        const int y = y0 - 5 + r, x = x0 - 5 + c;
        const bool in = x >= 0 && x < w && y >= 0 && y < h;
        uint32_t o[16];
#pragma unroll
        for (int n = 0; n < 16; n++) {
            const float lo = in ? fmaxf(__uint_as_float(v[q][2 * n]) + bias[2 * n], 0.0f) : 0.0f;
            const float hi = in ? fmaxf(__uint_as_float(v[q][2 * n + 1]) + bias[2 * n + 1], 0.0f) : 0.0f;
            const __nv_bfloat162 p2 = __floats2bfloat162_rn(lo, hi);
            o[n] = *reinterpret_cast<const uint32_t*>(&p2);
        }
        unsigned char* dst = obuf + (size_t)(r * FU_G + c) * 16;
#pragma unroll
        for (int cb = 0; cb < 4; cb++)
            *reinterpret_cast<uint4*>(dst + cb * FU_PLANE) = make_uint4(o[4 * cb], o[4 * cb + 1], o[4 * cb + 2], o[4 * cb + 3]);
    }
}

__global__ void __launch_bounds__(CT, 1) cnn_fused_kernel(FusedArgs a, int* err) {
    extern __shared__ __align__(1024) unsigned char fu_smem[];
    unsigned char* bufA = fu_smem;
    unsigned char* bufB = bufA + FU_ACT;
    unsigned char* w1 = bufB + FU_ACT;
    unsigned char* wh = w1 + FU_W1;  // layers 2..4
    unsigned char* w5 = wh + 3 * FU_WH;
    float* s_bias = reinterpret_cast<float*>(w5 + FU_W5);  // [5][32]
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_bias + 5 * 32);  // two
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(s_bar + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar = smem_u32(s_bar), bar1 = smem_u32(s_bar + 1);

    // everything the tensor cores may read stays finite: clear the buffers once
    for (int i = threadIdx.x; i < 2 * FU_ACT / 16; i += CT) reinterpret_cast<uint4*>(fu_smem)[i] = make_uint4(0, 0, 0, 0);
    // weights: [tap][8-channel block][n][8]
    for (int i = threadIdx.x; i < 9 * 2 * 32; i += CT) {
        const int tap = i / 64, r = i - tap * 64, cb = r / 32, n = r - cb * 32;
        *reinterpret_cast<uint4*>(w1 + (size_t)i * 16) =
            *reinterpret_cast<const uint4*>(a.wt[0] + (size_t)n * 144 + tap * 16 + cb * 8);
    }
    for (int l = 0; l < 3; l++)
        for (int i = threadIdx.x; i < 9 * 4 * 32; i += CT) {
            const int tap = i / 128, r = i - tap * 128, cb = r / 32, n = r - cb * 32;
            *reinterpret_cast<uint4*>(wh + (size_t)l * FU_WH + (size_t)i * 16) =
                *reinterpret_cast<const uint4*>(a.wt[1 + l] + (size_t)n * 288 + tap * 32 + cb * 8);
        }
    for (int i = threadIdx.x; i < 9 * 4 * 16; i += CT) {
        const int tap = i / 64, r = i - tap * 64, cb = r / 16, n = r - cb * 16;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (n < 8) v = *reinterpret_cast<const uint4*>(a.wt[4] + (size_t)n * 288 + tap * 32 + cb * 8);
        *reinterpret_cast<uint4*>(w5 + (size_t)i * 16) = v;
    }
    for (int i = threadIdx.x; i < 5 * 32; i += CT) {
        const int l = i / 32, n = i - l * 32;
        s_bias[i] = (l < 4 || n < 4) ? a.bias[l][n] : 0.0f;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;\n" ::"r"(smem_u32(s_taddr)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar1));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *s_taddr;
    const int tiles_x = cdiv_d(a.w, FU_O), tiles_y = cdiv_d(a.h, FU_O);
    const int tiles_img = tiles_x * tiles_y, ntiles = tiles_img * a.nimg;
    const long long img_px = (long long)a.w * a.h;
    uint32_t phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int img = t / tiles_img, tt = t - img * tiles_img;
        const int x0 = (tt % tiles_x) * FU_O, y0 = (tt / tiles_x) * FU_O;
        const float* in = a.in + (size_t)img * img_px * 4;
        // the network input: 34x34 pixels, 4 channels (sigma scaled) + 4 zero, bf16, into bufB
        constexpr int kPx = (FU_G * FU_G + CT - 1) / CT;  // pixels per thread; all loads first
        float4 f[kPx];
#pragma unroll
        for (int j = 0; j < kPx; j++) {
            const int p = threadIdx.x + j * CT, r = p / FU_G, c = p - r * FU_G;
            const int y = y0 - 5 + r, x = x0 - 5 + c;
            f[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (p < FU_G * FU_G && x >= 0 && x < a.w && y >= 0 && y < a.h)
                f[j] = __ldg(reinterpret_cast<const float4*>(in + ((size_t)y * a.w + x) * 4));
        }
#pragma unroll
        for (int j = 0; j < kPx; j++) {
            const int p = threadIdx.x + j * CT;
            if (p < FU_G * FU_G) {
                __nv_bfloat16 v[8];
                v[0] = __float2bfloat16_rn(f[j].x);
                v[1] = __float2bfloat16_rn(f[j].y);
                v[2] = __float2bfloat16_rn(f[j].z);
                v[3] = __float2bfloat16_rn(f[j].w * kSigmaScale);
#pragma unroll
                for (int k = 4; k < 8; k++) v[k] = __float2bfloat16_rn(0.0f);
                *reinterpret_cast<uint4*>(bufB + (size_t)p * 16) = *reinterpret_cast<const uint4*>(v);
            }
        }
        // layers 1-4: B -> A -> B -> A -> B ... then the head from B
        unsigned char* src = bufB;
        unsigned char* dst = bufA;
        for (int l = 0; l < 4 && ok; l++) {
            fu_sync_for_mma();
            if (threadIdx.x == 0) {
                if (l == 0)
                    fu_issue<1, 32>(taddr, smem_u32(src), 16, smem_u32(w1), kIdescBf16M128N32, bar, bar1);
                else
                    fu_issue<2, 32>(taddr, smem_u32(src), FU_PLANE, smem_u32(wh + (size_t)(l - 1) * FU_WH),
                                    kIdescBf16M128N32, bar, bar1);
            }
            for (int half = 0; half < 2 && ok; half++) {
                ok = fu_wait(half ? bar1 : bar, phase);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                fu_epilogue(taddr, dst, s_bias + 32 * l, y0, x0, a.w, a.h, 4 * half);
            }
            phase ^= 1u;
            if (!ok) break;
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            unsigned char* tmp = src;
            src = dst;
            dst = tmp;
        }
        if (!ok) break;
        // head: 32 -> 4 (N = 16), fp32 out for the tile's pixels inside the image
        fu_sync_for_mma();
        if (threadIdx.x == 0)
            fu_issue<2, 16>(taddr, smem_u32(src), FU_PLANE, smem_u32(w5), kIdescBf16M128N16, bar, bar1);
        ok = fu_wait(bar, phase) && fu_wait(bar1, phase);
        phase ^= 1u;
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        {
            const int m = warp * 32 + lane;
            float* out = a.out + (size_t)img * img_px * 4;
            for (int tl = 0; tl < 8; tl++) {
                uint32_t v[32];
                fu_ld32(taddr + ((uint32_t)(warp * 32) << 16) + 32u * tl, v);
                const int r = 1 + 16 * (tl >> 2) + (m >> 3), c = 1 + 8 * (tl & 3) + (m & 7);
                const int y = y0 - 5 + r, x = x0 - 5 + c;
                if (r >= 5 && r < 5 + FU_O && c >= 5 && c < 5 + FU_O && x < a.w && y < a.h) {
                    const float* b = s_bias + 32 * 4;
                    *reinterpret_cast<float4*>(out + ((size_t)y * a.w + x) * 4) =
                        make_float4(__uint_as_float(v[0]) + b[0], __uint_as_float(v[1]) + b[1],
                                    __uint_as_float(v[2]) + b[2], __uint_as_float(v[3]) + b[3]);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;\n" ::"r"(taddr));
}

// ---------------------------------------------------------------------------------------
// Weight gradient of one layer over one 8x16 pixel tile: dW[co][tap][ci] += sum_p
// dZ[p][co] * A[p + tap][ci] (A zero-padded), as an MMA with M = co, N = (tap, ci),
// K = the 16 pixels of a tile row.  Both operands are pixel-major in shared memory and
// come out of ldmatrix.trans in fragment order.  Each warp owns N / 4 columns; the block's
// partial (and the bias gradient) goes to its own row of `part`.
// ---------------------------------------------------------------------------------------
struct WgradArgs {
    const __nv_bfloat16* dz;  // [img][h][w][cout]
    int cout;
    const void* act;          // layer input: bf16 [img][h][w][cin_src] or fp32 for layer 0
    int cin_src;
    int w, h;
    size_t dz_stride, act_stride;
    float* part;              // [block][MOUT * 9 * CIN + MOUT]
};

template <int CIN, int MOUT, bool F32IN>
__global__ void __launch_bounds__(CT) wgrad_kernel(WgradArgs a) {
    constexpr int PS = CIN + 8, HW = TC + 2, HH = TR + 2;
    constexpr int N = 9 * CIN;
    constexpr int NTT = N / 8;              // n8 tiles in all
    constexpr int NTW = (NTT + 3) / 4;      // per warp: tiles warp, warp + 4, ...
    constexpr int MT = MOUT / 16;           // m16 tiles (MOUT 16 or 32)
    constexpr int DS = MOUT + 8;            // dz pixel stride
    __shared__ __align__(16) __nv_bfloat16 s_act[HH * HW * PS];
    __shared__ __align__(16) __nv_bfloat16 s_dz[TR * TC * DS];
    const int x0 = blockIdx.x * TC, y0 = blockIdx.y * TR, img = blockIdx.z;
    const int block = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const void* act = F32IN ? (const void*)((const float*)a.act + img * a.act_stride)
                            : (const void*)((const __nv_bfloat16*)a.act + img * a.act_stride);
    load_halo<CIN, F32IN>(s_act, act, a.cin_src, a.w, a.h, x0, y0);
    for (int i = threadIdx.x; i < TR * TC * (MOUT / 8); i += CT) {
        const int q = i % (MOUT / 8), p = i / (MOUT / 8);
        const int r = p / TC, c = p - r * TC, x = x0 + c, y = y0 + r;
        __nv_bfloat16 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = __float2bfloat16_rn(0.0f);
        if (x < a.w && y < a.h) {
            const __nv_bfloat16* b = a.dz + img * a.dz_stride + ((size_t)y * a.w + x) * a.cout;
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (q * 8 + k < a.cout) v[k] = b[q * 8 + k];
        }
        *reinterpret_cast<uint4*>(s_dz + (size_t)p * DS + q * 8) = *reinterpret_cast<uint4*>(v);
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    float acc[MT][NTW][4];
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
        for (int n = 0; n < NTW; n++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[m][n][k] = 0.0f;

    // A (M = co, K = pixel) from s_dz [pixel][co] through .trans: an x4 covers pixels 0-15
    // (K) x channels 16 (M): matrices (k 0-7, m 0-7), (k 0-7, m 8-15), (k 8-15, m 0-7),
    // (k 8-15, m 8-15) -> a0..a3 in fragment order needs (m0-7,k0-7), (m8-15,k0-7),
    // (m0-7,k8-15), (m8-15,k8-15).
    const int a_k = (lane & 7) + ((lane >> 4) << 3), a_m = ((lane >> 3) & 1) * 8;
    // B (K = pixel, N = (tap, ci)) from s_act through .trans: x2 over pixels 0-7 / 8-15 of
    // 8 channels; lane l -> pixel row (l & 7) + 8 * ((l >> 3) & 1)
    const int b_k = (lane & 7) + (((lane >> 3) & 1) << 3);
#pragma unroll 1
    for (int row = 0; row < TR; row++) {
        uint32_t af[MT][4];
#pragma unroll
        for (int m = 0; m < MT; m++)
            ldsm_x4_t(smem_u32(s_dz + (row * TC + a_k) * DS + m * 16 + a_m), af[m][0], af[m][1], af[m][2], af[m][3]);
#pragma unroll
        for (int n = 0; n < NTW; n++) {
            if (warp + 4 * n >= NTT) break;
            const int col = (warp + 4 * n) * 8;  // first (tap, ci) column of the tile
            const int tap = col / CIN, ci0 = col - tap * CIN;
            const int dy = tap / 3, dx = tap % 3;
            uint32_t b0, b1;
            ldsm_x2_t(smem_u32(s_act + ((row + dy) * HW + b_k + dx) * PS + ci0), b0, b1);
#pragma unroll
            for (int m = 0; m < MT; m++) mma_bf16(acc[m][n], af[m], b0, b1);
        }
    }
    // write the block's partial: thread holds rows (co) g, g + 8 and columns 2t, 2t + 1
    float* out = a.part + (size_t)block * (MOUT * N + MOUT);
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
        for (int n = 0; n < NTW; n++) {
            if (warp + 4 * n >= NTT) break;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int co = m * 16 + g + 8 * (k >> 1), col = (warp + 4 * n) * 8 + 2 * t + (k & 1);
                out[(size_t)co * N + col] = acc[m][n][k];
            }
        }
    // bias gradient: sum over the tile's pixels (fixed order)
    if (threadIdx.x < MOUT) {
        float s = 0.0f;
        for (int p = 0; p < TR * TC; p++) s += __bfloat162float(s_dz[p * DS + threadIdx.x]);
        out[MOUT * N + threadIdx.x] = s;
    }
}

// sum of the per-block partials, fixed order; one thread per output element
__global__ void reduce_rows_kernel(const float* part, int rows, int cols, float* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < rows; r++) s += part[(size_t)r * cols + j];
    out[j] = s;
}

// ---------------------------------------------------------------------------------------
// Loss of a batch and its gradient at the head.  in: [img][h][w][4] fp32 (R, G, B, sigma);
// head: [img][h][w][4] fp32 (strength logit, residual RGB in units of sigma); gt:
// [img][h][w][3] fp32.
//   residual loss  mean over pixels and channels of (in_rgb + sigma * r - gt)^2
//   strength loss  lambda * mean over pixels of (sigmoid(s) - tgt)^2, tgt = min(1, e2 / sigma^2) / 2
//                  with e2 the mean squared residual error of the pixel (no gradient through tgt);
//                  the pipeline scales the level-0 noise model by 2 sigmoid(s) (<= 1 after
//                  training; exactly 1 for a zero logit)
// The per-block sums of both losses go to part[block][2].
// ---------------------------------------------------------------------------------------
constexpr float kStrengthWeight = 0.1f;

__global__ void loss_grad_kernel(const float* in, const float* head, const float* gt, size_t npx, float inv_n,
                                 __nv_bfloat16* dhead, float* part) {
    __shared__ float red[2][8];
    float l0 = 0.0f, l1 = 0.0f;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npx; p += (size_t)gridDim.x * blockDim.x) {
        const float4 x = reinterpret_cast<const float4*>(in)[p];
        const float4 o = reinterpret_cast<const float4*>(head)[p];
        const float e0 = x.x + x.w * o.y - gt[3 * p + 0], e1 = x.y + x.w * o.z - gt[3 * p + 1],
                    e2 = x.z + x.w * o.w - gt[3 * p + 2];
        const float mse = (e0 * e0 + e1 * e1 + e2 * e2) * (1.0f / 3.0f);
        const float tgt = 0.5f * fminf(1.0f, mse / fmaxf(x.w * x.w, 1e-8f));
        const float s = 1.0f / (1.0f + expf(-o.x));
        l0 += 3.0f * mse;
        l1 += (s - tgt) * (s - tgt);
        const float gr = 2.0f * inv_n * (1.0f / 3.0f) * x.w;
        const float gs = kStrengthWeight * 2.0f * inv_n * (s - tgt) * s * (1.0f - s);
        __nv_bfloat16* d = dhead + 4 * p;
        d[0] = __float2bfloat16_rn(gs);
        d[1] = __float2bfloat16_rn(gr * e0);
        d[2] = __float2bfloat16_rn(gr * e1);
        d[3] = __float2bfloat16_rn(gr * e2);
    }
    for (int o = 16; o > 0; o >>= 1) {
        l0 += __shfl_xor_sync(0xffffffffu, l0, o);
        l1 += __shfl_xor_sync(0xffffffffu, l1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = l0;
        red[1][threadIdx.x >> 5] = l1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f, b = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            a += red[0][w];
            b += red[1][w];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// Adam on the FP32 master parameters, then the bf16 copies both convolutions read:
// forward [NOUT][9][CIN] and input-gradient [CIN_T][9][NOUT_T] (taps flipped).
struct AdamArgs {
    float* p;
    float* m;
    float* v;
    const float* g;
    int n;
    float lr, b1, b2, eps, c1, c2;  // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
};

__global__ void adam_kernel(AdamArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float g = a.g[i];
    const float m = a.b1 * a.m[i] + (1.0f - a.b1) * g;
    const float v = a.b2 * a.v[i] + (1.0f - a.b2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    a.p[i] -= a.lr * (m * a.c1) / (sqrtf(v * a.c2) + a.eps);
}

// master layout of layer l: W [cout][3][3][cin] then b [cout]
__global__ void pack_weights_kernel(const float* wl, int cin, int cout, int cin_p, int nout_p, __nv_bfloat16* fwd,
                                    int cint_p, int noutt_p, __nv_bfloat16* bwd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // forward: [nout_p][9][cin_p]
    if (i < nout_p * 9 * cin_p) {
        const int co = i / (9 * cin_p), r = i - co * 9 * cin_p, tap = r / cin_p, ci = r - tap * cin_p;
        const float v = (co < cout && ci < cin) ? wl[((size_t)co * 9 + tap) * cin + ci] : 0.0f;
        fwd[i] = __float2bfloat16_rn(v);
    }
    // input gradient: [noutt_p = cin channels out][9][cint_p = cout channels in], tap flipped
    if (bwd && i < noutt_p * 9 * cint_p) {
        const int ci = i / (9 * cint_p), r = i - ci * 9 * cint_p, tap = r / cint_p, co = r - tap * cint_p;
        const float v = (co < cout && ci < cin) ? wl[((size_t)co * 9 + (8 - tap)) * cin + ci] : 0.0f;
        bwd[i] = __float2bfloat16_rn(v);
    }
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// sum the wgrad partials of layer l and scatter into grad[off[l]...] (W [cout][9][cin], b)
__global__ void scatter_wgrad_kernel(const float* part, int rows, int mout, int cin_p, int cout, int cin, float* gw) {
    const int n = 9 * cin_p;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= mout * n + mout) return;
    float s = 0.0f;
    const int cols = mout * n + mout;
    for (int r = 0; r < rows; r++) s += part[(size_t)r * cols + j];
    if (j < mout * n) {
        const int co = j / n, k = j - co * n, tap = k / cin_p, ci = k - tap * cin_p;
        if (co < cout && ci < cin) gw[((size_t)co * 9 + tap) * cin + ci] = s;
    } else {
        const int co = j - mout * n;
        if (co < cout) gw[(size_t)cout * 9 * cin + co] = s;
    }
}


}  // namespace
}  // namespace gls

using namespace gls;

// ---------------------------------------------------------------------------------------
// the network object
// ---------------------------------------------------------------------------------------
struct gls_cnn {
    gls_ctx* ctx = nullptr;
    float* master = nullptr;  // all layers' parameters, FP32
    float* grad = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int nparam = 0;
    int off[kLayers] = {};  // offset of layer l in master
    __nv_bfloat16* wfwd[kLayers] = {};
    __nv_bfloat16* wbwd[kLayers] = {};
    long step = 0;
    // activations of the last forward (training keeps them for the backward)
    int cap_px = 0;  // pixels (all images) the buffers hold
    __nv_bfloat16* act[kLayers - 1] = {};  // layer outputs 0..3 (32 ch)
    __nv_bfloat16* grad_a = nullptr;       // 32-ch gradient ping
    __nv_bfloat16* grad_b = nullptr;       // 32-ch gradient pong
    __nv_bfloat16* dhead = nullptr;        // 4 ch
    float* head = nullptr;                 // 4 ch fp32
    float* part = nullptr;
    size_t part_floats = 0;
    float* loss_dev = nullptr;
    float* loss_host = nullptr;
    // forward pass: 2 one fused tcgen05 kernel for inference (training keeps the per-layer
    // path, whose activations the backward pass reads), 1 tcgen05 hidden layers (default),
    // 0 mma.sync; the backward pass is mma.sync
    int backend = 1;
    int* err_dev = nullptr;  // set by a tcgen05 block whose wait ran out

    ~gls_cnn() {
        void* ps[] = {master, grad, adam_m, adam_v, grad_a, grad_b, dhead, head, part, loss_dev, err_dev};
        for (void* p : ps)
            if (p) cudaFree(p);
        for (int l = 0; l < kLayers; l++) {
            if (wfwd[l]) cudaFree(wfwd[l]);
            if (wbwd[l]) cudaFree(wbwd[l]);
        }
        for (int l = 0; l < kLayers - 1; l++)
            if (act[l]) cudaFree(act[l]);
        if (loss_host) cudaFreeHost(loss_host);
    }

    static int cin_p(int l) { return l == 0 ? 16 : 32; }
    static int nout_p(int l) { return l == kLayers - 1 ? 8 : 32; }
    // input-gradient convolution of layer l >= 1: in = cout (padded to 16/32), out = cin
    static int cint_p(int l) { return kCout[l] <= 16 ? 16 : 32; }

    gls_status pack() {
        for (int l = 0; l < kLayers; l++) {
            const int nf = nout_p(l) * 9 * cin_p(l), nb = l > 0 ? 32 * 9 * cint_p(l) : 0;
            pack_weights_kernel<<<cdiv(nf > nb ? nf : nb, 256), 256, 0, ctx->stream>>>(
                master + off[l], kCin[l], kCout[l], cin_p(l), nout_p(l), wfwd[l], cint_p(l), 32, l > 0 ? wbwd[l] : nullptr);
            ctx->launches++;
        }
        return check_launch(ctx, "CNN weight packing");
    }

    gls_status ensure_batch(int px) {
        if (px <= cap_px) return GLS_OK;
        cudaStreamSynchronize(ctx->stream);
        for (int l = 0; l < kLayers - 1; l++) {
            if (act[l]) cudaFree(act[l]);
            act[l] = nullptr;
        }
        void* ps[] = {grad_a, grad_b, dhead, head};
        for (void* p : ps)
            if (p) cudaFree(p);
        grad_a = grad_b = dhead = nullptr;
        head = nullptr;
        cap_px = 0;
        for (int l = 0; l < kLayers - 1; l++)
            GLS_CHECK(check_cuda(ctx, cudaMalloc(&act[l], (size_t)px * 32 * 2), "cudaMalloc(CNN activations)"));
        GLS_CHECK(check_cuda(ctx, cudaMalloc(&grad_a, (size_t)px * 32 * 2), "cudaMalloc(CNN gradients)"));
        GLS_CHECK(check_cuda(ctx, cudaMalloc(&grad_b, (size_t)px * 32 * 2), "cudaMalloc(CNN gradients)"));
        GLS_CHECK(check_cuda(ctx, cudaMalloc(&dhead, (size_t)px * 4 * 2), "cudaMalloc(CNN gradients)"));
        GLS_CHECK(check_cuda(ctx, cudaMalloc(&head, (size_t)px * 4 * 4), "cudaMalloc(CNN head)"));
        cap_px = px;
        return GLS_OK;
    }

    gls_status ensure_part(size_t floats) {
        if (floats <= part_floats) return GLS_OK;
        cudaStreamSynchronize(ctx->stream);
        if (part) cudaFree(part);
        part = nullptr;
        part_floats = 0;
        GLS_CHECK(check_cuda(ctx, cudaMalloc(&part, floats * 4), "cudaMalloc(CNN partials)"));
        part_floats = floats;
        return GLS_OK;
    }

    // one convolution over a batch of n images of w x h
    template <int CIN, int NOUT, int EPI, bool F32IN>
    void conv(const void* in, int cin_src, size_t in_stride, const __nv_bfloat16* wt, const float* bias, void* out,
              int cout, size_t out_stride, const __nv_bfloat16* mask, size_t mask_stride, int w, int h, int n) {
        ConvArgs a{in, cin_src, wt, bias, out, cout, mask, w, h, in_stride, out_stride, mask_stride};
        conv3x3_kernel<CIN, NOUT, EPI, F32IN><<<dim3(cdiv(w, TC), cdiv(h, TR), n), CT, 0, ctx->stream>>>(a);
        ctx->launches++;
    }

    // one layer on tcgen05 (MODE as conv3x3_tc05_kernel)
    template <int MODE>
    gls_status tc05(const ConvArgs& a, int w, int h, int n) {
        using K = Tc5<kTc5Stack, MODE>;
        static bool attr_set = false;
        if (!attr_set) {
            GLS_CHECK(check_cuda(ctx, cudaFuncSetAttribute(conv3x3_tc05_kernel<kTc5Stack, MODE>,
                                                           cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM),
                                 "cudaFuncSetAttribute(tcgen05 convolution)"));
            attr_set = true;
        }
        const int tiles = cdiv(w, TC5_C) * cdiv(h, K::R) * n;
        const int per = kTc5BlocksPerSm * (ctx->num_sms > 0 ? ctx->num_sms : 148);
        conv3x3_tc05_kernel<kTc5Stack, MODE><<<tiles < per ? tiles : per, K::THREADS, K::SMEM, ctx->stream>>>(
            a, n, err_dev);
        ctx->launches++;
        return GLS_OK;
    }

    // forward over n images [n][h][w][4] fp32 -> head [n][h][w][4] fp32 (out or this->head)
    gls_status forward(const float* in, int w, int h, int n, float* out) {
        const size_t px = (size_t)w * h;
        if (backend == 2 && out) {  // inference: the fused kernel, no activations kept
            static bool attr_set = false;
            if (!attr_set) {
                GLS_CHECK(check_cuda(ctx, cudaFuncSetAttribute(cnn_fused_kernel,
                                                               cudaFuncAttributeMaxDynamicSharedMemorySize, FU_SMEM),
                                     "cudaFuncSetAttribute(CNN fused)"));
                attr_set = true;
            }
            FusedArgs fa;
            fa.in = in;
            fa.out = out;
            fa.w = w;
            fa.h = h;
            fa.nimg = n;
            for (int l = 0; l < kLayers; l++) {
                fa.wt[l] = wfwd[l];
                fa.bias[l] = master + off[l] + kCout[l] * 9 * kCin[l];
            }
            const int tiles = cdiv(w, FU_O) * cdiv(h, FU_O) * n;
            const int sms = ctx->num_sms > 0 ? ctx->num_sms : 148;
            cnn_fused_kernel<<<tiles < sms ? tiles : sms, CT, FU_SMEM, ctx->stream>>>(fa, err_dev);
            ctx->launches++;
            return check_launch(ctx, "CNN forward (fused)");
        }
        GLS_CHECK(ensure_batch((int)(px * n)));
        const float* b = master;
        if (backend == 1) {  // every layer on tcgen05
            GLS_CHECK(tc05<1>(ConvArgs{in, 4, wfwd[0], b + off[0] + 32 * 9 * 4, act[0], 32, nullptr, w, h, px * 4,
                                       px * 32, 0},
                              w, h, n));
            for (int l = 1; l < kLayers - 1; l++)
                GLS_CHECK(tc05<0>(ConvArgs{act[l - 1], 32, wfwd[l], b + off[l] + 32 * 9 * 32, act[l], 32, nullptr, w,
                                           h, px * 32, px * 32, 0},
                                  w, h, n));
            GLS_CHECK(tc05<2>(ConvArgs{act[3], 32, wfwd[4], b + off[4] + 4 * 9 * 32, out ? out : head, 4, nullptr, w,
                                       h, px * 32, px * 4, 0},
                              w, h, n));
            return check_launch(ctx, "CNN forward");
        }
        conv<16, 32, 0, true>(in, 4, px * 4, wfwd[0], b + off[0] + 32 * 9 * 4, act[0], 32, px * 32, nullptr, 0, w, h, n);
        for (int l = 1; l < kLayers - 1; l++)
            conv<32, 32, 0, false>(act[l - 1], 32, px * 32, wfwd[l], b + off[l] + 32 * 9 * 32, act[l], 32, px * 32,
                                   nullptr, 0, w, h, n);
        conv<32, 8, 1, false>(act[3], 32, px * 32, wfwd[4], b + off[4] + 4 * 9 * 32, out ? out : head, 4, px * 4,
                              nullptr, 0, w, h, n);
        return check_launch(ctx, "CNN forward");
    }
};


extern "C" {

gls_status gls_cnn_create(gls_ctx* ctx, gls_cnn** out) {
    if (!ctx || !out) return GLS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    gls_cnn* c = new gls_cnn();
    c->ctx = ctx;
    int n = 0;
    for (int l = 0; l < kLayers; l++) {
        c->off[l] = n;
        n += kCout[l] * 9 * kCin[l] + kCout[l];
    }
    c->nparam = n;
    gls_status s = GLS_OK;
    auto al = [&](void** p, size_t bytes) {
        if (s == GLS_OK) s = check_cuda(ctx, cudaMalloc(p, bytes), "cudaMalloc(CNN parameters)");
        if (s == GLS_OK) s = check_cuda(ctx, cudaMemsetAsync(*p, 0, bytes, ctx->stream), "clear CNN parameters");
    };
    al((void**)&c->master, (size_t)n * 4);
    al((void**)&c->grad, (size_t)n * 4);
    al((void**)&c->adam_m, (size_t)n * 4);
    al((void**)&c->adam_v, (size_t)n * 4);
    for (int l = 0; l < kLayers; l++) {
        al((void**)&c->wfwd[l], (size_t)gls_cnn::nout_p(l) * 9 * gls_cnn::cin_p(l) * 2);
        if (l > 0) al((void**)&c->wbwd[l], (size_t)32 * 9 * gls_cnn::cint_p(l) * 2);
    }
    al((void**)&c->loss_dev, 64 * 4);
    al((void**)&c->err_dev, sizeof(int));
    if (s == GLS_OK) s = check_cuda(ctx, cudaMallocHost(&c->loss_host, 64 * 4), "cudaMallocHost");
    if (s != GLS_OK) {
        delete c;
        return s;
    }
    *out = c;
    return GLS_OK;
}

gls_status gls_cnn_destroy(gls_cnn* c) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(c->ctx->stream);
    delete c;
    return GLS_OK;
}

int gls_cnn_param_count(void) {
    int n = 0;
    for (int l = 0; l < kLayers; l++) n += kCout[l] * 9 * kCin[l] + kCout[l];
    return n;
}

gls_status gls_cnn_set_backend(gls_cnn* c, int backend) {
    if (!c || backend < 0 || backend > 2) return GLS_ERR_INVALID_ARGUMENT;
    c->backend = backend;
    return GLS_OK;
}

int gls_cnn_get_backend(gls_cnn* c) { return c ? c->backend : -1; }

gls_status gls_cnn_status(gls_cnn* c) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    int e = 0;
    GLS_CHECK(check_cuda(c->ctx, cudaMemcpyAsync(&e, c->err_dev, sizeof(int), cudaMemcpyDeviceToHost, c->ctx->stream),
                         "read CNN status"));
    GLS_CHECK(check_cuda(c->ctx, cudaStreamSynchronize(c->ctx->stream), "synchronize"));
    if (e) {
        // reported once: the flag is cleared for the calls that follow
        GLS_CHECK(check_cuda(c->ctx, cudaMemsetAsync(c->err_dev, 0, sizeof(int), c->ctx->stream), "clear CNN status"));
        return set_error(c->ctx, GLS_ERR_TIMEOUT, "CNN: a tensor-core wait ran out");
    }
    return GLS_OK;
}

gls_status gls_cnn_wait_probe(gls_cnn* c, unsigned polls) {
    if (!c || polls == 0 || polls > kWaitLimit) return GLS_ERR_INVALID_ARGUMENT;
    wait_probe_kernel<<<1, 128, 0, c->ctx->stream>>>(c->err_dev, polls);
    c->ctx->launches++;
    return check_launch(c->ctx, "CNN wait probe");
}

gls_status gls_cnn_set_params(gls_cnn* c, const float* params, int n) {
    if (!c || !params) return GLS_ERR_INVALID_ARGUMENT;
    if (n != c->nparam) return set_error(c->ctx, GLS_ERR_INVALID_SIZE, "CNN: %d parameters expected, got %d", c->nparam, n);
    GLS_CHECK(check_cuda(c->ctx, cudaMemcpyAsync(c->master, params, (size_t)n * 4, cudaMemcpyHostToDevice, c->ctx->stream),
                         "copy CNN parameters"));
    GLS_CHECK(check_cuda(c->ctx, cudaMemsetAsync(c->adam_m, 0, (size_t)n * 4, c->ctx->stream), "reset Adam"));
    GLS_CHECK(check_cuda(c->ctx, cudaMemsetAsync(c->adam_v, 0, (size_t)n * 4, c->ctx->stream), "reset Adam"));
    c->step = 0;
    GLS_CHECK(c->pack());
    return check_cuda(c->ctx, cudaStreamSynchronize(c->ctx->stream), "synchronize");
}

gls_status gls_cnn_get_params(gls_cnn* c, float* params, int n) {
    if (!c || !params) return GLS_ERR_INVALID_ARGUMENT;
    if (n != c->nparam) return set_error(c->ctx, GLS_ERR_INVALID_SIZE, "CNN: %d parameters expected, got %d", c->nparam, n);
    GLS_CHECK(check_cuda(c->ctx, cudaMemcpyAsync(params, c->master, (size_t)n * 4, cudaMemcpyDeviceToHost, c->ctx->stream),
                         "copy CNN parameters"));
    return check_cuda(c->ctx, cudaStreamSynchronize(c->ctx->stream), "synchronize");
}

gls_status gls_cnn_get_grads(gls_cnn* c, float* grads, int n) {
    if (!c || !grads) return GLS_ERR_INVALID_ARGUMENT;
    if (n != c->nparam) return set_error(c->ctx, GLS_ERR_INVALID_SIZE, "CNN: %d parameters expected, got %d", c->nparam, n);
    GLS_CHECK(check_cuda(c->ctx, cudaMemcpyAsync(grads, c->grad, (size_t)n * 4, cudaMemcpyDeviceToHost, c->ctx->stream),
                         "copy CNN gradients"));
    return check_cuda(c->ctx, cudaStreamSynchronize(c->ctx->stream), "synchronize");
}

// in: device [n][h][w][4] fp32 (R, G, B, sigma); out: device [n][h][w][4] fp32 (strength logit, residual RGB)
gls_status gls_cnn_forward(gls_cnn* c, const float* in, int width, int height, int n, float* out) {
    if (!c || !in || !out) return GLS_ERR_INVALID_ARGUMENT;
    if (width <= 0 || height <= 0 || n <= 0) return set_error(c->ctx, GLS_ERR_INVALID_SIZE, "CNN: empty batch");
    return c->forward(in, width, height, n, out);
}

// One training step on a batch: forward, loss, backward, Adam.  gt: device [n][h][w][3]
// fp32.  loss[0] = mean squared residual error per channel, loss[1] = strength loss.
// With lr = 0 the parameters stay and the gradients of the batch are left for
// gls_cnn_get_grads.
gls_status gls_cnn_train_step(gls_cnn* c, const float* in, const float* gt, int w, int h, int n, float lr,
                              float loss[2]) {
    if (!c || !in || !gt) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = c->ctx;
    if (w <= 0 || h <= 0 || n <= 0) return set_error(ctx, GLS_ERR_INVALID_SIZE, "CNN: empty batch");
    const size_t px = (size_t)w * h, npx = px * n;
    GLS_CHECK(c->forward(in, w, h, n, nullptr));
    // loss and head gradient
    const int lblocks = 256;
    GLS_CHECK(c->ensure_part((size_t)lblocks * 2));
    loss_grad_kernel<<<lblocks, 256, 0, ctx->stream>>>(in, c->head, gt, npx, 1.0f / (float)npx, c->dhead, c->part);
    reduce_rows_kernel<<<1, 32, 0, ctx->stream>>>(c->part, lblocks, 2, c->loss_dev);
    ctx->launches += 2;
    cudaMemcpyAsync(c->loss_host, c->loss_dev, 2 * 4, cudaMemcpyDeviceToHost, ctx->stream);

    const dim3 grid(cdiv(w, TC), cdiv(h, TR), n);
    const int blocks = grid.x * grid.y * grid.z;
    auto wgrad_layer = [&](int l, const __nv_bfloat16* dz) -> gls_status {
        const int mout = l == kLayers - 1 ? 16 : 32, cinp = gls_cnn::cin_p(l);
        const int cols = mout * 9 * cinp + mout;
        GLS_CHECK(c->ensure_part((size_t)blocks * cols));
        WgradArgs a{dz, kCout[l], l == 0 ? (const void*)in : (const void*)c->act[l - 1], l == 0 ? 4 : 32, w, h,
                    px * kCout[l], px * (l == 0 ? 4 : 32), c->part};
        if (l == 0) wgrad_kernel<16, 32, true><<<grid, CT, 0, ctx->stream>>>(a);
        else if (l == kLayers - 1) wgrad_kernel<32, 16, false><<<grid, CT, 0, ctx->stream>>>(a);
        else wgrad_kernel<32, 32, false><<<grid, CT, 0, ctx->stream>>>(a);
        scatter_wgrad_kernel<<<cdiv(cols, 256), 256, 0, ctx->stream>>>(c->part, blocks, mout, cinp, kCout[l], kCin[l],
                                                                        c->grad + c->off[l]);
        ctx->launches += 2;
        return GLS_OK;
    };
    // layer 4 (head): dz = dhead (4 ch)
    GLS_CHECK(wgrad_layer(4, c->dhead));
    // dA3 = conv(dhead, W4 flipped) masked by act[3] > 0
    c->conv<16, 32, 2, false>(c->dhead, 4, px * 4, c->wbwd[4], nullptr, c->grad_a, 32, px * 32, c->act[3], px * 32, w, h,
                              n);
    __nv_bfloat16* dz = c->grad_a;
    __nv_bfloat16* other = c->grad_b;
    for (int l = kLayers - 2; l >= 1; l--) {
        GLS_CHECK(wgrad_layer(l, dz));
        c->conv<32, 32, 2, false>(dz, 32, px * 32, c->wbwd[l], nullptr, other, 32, px * 32, c->act[l - 1], px * 32, w,
                                  h, n);
        __nv_bfloat16* t = dz;
        dz = other;
        other = t;
    }
    GLS_CHECK(wgrad_layer(0, dz));
    GLS_CHECK(check_launch(ctx, "CNN backward"));
    if (lr > 0.0f) {
        c->step++;
        AdamArgs a;
        a.p = c->master;
        a.m = c->adam_m;
        a.v = c->adam_v;
        a.g = c->grad;
        a.n = c->nparam;
        a.lr = lr;
        a.b1 = 0.9f;
        a.b2 = 0.999f;
        a.eps = 1e-8f;
        a.c1 = (float)(1.0 / (1.0 - pow(0.9, (double)c->step)));
        a.c2 = (float)(1.0 / (1.0 - pow(0.999, (double)c->step)));
        adam_kernel<<<cdiv(c->nparam, 256), 256, 0, ctx->stream>>>(a);
        ctx->launches++;
        GLS_CHECK(c->pack());
    }
    GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize"));
    if (loss) {
        loss[0] = c->loss_host[0] / (float)(3 * npx);
        loss[1] = c->loss_host[1] / (float)npx;
    }
    return check_launch(ctx, "CNN training step");
}

}  // extern "C"
