// k_fused.cu -- the RAW pipeline as a handful of fused, shared-memory-tiled kernels.
//
// Each kernel reads its input tile (with the halo its stencils need) from HBM once,
// runs several reference stages back to back out of shared memory, and writes only the
// images that later passes need.  Every value that the reference stores in an
// intermediate image is rounded to that image's storage precision at the same point,
// and every image read outside the frame is clamped to the edge exactly as the
// reference's sampler-less reads are, so the results equal the single-stage kernels
// (k_stages.cu) and the CPU oracle bit for bit.
//
//   raw_pass1      scaleRawData on the fly + rawNoiseStatistics + pass-1 regression sums
//   demosaic       scaleRawData + interpolateGreen (shared Sobel map) + interpolateRedBlue
//                  + blendHighlights + transformImage(cam->YCbCr) + despeckleImage
//                  -> level 0 of the pyramid (binary16: the despeckle already rounds
//                  every value to binary16, so this storage is exact)
//   level_pass1    noiseStatistics + pass-1 sums of level i, downsampleImage -> level i+1
//   denoise_reasm  denoiseImage (+ reassembleImage) of levels >= 1
//   final          denoiseImage + reassembleImage of level 0, localToneMappingMask,
//                  transformImage(YCbCr->camera), convertTosRGB -> RGBA8 / RGBA fp32
#include <cuda.h>

#include <cstring>

#include "gls_fused.h"
#include "gls_nlf.cuh"
#include "gls_tune.h"

namespace gls {
namespace {

constexpr int kT = 256;
static_assert(kT == kThreads, "the regression epilogue reduces over blocks of kThreads");

// ---- shared-memory accessors (coordinates in image space, origin at (x0, y0)) ----
struct SAcc1 {
    const float* s;
    int x0, y0, ld;
    GLS_DI float at(int x, int y) const { return s[(y - y0) * ld + (x - x0)]; }
};

struct SAcc4h {
    const half4* s;
    int x0, y0, ld;
    GLS_DI float4 at(int x, int y) const { return Storage<__half>::cvt(s[(y - y0) * ld + (x - x0)]); }
};

struct SAcc4f {
    const float4* s;
    int x0, y0, ld;
    GLS_DI float4 at(int x, int y) const { return s[(y - y0) * ld + (x - x0)]; }
};

// a staged RGBA tile whose .w the kernel set to 1 (see unit_w in gls_pixel_ops.cuh)
struct SAcc4f1 : SAcc4f {
    static constexpr bool kUnitW = true;
};

struct SobelMap {
    const float4* base;  // {|gx|, |gy|, length, -}
    int x0, y0, ld, x, y;
    GLS_DI SobelVal operator()(int i, int j) const {
        const float4 q = base[(y + j - y0) * ld + (x + i - x0)];
        SobelVal v;
        v.gx = q.x;
        v.gy = q.y;
        v.len = q.z;
        return v;
    }
};

GLS_DI half4 to_half4(float4 v) {
    half4 h;
    h.xy = __halves2half2(__float2half_rn(v.x), __float2half_rn(v.y));
    h.zw = __halves2half2(__float2half_rn(v.z), __float2half_rn(v.w));
    return h;
}

template <class S>
GLS_DI float3 round3(float3 v) {
    return make_float3(Storage<S>::round(v.x), Storage<S>::round(v.y), Storage<S>::round(v.z));
}

template <class S>
GLS_DI float4 round4(float4 v) {
    return make_float4(Storage<S>::round(v.x), Storage<S>::round(v.y), Storage<S>::round(v.z), Storage<S>::round(v.w));
}

// ---- TMA tile staging (raw_pass1, level_pass1) ----
constexpr uint32_t kStageWaitPolls = 1u << 22;  // bound of a staging wait (each poll a try_wait)

GLS_DI void tma_issue_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// every thread of the block calls it; true once phase `parity` of the barrier completed
GLS_DI bool stage_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
    uint32_t done = 0;
    for (uint32_t k = 0; k < limit && !done; k++) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
    }
    return __syncthreads_and(done) != 0;
}

// =========================================================================================
// raw_pass1: per 2x2 quad, the 5x5-quad statistics of the scaled raw planes and the
// pass-1 sums of computeRawNoiseStatistics.  Tiles of 32x32 quads: the scaled values are
// staged once per quad as a float4 of its four CFA channels (kernel order), each thread
// sums the windows of 4 quads of a column from one pass over 8 staged rows (every window
// still sums its taps in the reference's row-major order), the channel pairs (0, 1) and
// (2, 3) run as packed fp32x2 chains, and the regression sums are packed likewise.
// =========================================================================================
constexpr int RQ = 32;        // quads per tile side
constexpr int RQS = RQ + 4;   // staged quads per side (halo of 2 quads)

// x / 25 per lane by the shortcut of div25 (reciprocal 0.04, one correction step), exact for
// a lane that is 0 or in [2^-83, 2^60]; CHECK sends other lanes to the literal division.
template <bool CHECK>
GLS_DI float2 div25_x2(float2 x) {
    const float2 y = f2(0.04f, 0.04f);
    const float2 q0 = mul2(x, y);  // a multiplicand and an fma addend only
    float2 q = fma2(fma2(q0, f2(-25.0f, -25.0f), x), y, q0);
    if (CHECK) {
        if (!FastDiv::in_range(x.x)) q.x = glsm::div_slow(x.x, 25.0f);
        if (!FastDiv::in_range(x.y)) q.y = glsm::div_slow(x.y, 25.0f);
    }
    return q;
}

// The raw region of a tile by TMA: 80 x 72 pixels from (2 qx0 - 8, 2 qy0 - 4), so that x is
// a multiple of 8 pixels (16 bytes) and a row of the box is 160 bytes; the staged quads
// start 4 pixels in.
constexpr int RBW = 2 * RQS + 8, RBH = 2 * RQS;

template <class S, int BAYER>
__global__ void __launch_bounds__(kT, 2) raw_pass1_kernel(RawPass1Args a, const __grid_constant__ CUtensorMap tmap) {  // 2 resident blocks per SM
    constexpr uint32_t kStageBytes = RBW * RBH * 2;
    __shared__ float4 s_q[RQS * RQS];
    __shared__ __align__(128) uint16_t s_stage[2][RBW * RBH];
    __shared__ __align__(8) uint64_t s_bar[2];
    RawPass1Acc2 acc;
    acc.init();
    const int qw = a.w / 2, qh = a.h / 2;
    const int tiles_x = (qw + RQ - 1) / RQ, tiles_y = (qh + RQ - 1) / RQ, ntiles = tiles_x * tiles_y;
    const int col = threadIdx.x & 31, row0 = (threadIdx.x >> 5) * 4;
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&s_bar[0]);
    const uint32_t stage0 = (uint32_t)__cvta_generic_to_shared(&s_stage[0][0]);
    if (threadIdx.x == 0 && a.tma) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto by_tma = [&](int t) {
        const int px0 = 2 * (t % tiles_x) * RQ, py0 = 2 * (t / tiles_x) * RQ;
        return a.tma && px0 >= 8 && py0 >= 4 && px0 + 2 * RQ + 8 <= a.w && py0 + 2 * RQ + 4 <= a.h;
    };
    auto issue = [&](int t, int b) {  // thread 0
        const int px0 = 2 * (t % tiles_x) * RQ, py0 = 2 * (t / tiles_x) * RQ;
        tma_issue_2d(stage0 + (uint32_t)b * kStageBytes, &tmap, px0 - 8, py0 - 4, bar0 + 8u * (uint32_t)b, kStageBytes);
    };
    uint32_t parity = 0;
    bool pending = false;
    int buf = 0;
    int t = blockIdx.x;
    if (t < ntiles && by_tma(t)) {
        if (threadIdx.x == 0) issue(t, 0);
        pending = true;
    }
    for (; t < ntiles; t += gridDim.x, buf ^= 1) {
        const int qx0 = (t % tiles_x) * RQ, qy0 = (t / tiles_x) * RQ;
        if (pending) {
            const uint32_t par = (parity >> buf) & 1u;
            parity ^= 1u << buf;
            if (!stage_wait(bar0 + 8u * (uint32_t)buf, par, kStageWaitPolls)) {
                if (threadIdx.x == 0) atomicOr(a.nlf.err, 1u);
                stage_wait(bar0 + 8u * (uint32_t)buf, par, kStageWaitPolls);
                break;
            }
            // quads from the staged pixels: (2c + 4 + dx, 2r + dy); the pixel's parity is the
            // channel's (dx, dy), as the frame's coordinates are even at the quad
            const uint16_t* st = s_stage[buf];
            for (int i = threadIdx.x; i < RQS * RQS; i += kT) {
                const int r = i / RQS, c = i - r * RQS;
                float v[4];
#pragma unroll
                for (int ch = 0; ch < 4; ch++) {
                    const int dx = bayer_dx(BAYER, ch), dy = bayer_dy(BAYER, ch);
                    v[ch] = Storage<S>::round(scale_value(st[(2 * r + dy) * RBW + 2 * c + 4 + dx], a.sm[(dy << 1) | dx], a.black));
                }
                s_q[i] = make_float4(v[0], v[1], v[2], v[3]);
            }
        } else {
            for (int i = threadIdx.x; i < RQS * RQS; i += kT) {
                const int r = i / RQS, c = i - r * RQS;
                const int px = 2 * (qx0 - 2 + c), py = 2 * (qy0 - 2 + r);
                float v[4];
#pragma unroll
                for (int ch = 0; ch < 4; ch++) {  // the pixel of channel ch, clamped to the frame
                    const int gx = clampi(px + bayer_dx(BAYER, ch), 0, a.w - 1);
                    const int gy = clampi(py + bayer_dy(BAYER, ch), 0, a.h - 1);
                    v[ch] = Storage<S>::round(
                        scale_value(__ldg(a.raw + (size_t)gy * a.pitch + gx), a.sm[((gy & 1) << 1) | (gx & 1)], a.black));
                }
                s_q[i] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
        __syncthreads();
        // the next tile's pixels stream into the other buffer while this one is summed
        const int tn = t + gridDim.x;
        pending = tn < ntiles && by_tma(tn);
        if (pending && threadIdx.x == 0) issue(tn, buf ^ 1);
        // window sums of quads (qx0 + col, qy0 + row0 + j), j = 0..3
        float2 s01[4], q01[4], s23[4], q23[4];
#pragma unroll
        for (int j = 0; j < 4; j++) s01[j] = q01[j] = s23[j] = q23[j] = f2(0.0f, 0.0f);
#pragma unroll
        for (int rr = 0; rr < 8; rr++) {
#pragma unroll
            for (int dx = 0; dx < 5; dx++) {
                const float4 v = s_q[(row0 + rr) * RQS + col + dx];
                const float2 a01 = f2(v.x, v.y), a23 = f2(v.z, v.w);
                const float2 p01 = mul2s(a01, a01), p23 = mul2s(a23, a23);  // summed: scalar multiplies
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (rr - j >= 0 && rr - j <= 4) {
                        s01[j] = add2(s01[j], a01);
                        q01[j] = add2(q01[j], p01);
                        s23[j] = add2(s23[j], a23);
                        q23[j] = add2(q23[j], p23);
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int qx = qx0 + col, qy = qy0 + row0 + j;
            if (qx < qw && qy < qh) {
                // mean = sum / 25, var = (sq - sum^2 / 25) / 25 (demosaic.cl:1288-1324)
                float2 m[2], v[2];
                const float2 sp[2] = {s01[j], s23[j]}, qp[2] = {q01[j], q23[j]};
#pragma unroll
                for (int p = 0; p < 2; p++) {
                    if (a.sums_exact) {
                        m[p] = div25_x2<false>(sp[p]);
                        v[p] = div25_x2<true>(sub2(qp[p], div25_x2<false>(mul2(sp[p], sp[p]))));
                    } else {
                        m[p] = div25_x2<true>(sp[p]);
                        v[p] = div25_x2<true>(sub2(qp[p], div25_x2<true>(mul2(sp[p], sp[p]))));
                    }
                }
                if (a.stats_half) {  // the statistics as the reference's fp16 build stores them
#pragma unroll
                    for (int p = 0; p < 2; p++) {
                        m[p] = __half22float2(__float22half2_rn(m[p]));
                        v[p] = __half22float2(__float22half2_rn(v[p]));
                    }
                }
                const float mm[4] = {m[0].x, m[0].y, m[1].x, m[1].y}, vv[4] = {v[0].x, v[0].y, v[1].x, v[1].y};
                if (in_range<4, 4>(mm, vv, a.th)) acc.add_selected(m, v);
            }
        }
        // the staged pixels were read before this iteration's first barrier; s_q until here
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
    }
    Pass1Acc<4, 4> out;
    acc.unpack(out);
    pass1_epilogue<4, 4>(out, a.nlf, a.nlf_out);
}

// =========================================================================================
// demosaic: TW x TH output tile (44 x 28), 256 threads, 5 resident blocks per SM.
// =========================================================================================
// Shared memory of a demosaic tile and the blocks per SM it allows (at most 5: 48 registers)
constexpr int demosaic_smem(int TW, int TH) {
    return (TW + 10) * (TH + 10) * 4 + (TW + 4) * (TH + 4) * 4 + (TW + 8) * (TH + 8) * 16;
}
constexpr int demosaic_min_blocks(int TW, int TH) {
    return (228 * 1024) / (demosaic_smem(TW, TH) + 1024) < 5 ? (228 * 1024) / (demosaic_smem(TW, TH) + 1024) : 5;
}

template <int TW, int TH, bool RAW_U16, class S, bool CNNIN>
__global__ void __launch_bounds__(kT, demosaic_min_blocks(TW, TH)) demosaic_kernel(DemosaicArgs a) {
    constexpr int RW = TW + 10, RH = TH + 10;  // scaled raw, origin (x0 - 5, y0 - 5)
    constexpr int SW = TW + 8, SH = TH + 8;    // Sobel map, origin (x0 - 4, y0 - 4)
    constexpr int GW = TW + 4, GH = TH + 4;    // green, origin (x0 - 2, y0 - 2)
    constexpr int CW = TW + 2, CH = TH + 2;    // YCbCr (binary16), origin (x0 - 1, y0 - 1)
    static_assert(CW * CH * 8 <= SW * SH * 16, "YCbCr tile must fit in the Sobel map space");
    static_assert(GW % 2 == 0, "green region pairs");
    __shared__ float s_raw[RH * RW];
    __shared__ float s_green[GH * GW];
    __shared__ float4 s_sob[SH * SW];
    half4* s_ycc = reinterpret_cast<half4*>(s_sob);

    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int w = a.w, h = a.h, bayer = a.bayer;
    const int tid = threadIdx.x;
    const bool border = x0 - 5 < 0 || y0 - 5 < 0 || x0 + TW + 5 > w || y0 + TH + 5 > h;

    // 1. scaled raw tile: an interior tile whose rows start aligned reads words of 4 pixels
    // (uint16 raw: 8 bytes; the scaled raw in the storage precision: a float4 or half4), TW + 16
    // a row from x0 - 8 (TW and so x0 are multiples of 4), the pixels outside the staged
    // region skipped; other tiles read pixel by pixel, clamped to the frame
    typedef typename Storage<S>::T4 T4;
    constexpr int WPR = (TW + 16) / 4;
    static_assert(TW % 4 == 0, "tile columns in words of 4 pixels");
    const bool words = x0 >= 8 && x0 + TW + 8 <= w && y0 >= 5 && y0 + TH + 5 <= h && (a.in_pitch & 3) == 0 &&
                       (reinterpret_cast<uintptr_t>(a.in) & (uintptr_t)(RAW_U16 ? 7 : sizeof(T4) - 1)) == 0;
    if (words) {
        for (int i = tid; i < RH * WPR; i += kT) {
            const int r = i / WPR, q = i - r * WPR;
            float v[4];
            if (RAW_U16) {
                const uint16_t* row = (const uint16_t*)a.in + (size_t)(y0 - 5 + r) * a.in_pitch + (x0 - 8);
                const uint2 u = __ldg(reinterpret_cast<const uint2*>(row) + q);
                const int py = (y0 - 5 + r) & 1;
                const float s0 = a.sm[py << 1], s1 = a.sm[(py << 1) | 1];  // even and odd columns
                v[0] = Storage<S>::round(scale_value((uint16_t)(u.x & 0xffffu), s0, a.black));
                v[1] = Storage<S>::round(scale_value((uint16_t)(u.x >> 16), s1, a.black));
                v[2] = Storage<S>::round(scale_value((uint16_t)(u.y & 0xffffu), s0, a.black));
                v[3] = Storage<S>::round(scale_value((uint16_t)(u.y >> 16), s1, a.black));
            } else {
                const S* row = (const S*)a.in + (size_t)(y0 - 5 + r) * a.in_pitch + (x0 - 8);
                const float4 f = Storage<S>::ldg4(reinterpret_cast<const T4*>(row) + q);
                v[0] = f.x;
                v[1] = f.y;
                v[2] = f.z;
                v[3] = f.w;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int c = 4 * q + k - 3;  // staged column of pixel x0 - 8 + 4q + k
                if (c >= 0 && c < RW) s_raw[r * RW + c] = v[k];
            }
        }
    } else {
        for (int i = tid; i < RH * RW; i += kT) {
            const int r = i / RW, c = i - r * RW;
            const int gx = clampi(x0 - 5 + c, 0, w - 1), gy = clampi(y0 - 5 + r, 0, h - 1);
            float v;
            if (RAW_U16) {
                v = Storage<S>::round(scale_value(__ldg((const uint16_t*)a.in + (size_t)gy * a.in_pitch + gx),
                                                  a.sm[((gy & 1) << 1) | (gx & 1)], a.black));
            } else {
                v = Storage<S>::ldg((const S*)a.in + (size_t)gy * a.in_pitch + gx);
            }
            s_raw[i] = v;
        }
    }
    __syncthreads();
    const SAcc1 R{s_raw, x0 - 5, y0 - 5, RW};

    // 2. Sobel map (|gx|, |gy|, length) at every position a bilateralSobel may visit
    for (int i = tid; i < SH * SW; i += kT) {
        const int r = i / SW, c = i - r * SW;
        const SobelVal sv = sobel_abs<true>(R, x0 - 4 + c, y0 - 4 + r);  // finite scaled raw
        s_sob[i] = make_float4(sv.gx, sv.gy, sv.len, 0.0f);
    }
    if (a.tap_scaled) {
        for (int i = tid; i < TW * TH; i += kT) {
            const int r = i / TW, c = i - r * TW, x = x0 + c, y = y0 + r;
            if (x < w && y < h) a.tap_scaled[(size_t)y * a.tap_pitch + x] = R.at(x, y);
        }
    }
    __syncthreads();

    // 3. green at every in-frame position of the green region; pairs of pixels hold one
    //    red/blue site and one green site, so the work is even across threads
    {
        const float lv = mmax(a.rawB_dev ? a.rawB_dev[1] : a.lv_host, 1e-4f);
        for (int p = tid; p < GH * GW / 2; p += kT) {
            const int r = p / (GW / 2), k = p - r * (GW / 2);
            const int y = y0 - 2 + r;
            const int xa = x0 - 2 + 2 * k;
            // every thread interpolates the red/blue site of its pair at the same time
            const int e_rb = green_needs_interp(xa, y, bayer) ? 0 : 1;
            const int xr = xa + e_rb, xg = xa + (1 - e_rb);
            const bool yin = y >= 0 && y < h;
            if (yin && xr >= 0 && xr < w) {
                const SobelMap sob{s_sob, x0 - 4, y0 - 4, SW, xr, y};
                s_green[r * GW + 2 * k + e_rb] = Storage<S>::round(green_at(R, xr, y, lv, sob));
            }
            if (yin && xg >= 0 && xg < w) s_green[r * GW + 2 * k + 1 - e_rb] = Storage<S>::round(R.at(xg, y));
        }
    }
    __syncthreads();
    if (border) {  // out-of-frame green reads clamp to the frame
        for (int i = tid; i < GH * GW; i += kT) {
            const int r = i / GW, c = i - r * GW, x = x0 - 2 + c, y = y0 - 2 + r;
            if (x >= 0 && x < w && y >= 0 && y < h) continue;
            const int cx = clampi(x, 0, w - 1) - (x0 - 2), cy = clampi(y, 0, h - 1) - (y0 - 2);
            s_green[i] = s_green[cy * GW + cx];
        }
        __syncthreads();
    }
    const SAcc1 G{s_green, x0 - 2, y0 - 2, GW};

    if (CNNIN) {  // the learned stage's input: red/blue at the tile, and the noise sigma
        const float cv = mmax(a.rawB_dev ? div_(a.rawB_dev[0] + a.rawB_dev[2], 2.0f) : a.cv_host, 1e-6f);
        for (int i = tid; i < TW * TH; i += kT) {
            const int r = i / TW, c = i - r * TW, x = x0 + c, y = y0 + r;
            if (x >= w || y >= h) continue;
            const float3 p = round3<S>(red_blue_at(R, G, x, y, bayer, cv));
            const float sig = sqrt_(mmax(a.rawA_dev[1] + a.rawB_dev[1] * p.y, 1e-8f));
            reinterpret_cast<float4*>(a.cnn_in)[(size_t)y * w + x] = make_float4(p.x, p.y, p.z, sig);
        }
        return;
    }

    // 4. red/blue, highlight recovery, camera -> YCbCr (the Sobel map is dead: reuse it)
    {
        const float cv = mmax(a.rawB_dev ? div_(a.rawB_dev[0] + a.rawB_dev[2], 2.0f) : a.cv_host, 1e-6f);
        for (int i = tid; i < CH * CW; i += kT) {
            const int r = i / CW, c = i - r * CW, x = x0 - 1 + c, y = y0 - 1 + r;
            if (x < 0 || x >= w || y < 0 || y >= h) continue;
            float3 p = round3<S>(red_blue_at(R, G, x, y, bayer, cv));
            p = round3<S>(blend_highlights_px(p, 1.0f));
            p = round3<S>(transform_px(a.cam_ycbcr, p));
            s_ycc[i] = to_half4(make_float4(p.x, p.y, p.z, 0.0f));
        }
    }
    if (a.tap_green) {
        for (int i = tid; i < TW * TH; i += kT) {
            const int r = i / TW, c = i - r * TW, x = x0 + c, y = y0 + r;
            if (x < w && y < h) a.tap_green[(size_t)y * a.tap_pitch + x] = G.at(x, y);
        }
    }
    __syncthreads();
    if (border) {
        for (int i = tid; i < CH * CW; i += kT) {
            const int r = i / CW, c = i - r * CW, x = x0 - 1 + c, y = y0 - 1 + r;
            if (x >= 0 && x < w && y >= 0 && y < h) continue;
            const int cx = clampi(x, 0, w - 1) - (x0 - 1), cy = clampi(y, 0, h - 1) - (y0 - 1);
            s_ycc[i] = s_ycc[cy * CW + cx];
        }
        __syncthreads();
    }

    // 5. luma despeckle / chroma median -> level 0
    const SAcc4h Y{s_ycc, x0 - 1, y0 - 1, CW};
    for (int i = tid; i < TW * TH; i += kT) {
        const int r = i / TW, c = i - r * TW, x = x0 + c, y = y0 + r;
        if (x >= w || y >= h) continue;
        a.level0[(size_t)y * a.l0_pitch + x] = to_half4(despeckle_px<true>(Y, x, y, a.va0, a.vb0));
    }
}

// =========================================================================================
// The split demosaic (a tile shape of the tuner): the green of every red/blue site computed
// once by its own kernel (no halo of green recomputed: the fused kernel interpolates 1.25x
// its tile's sites and evaluates its Sobel map over 1.52x its tile), written to the green
// image in the storage precision -- where the fused kernel keeps it in shared memory, rounded
// the same way -- then red/blue, highlights, cam -> YCbCr and the despeckle by a second
// kernel reading that image (clamped to the frame, as the fused kernel's border copies do).
// =========================================================================================
constexpr int SGW = 64, SGH = 32;  // green kernel tile

template <bool RAW_U16, class S>
__global__ void __launch_bounds__(kT, 4) green_split_kernel(DemosaicArgs a) {
    constexpr int RW = SGW + 6, RH = SGH + 6;  // scaled raw, origin (x0 - 3, y0 - 3)
    constexpr int SW = SGW + 4, SH = SGH + 4;  // Sobel map, origin (x0 - 2, y0 - 2)
    __shared__ float s_raw[RH * RW];
    __shared__ float4 s_sob[SH * SW];
    const int x0 = blockIdx.x * SGW, y0 = blockIdx.y * SGH;
    const int w = a.w, h = a.h, bayer = a.bayer;
    // An interior tile of uint16 raw whose rows start 8-byte aligned reads its region as
    // 8-byte words: 72 pixels a row from x0 - 4 (x0 is a multiple of 64), one word per thread
    // step, the first and last pixel of a row outside the staged 70; other tiles read pixel
    // by pixel with the frame's edges clamped.
    const bool words = RAW_U16 && x0 >= 4 && x0 + SGW + 4 <= w && y0 >= 3 && y0 + SGH + 3 <= h &&
                       (reinterpret_cast<uintptr_t>(a.in) & 7u) == 0 && (a.in_pitch & 3) == 0;
    if (words) {
        constexpr int WPR = (RW + 2) / 4;  // words per row: 18
        const uint16_t* base = (const uint16_t*)a.in + (size_t)(y0 - 3) * a.in_pitch + (x0 - 4);
        for (int i = threadIdx.x; i < RH * WPR; i += kT) {
            const int r = i / WPR, q = i - r * WPR;
            const uint2 u = __ldg(reinterpret_cast<const uint2*>(base + (size_t)r * a.in_pitch) + q);
            const int py = (y0 - 3 + r) & 1;
            const float s0 = a.sm[py << 1], s1 = a.sm[(py << 1) | 1];  // even and odd columns
            const uint16_t px[4] = {(uint16_t)(u.x & 0xffffu), (uint16_t)(u.x >> 16), (uint16_t)(u.y & 0xffffu),
                                    (uint16_t)(u.y >> 16)};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int c = 4 * q + k - 1;  // staged column of pixel x0 - 4 + 4q + k
                if (c >= 0 && c < RW) s_raw[r * RW + c] = Storage<S>::round(scale_value(px[k], (k & 1) ? s1 : s0, a.black));
            }
        }
    } else {
        for (int i = threadIdx.x; i < RH * RW; i += kT) {
            const int r = i / RW, c = i - r * RW;
            const int gx = clampi(x0 - 3 + c, 0, w - 1), gy = clampi(y0 - 3 + r, 0, h - 1);
            float v;
            if (RAW_U16) {
                v = Storage<S>::round(scale_value(__ldg((const uint16_t*)a.in + (size_t)gy * a.in_pitch + gx),
                                                  a.sm[((gy & 1) << 1) | (gx & 1)], a.black));
            } else {
                v = Storage<S>::ldg((const S*)a.in + (size_t)gy * a.in_pitch + gx);
            }
            s_raw[i] = v;
        }
    }
    __syncthreads();
    const SAcc1 R{s_raw, x0 - 3, y0 - 3, RW};
    for (int i = threadIdx.x; i < SH * SW; i += kT) {
        const int r = i / SW, c = i - r * SW;
        const SobelVal sv = sobel_abs<true>(R, x0 - 2 + c, y0 - 2 + r);  // finite scaled raw
        s_sob[i] = make_float4(sv.gx, sv.gy, sv.len, 0.0f);
    }
    __syncthreads();
    const float lv = mmax(a.rawB_dev ? a.rawB_dev[1] : a.lv_host, 1e-4f);
    S* const green = (S*)a.green;
    for (int p = threadIdx.x; p < SGW * SGH / 2; p += kT) {
        const int r = p / (SGW / 2), k = p - r * (SGW / 2);
        const int y = y0 + r, xa = x0 + 2 * k;
        if (y >= h) continue;
        const int e_rb = green_needs_interp(xa, y, bayer) ? 0 : 1;
        const int xr = xa + e_rb, xg = xa + (1 - e_rb);
        if (xr < w) {
            const SobelMap sob{s_sob, x0 - 2, y0 - 2, SW, xr, y};
            const float g = Storage<S>::round(green_at(R, xr, y, lv, sob));
            Storage<S>::st(green + (size_t)y * a.green_pitch + xr, g);
            if (a.tap_green) a.tap_green[(size_t)y * a.tap_pitch + xr] = g;
        }
        if (xg < w) {
            const float g = Storage<S>::round(R.at(xg, y));
            Storage<S>::st(green + (size_t)y * a.green_pitch + xg, g);
            if (a.tap_green) a.tap_green[(size_t)y * a.tap_pitch + xg] = g;
        }
    }
    if (a.tap_scaled) {
        for (int i = threadIdx.x; i < SGW * SGH; i += kT) {
            const int r = i / SGW, c = i - r * SGW, x = x0 + c, y = y0 + r;
            if (x < w && y < h) a.tap_scaled[(size_t)y * a.tap_pitch + x] = R.at(x, y);
        }
    }
}

template <bool RAW_U16, class S>
__global__ void __launch_bounds__(kT, 5) rb_despeckle_kernel(DemosaicArgs a) {
    constexpr int TW = 44, TH = 28;
    constexpr int RW = TW + 4, RH = TH + 4;  // scaled raw and green, origin (x0 - 2, y0 - 2)
    constexpr int CW = TW + 2, CH = TH + 2;  // YCbCr (binary16), origin (x0 - 1, y0 - 1)
    __shared__ float s_raw[RH * RW];
    __shared__ float s_green[RH * RW];
    __shared__ half4 s_ycc[CH * CW];
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int w = a.w, h = a.h, bayer = a.bayer;
    const bool border = x0 - 2 < 0 || y0 - 2 < 0 || x0 + TW + 2 > w || y0 + TH + 2 > h;
    const S* const green = (const S*)a.green;
    typedef typename Storage<S>::T4 T4;
    // An interior tile of uint16 raw whose raw and green rows start aligned reads both regions
    // as words of 4 pixels: 52 a row from x0 - 4 (x0 is a multiple of 44, so of 4), the two
    // pixels each side outside the staged 48; other tiles read pixel by pixel, clamped.
    const bool words = RAW_U16 && x0 >= 4 && x0 + TW + 4 <= w && y0 >= 2 && y0 + TH + 2 <= h &&
                       (reinterpret_cast<uintptr_t>(a.in) & 7u) == 0 && (a.in_pitch & 3) == 0 &&
                       (reinterpret_cast<uintptr_t>(green) & (sizeof(T4) - 1)) == 0 && (a.green_pitch & 3) == 0;
    if (words) {
        constexpr int WPR = (RW + 4) / 4;  // words per row: 13
        const uint16_t* rbase = (const uint16_t*)a.in + (size_t)(y0 - 2) * a.in_pitch + (x0 - 4);
        const S* gbase = green + (size_t)(y0 - 2) * a.green_pitch + (x0 - 4);
        for (int i = threadIdx.x; i < RH * WPR; i += kT) {
            const int r = i / WPR, q = i - r * WPR;
            const uint2 u = __ldg(reinterpret_cast<const uint2*>(rbase + (size_t)r * a.in_pitch) + q);
            const float4 g4 = Storage<S>::ldg4(reinterpret_cast<const T4*>(gbase + (size_t)r * a.green_pitch) + q);
            const int py = (y0 - 2 + r) & 1;
            const float s0 = a.sm[py << 1], s1 = a.sm[(py << 1) | 1];  // even and odd columns
            const uint16_t px[4] = {(uint16_t)(u.x & 0xffffu), (uint16_t)(u.x >> 16), (uint16_t)(u.y & 0xffffu),
                                    (uint16_t)(u.y >> 16)};
            const float gv[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int c = 4 * q + k - 2;  // staged column of pixel x0 - 4 + 4q + k
                if (c >= 0 && c < RW) {
                    s_raw[r * RW + c] = Storage<S>::round(scale_value(px[k], (k & 1) ? s1 : s0, a.black));
                    s_green[r * RW + c] = gv[k];
                }
            }
        }
    } else {
        for (int i = threadIdx.x; i < RH * RW; i += kT) {
            const int r = i / RW, c = i - r * RW;
            const int gx = clampi(x0 - 2 + c, 0, w - 1), gy = clampi(y0 - 2 + r, 0, h - 1);
            float v;
            if (RAW_U16) {
                v = Storage<S>::round(scale_value(__ldg((const uint16_t*)a.in + (size_t)gy * a.in_pitch + gx),
                                                  a.sm[((gy & 1) << 1) | (gx & 1)], a.black));
            } else {
                v = Storage<S>::ldg((const S*)a.in + (size_t)gy * a.in_pitch + gx);
            }
            s_raw[i] = v;
            s_green[i] = Storage<S>::ldg(green + (size_t)gy * a.green_pitch + gx);
        }
    }
    __syncthreads();
    const SAcc1 R{s_raw, x0 - 2, y0 - 2, RW};
    const SAcc1 G{s_green, x0 - 2, y0 - 2, RW};
    {
        const float cv = mmax(a.rawB_dev ? div_(a.rawB_dev[0] + a.rawB_dev[2], 2.0f) : a.cv_host, 1e-6f);
        for (int i = threadIdx.x; i < CH * CW; i += kT) {
            const int r = i / CW, c = i - r * CW, x = x0 - 1 + c, y = y0 - 1 + r;
            if (x < 0 || x >= w || y < 0 || y >= h) continue;
            float3 p = round3<S>(red_blue_at(R, G, x, y, bayer, cv));
            p = round3<S>(blend_highlights_px(p, 1.0f));
            p = round3<S>(transform_px(a.cam_ycbcr, p));
            s_ycc[i] = to_half4(make_float4(p.x, p.y, p.z, 0.0f));
        }
    }
    __syncthreads();
    if (border) {
        for (int i = threadIdx.x; i < CH * CW; i += kT) {
            const int r = i / CW, c = i - r * CW, x = x0 - 1 + c, y = y0 - 1 + r;
            if (x >= 0 && x < w && y >= 0 && y < h) continue;
            const int cx = clampi(x, 0, w - 1) - (x0 - 1), cy = clampi(y, 0, h - 1) - (y0 - 1);
            s_ycc[i] = s_ycc[cy * CW + cx];
        }
        __syncthreads();
    }
    const SAcc4h Y{s_ycc, x0 - 1, y0 - 1, CW};
    for (int i = threadIdx.x; i < TW * TH; i += kT) {
        const int r = i / TW, c = i - r * TW, x = x0 + c, y = y0 + r;
        if (x >= w || y >= h) continue;
        a.level0[(size_t)y * a.l0_pitch + x] = to_half4(despeckle_px<true>(Y, x, y, a.va0, a.vb0));
    }
}

// =========================================================================================
// post_cnn: the learned stage's residual (its RGB output times the pixel's sigma) added to
// the linear RGB, then blendHighlights,
// cam -> YCbCr over the tile and a one-pixel ring (clamped reads: the same values the
// fused kernel's border replication gives), despeckle -> level 0, and the level-0
// noise-model multiplier.  A residual that is exactly zero leaves the value as it is (also
// a -0), so a network with all-zero parameters reproduces the plain pipeline bit for bit.
// =========================================================================================
constexpr int PCW = 32, PCH = 8;

template <class S>
__global__ void __launch_bounds__(kT) post_cnn_kernel(PostCnnArgs a) {
    constexpr int CW = PCW + 2, CH = PCH + 2;
    __shared__ half4 s_ycc[CW * CH];
    const int x0 = blockIdx.x * PCW, y0 = blockIdx.y * PCH;
    for (int i = threadIdx.x; i < CW * CH; i += kT) {
        const int r = i / CW, c = i - r * CW;
        const int x = clampi(x0 - 1 + c, 0, a.w - 1), y = clampi(y0 - 1 + r, 0, a.h - 1);
        const size_t px = (size_t)y * a.w + x;
        const float4 lin = reinterpret_cast<const float4*>(a.cnn_in)[px];
        const float4 o = reinterpret_cast<const float4*>(a.head)[px];
        const float rx = lin.w * o.y, ry = lin.w * o.z, rz = lin.w * o.w;  // residual = sigma * output
        float3 p = make_float3(rx == 0.0f ? lin.x : lin.x + rx, ry == 0.0f ? lin.y : lin.y + ry,
                               rz == 0.0f ? lin.z : lin.z + rz);
        p = round3<S>(p);
        p = round3<S>(blend_highlights_px(p, 1.0f));
        p = round3<S>(transform_px(a.cam_ycbcr, p));
        s_ycc[i] = to_half4(make_float4(p.x, p.y, p.z, 0.0f));
    }
    __syncthreads();
    const SAcc4h Y{s_ycc, x0 - 1, y0 - 1, CW};
    for (int i = threadIdx.x; i < PCW * PCH; i += kT) {
        const int r = i / PCW, c = i - r * PCW, x = x0 + c, y = y0 + r;
        if (x >= a.w || y >= a.h) continue;
        a.level0[(size_t)y * a.l0_pitch + x] = to_half4(despeckle_px<true>(Y, x, y, a.va0, a.vb0));
        const float lg = a.head[((size_t)y * a.w + x) * 4];
        a.strength[(size_t)y * a.w + x] = 2.0f * div_(1.0f, 1.0f + glsm::exp2_(-lg * 1.44269504f));
    }
}

// =========================================================================================
// level_pass1: noiseStatistics + pass-1 sums of level i, and downsampleImage to level i+1.
// Persistent blocks walk 32x32 tiles; each thread owns a column of 4 pixels and reuses
// the loaded rows across them (each output still sums its 5x5 window in the reference's
// row-major order).
//
// Staging: the 36x36 input region of a tile is double-buffered.  Where the region lies inside
// the image, one thread brings it in with a TMA tensor copy (cp.async.bulk.tensor) while the
// block sums the previous tile, completing on an mbarrier; at the image's edges (clamped
// reads) the block loads it itself.  A binary16 level is widened into a third buffer once
// it has landed.
// =========================================================================================
constexpr int LT = 32;
constexpr int LP = LT + 4;
// downsampleImage's taps for a tile's 16 output columns and rows ([0] at -0.5 output pixel, [1]
// at +0.5: downsample_px's px -+ sx), relative to the staged region; threads 0..63 of the block
// (the same float operations as downsample_px's coordinates and tap1, once per column and row)
GLS_DI void level_tables(int x0, int y0, int w, int h, int ow, int oh, TabTap (*s_tx)[LT / 2], TabTap (*s_ty)[LT / 2]) {
    if (threadIdx.x >= 2 * LT) return;
    const int e = threadIdx.x & (LT - 1), k = e >> 4, o = e & 15;
    if (threadIdx.x < LT) {
        const float n = div_(1.0f, (float)ow);
        const float pc = ((float)(x0 / 2 + o) + 0.5f) * n, sh = 0.5f * n;
        s_tx[k][o] = tab_tap(tap1(k ? pc + sh : pc + -sh, w), w, x0 - 2, LP, 1);
    } else {
        const float n = div_(1.0f, (float)oh);
        const float pc = ((float)(y0 / 2 + o) + 0.5f) * n, sh = 0.5f * n;
        s_ty[k][o] = tab_tap(tap1(k ? pc + sh : pc + -sh, h), h, y0 - 2, LP, LP);
    }
}

// One 32x32 tile from its staged 36x36 region (fp32, origin (x0 - 2, y0 - 2)): the
// noiseStatistics of its pixels added to acc, and its 16x16 downsampled block written to out
// (when out is not null).
template <class SOut>
GLS_DI void level_tile(const float4* s_in, const TabTap (*s_tx)[LT / 2], const TabTap (*s_ty)[LT / 2], int x0, int y0,
                       int w, int h, void* out, int ow, int oh, int opitch, const NlfThresholds& th, int stats_half,
                       LevelPass1Acc2& acc) {
    const int col = threadIdx.x & 31, row0 = (threadIdx.x >> 5) * 4;
    // window sums for pixels (x0 + col, y0 + row0 + j), j = 0..3: (s0, s1), (q0, q1) and
    // (s2, q2) as packed pairs, every window summed in the reference's row-major order
    float2 s01[4], q01[4], s2q2[4];
#pragma unroll
    for (int j = 0; j < 4; j++) s01[j] = q01[j] = s2q2[j] = f2(0.0f, 0.0f);
#pragma unroll
    for (int rr = 0; rr < 8; rr++) {
#pragma unroll
        for (int dx = 0; dx < 5; dx++) {
            const float4 v = s_in[(row0 + rr) * LP + col + dx];
            const float2 a01 = f2(v.x, v.y);
            const float2 p01 = mul2s(a01, a01);  // summed: scalar multiplies
            const float2 z = f2(v.z, __fmul_rn(v.z, v.z));
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (rr - j >= 0 && rr - j <= 4) {
                    s01[j] = add2(s01[j], a01);
                    q01[j] = add2(q01[j], p01);
                    s2q2[j] = add2(s2q2[j], z);
                }
            }
        }
    }
    const FastDiv d25 = div25();
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + col, y = y0 + row0 + j;
        if (x < w && y < h) {
            // noiseStatistics (demosaic.cl:1267-1286): mean Y = s0 / 25, var_k = (q_k - s_k^2 / 25) / 25
            const float2 mt = div25_x2<true>(f2(s01[j].x, s2q2[j].x * s2q2[j].x));  // (mean Y, s2^2 / 25)
            float2 v01 = div25_x2<true>(sub2(q01[j], div25_x2<true>(mul2(s01[j], s01[j]))));
            float v2 = d25(s2q2[j].y - mt.y), my = mt.x;
            if (stats_half) {  // the statistics as the reference's fp16 build stores them
                v01 = __half22float2(__float22half2_rn(v01));
                v2 = glsm::round_half(v2);
                my = glsm::round_half(my);
            }
            const float m[1] = {my}, v[3] = {v01.x, v01.y, v2};
            if (in_range<1, 3>(m, v, th)) acc.add_selected(my, v01, v2);
        }
    }
    // downsample: the coarse 16x16 block under this tile, from the staged region through the
    // tap tables (downsample_px's samples and their average, bit for bit)
    if (out) {
        const int oc = threadIdx.x & 15, orow = threadIdx.x >> 4;
        const int ox = x0 / 2 + oc, oy = y0 / 2 + orow;
        if (ox < ow && oy < oh) {
            const float4 t0 = tab_sample4(s_in, s_tx[0][oc], s_ty[0][orow]);
            const float4 t1 = tab_sample4(s_in, s_tx[1][oc], s_ty[0][orow]);
            const float4 t2 = tab_sample4(s_in, s_tx[0][oc], s_ty[1][orow]);
            const float4 t3 = tab_sample4(s_in, s_tx[1][oc], s_ty[1][orow]);
            // 0.25 (t0 + t1 + t2 + t3) per channel, the channel pairs packed
            const float2 q = f2(0.25f, 0.25f);
            const float2 xy = mul2(q, add2(add2(add2(f2(t0.x, t0.y), f2(t1.x, t1.y)), f2(t2.x, t2.y)), f2(t3.x, t3.y)));
            const float2 zw = mul2(q, add2(add2(add2(f2(t0.z, t0.w), f2(t1.z, t1.w)), f2(t2.z, t2.w)), f2(t3.z, t3.w)));
            const float4 d = make_float4(xy.x, xy.y, zw.x, zw.y);
            typedef typename Storage<SOut>::T4 TOut;
            Storage<SOut>::st4((TOut*)out + (size_t)oy * opitch + ox, d);
        }
    }
}

template <class SIn, class SOut>
__global__ void __launch_bounds__(kT, 3) level_pass1_kernel(LevelPass1Args a, const __grid_constant__ CUtensorMap tmap) {
    typedef typename Storage<SIn>::T4 TIn;
    constexpr bool HALF_IN = sizeof(TIn) == 8;
    constexpr uint32_t kStageBytes = LP * LP * sizeof(TIn);
    __shared__ __align__(128) TIn s_stage[2][LP * LP];  // the tile's region as stored
    __shared__ __align__(16) float4 s_wide[HALF_IN ? LP * LP : 1];  // a binary16 region widened
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ TabTap s_tx[2][LT / 2], s_ty[2][LT / 2];  // downsampleImage's taps (level_tables)
    LevelPass1Acc2 acc;
    acc.init();
    const TIn* in = (const TIn*)a.in;
    const int tiles_x = (a.w + LT - 1) / LT, tiles_y = (a.h + LT - 1) / LT, ntiles = tiles_x * tiles_y;
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&s_bar[0]);
    const uint32_t stage0 = (uint32_t)__cvta_generic_to_shared(&s_stage[0][0]);
    if (threadIdx.x == 0 && a.tma) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    // a tile's region by TMA when it lies inside the image (x in 8-byte units: even)
    auto by_tma = [&](int t) {
        const int x0 = (t % tiles_x) * LT, y0 = (t / tiles_x) * LT;
        return a.tma && x0 >= 2 && y0 >= 2 && x0 + LT + 2 <= a.w && y0 + LT + 2 <= a.h;
    };
    auto issue = [&](int t, int b) {  // thread 0
        const int x0 = (t % tiles_x) * LT, y0 = (t / tiles_x) * LT;
        tma_issue_2d(stage0 + (uint32_t)b * kStageBytes, &tmap, (x0 - 2) * (int)(sizeof(TIn) / 8), y0 - 2,
                     bar0 + 8u * (uint32_t)b, kStageBytes);
    };
    uint32_t parity = 0;  // bit b: the phase of barrier b to wait for next
    bool pending = false;  // this iteration's buffer is being filled by TMA
    int buf = 0;
    int t = blockIdx.x;
    if (t < ntiles && by_tma(t)) {
        if (threadIdx.x == 0) issue(t, 0);
        pending = true;
    }
    for (; t < ntiles; t += gridDim.x, buf ^= 1) {
        const int x0 = (t % tiles_x) * LT, y0 = (t / tiles_x) * LT;
        TIn* const stage = s_stage[buf];
        if (pending) {
            const uint32_t par = (parity >> buf) & 1u;
            parity ^= 1u << buf;
            if (!stage_wait(bar0 + 8u * (uint32_t)buf, par, kStageWaitPolls)) {
                // the copy did not complete: record it, give it one more bounded wait, and
                // leave the tile loop (the sums so far still reach the totals, so the
                // regression's ticket stays consistent)
                if (threadIdx.x == 0) atomicOr(a.nlf.err, 1u);
                stage_wait(bar0 + 8u * (uint32_t)buf, par, kStageWaitPolls);
                break;
            }
        } else {
            for (int i = threadIdx.x; i < LP * LP; i += kT) {
                const int r = i / LP, c = i - r * LP;
                const int gx = clampi(x0 - 2 + c, 0, a.w - 1), gy = clampi(y0 - 2 + r, 0, a.h - 1);
                stage[i] = in[(size_t)gy * a.pitch + gx];
            }
        }
        if (a.out) level_tables(x0, y0, a.w, a.h, a.ow, a.oh, s_tx, s_ty);
        __syncthreads();
        if constexpr (HALF_IN) {
            for (int i = threadIdx.x; i < LP * LP; i += kT) s_wide[i] = Storage<__half>::cvt(stage[i]);
            __syncthreads();
        }
        const float4* const s_in = HALF_IN ? s_wide : reinterpret_cast<const float4*>(stage);
        // the next tile's region streams into the other buffer while this one is summed (its
        // previous contents were consumed before the barrier that ended the last iteration)
        const int tn = t + gridDim.x;
        pending = tn < ntiles && by_tma(tn);
        if (pending && threadIdx.x == 0) issue(tn, buf ^ 1);
        level_tile<SOut>(s_in, s_tx, s_ty, x0, y0, a.w, a.h, a.out, a.ow, a.oh, a.opitch, a.th, a.stats_half, acc);
        // this tile's buffers may next be written by the async proxy (a TMA copy)
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
    }
    Pass1Acc<1, 3> out;
    acc.unpack(out);
    pass1_epilogue<1, 3>(out, a.nlf, a.nlf_out);
}

// =========================================================================================
// pyramid_stats: levels 1 .. L-1 of the pyramid (statistics, regression sums, downsample to
// the next level) in one launch.  Blocks take 32x32 tiles from a work queue ordered by level
// (an atomic counter); a tile of level p >= 2 first waits (bounded) for the tiles of level
// p - 1 whose downsampled blocks its 36x36 region reads, which were all taken from the queue
// before it by running blocks, so every wait ends.  A block keeps the sums of one level at a
// time and adds them to that level's totals when it moves to another level or leaves; the
// block whose addition completes a level's tile count solves that level's fit.  Level 1 was
// written by the previous launch and comes in by TMA (the next item's region while the
// current one is summed); the later levels are read through L2 (ld.global.cg).
// =========================================================================================
constexpr uint32_t kPyrWaitPolls = 1u << 20;  // bound of a dependency wait (polls of ~0.1-1 us)

GLS_DI unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// a pixel through L2 only (ld.global.cg): data written by other blocks of the same launch
GLS_DI float4 ld_cg(const float4* p) { return __ldcg(p); }
GLS_DI half4 ld_cg(const half4* p) {
    const uint2 u = __ldcg(reinterpret_cast<const uint2*>(p));
    half4 h;
    *reinterpret_cast<uint2*>(&h) = u;
    return h;
}
GLS_DI void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// The statistics kernels' two bounded waits run out on purpose: a mark that nothing sets
// (the pyramid's dependency wait) and an mbarrier that nothing arrives at and no copy
// targets (the TMA staging wait), so nothing is in flight when they give up; each records
// its bit in the error word exactly as the kernels do.
__global__ void __launch_bounds__(kT) stage_wait_probe_kernel(NlfScratch s, uint32_t polls) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const unsigned* word = reinterpret_cast<const unsigned*>(reinterpret_cast<const char*>(s.fit) + kNlfProbeOff);
    bool ok = true;
    if (threadIdx.x < 16) {
        uint32_t k = 0;
        while (ld_acquire_u32(word) != 1u && k < polls) {
            __nanosleep(64);
            k++;
        }
        ok = k < polls;
    }
    if (!__syncthreads_and(ok) && threadIdx.x == 0) atomicOr(s.err, 2u);
    if (!stage_wait(b, 0u, polls) && threadIdx.x == 0) atomicOr(s.err, 1u);
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(b) : "memory");
}

template <class S>
__global__ void __launch_bounds__(kT, 3) pyramid_stats_kernel(const __grid_constant__ PyramidArgs a,
                                                               const __grid_constant__ CUtensorMap tmap) {
    typedef typename Storage<S>::T4 T4;
    constexpr bool HALF = sizeof(T4) == 8;
    constexpr uint32_t kStageBytes = LP * LP * sizeof(T4);
    __shared__ __align__(128) T4 s_stage[2][LP * LP];
    __shared__ __align__(16) float4 s_wide[HALF ? LP * LP : 1];
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ TabTap s_tx[2][LT / 2], s_ty[2][LT / 2];
    __shared__ int s_item, s_flag;
    __shared__ unsigned s_mark;
    const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&s_bar[0]);
    const uint32_t stage0 = (uint32_t)__cvta_generic_to_shared(&s_stage[0][0]);
    if (threadIdx.x == 0) {
        if (a.tma) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        s_mark = ld_acquire_u32(&a.ctl->mark) + 1u;
        s_item = (int)atomicAdd(&a.ctl->queue, 1u);
    }
    __syncthreads();
    const unsigned mark = s_mark;
    auto level_of = [&](int item) {
        int p = 0;
        while (p + 1 < a.nlev && item >= a.lv[p + 1].first) p++;
        return p;
    };
    auto by_tma = [&](int item) {  // a level-1 tile inside the image
        if (!a.tma || item >= a.lv[0].count) return false;
        const PyrLevel& L = a.lv[0];
        const int x0 = (item % L.tiles_x) * LT, y0 = (item / L.tiles_x) * LT;
        return x0 >= 2 && y0 >= 2 && x0 + LT + 2 <= L.w && y0 + LT + 2 <= L.h;
    };
    auto issue = [&](int item, int b) {  // thread 0
        const int x0 = (item % a.lv[0].tiles_x) * LT, y0 = (item / a.lv[0].tiles_x) * LT;
        tma_issue_2d(stage0 + (uint32_t)b * kStageBytes, &tmap, (x0 - 2) * (int)(sizeof(T4) / 8), y0 - 2,
                     bar0 + 8u * (uint32_t)b, kStageBytes);
    };
    // this block's sums of level `cur` (over `ntiles` of its tiles) to that level's totals, and
    // the level's solve when they were the last
    LevelPass1Acc2 acc;
    acc.init();
    int cur = -1, ntiles = 0;
    auto flush = [&]() {
        const PyrLevel& L = a.lv[cur];
        Pass1Acc<1, 3> out;
        acc.unpack(out);
        out.write_fixed(L.nlf);
        out.write_minmax(L.nlf);
        if (threadIdx.x == 0) {
            __threadfence();
            s_flag = atomicAdd(&a.ctl->flushed[cur], (unsigned)ntiles) + (unsigned)ntiles == (unsigned)L.count;
        }
        __syncthreads();
        if (s_flag) {
            __threadfence();
            solve_fixed<3>(L.nlf, 1, L.nlf_out);
            if (threadIdx.x == 0) a.ctl->flushed[cur] = 0u;
        }
        __syncthreads();
        acc.init();
        ntiles = 0;
    };
    uint32_t parity = 0;
    int buf = 0;
    int item = s_item;
    bool pending = item < a.items && by_tma(item);
    if (pending && threadIdx.x == 0) issue(item, 0);
    bool failed = false;
    while (item < a.items) {
        const int p = level_of(item);
        const PyrLevel& L = a.lv[p];
        const int t = item - L.first;
        const int x0 = (t % L.tiles_x) * LT, y0 = (t / L.tiles_x) * LT;
        if (p != cur) {
            if (cur >= 0) flush();
            cur = p;
        }
        T4* const stage = s_stage[buf];
        if (pending) {
            const uint32_t par = (parity >> buf) & 1u;
            parity ^= 1u << buf;
            if (!stage_wait(bar0 + 8u * (uint32_t)buf, par, kStageWaitPolls)) {
                if (threadIdx.x == 0) atomicOr(L.nlf.err, 1u);
                stage_wait(bar0 + 8u * (uint32_t)buf, par, kStageWaitPolls);
                failed = true;
                break;
            }
        } else {
            if (p >= 1) {
                // the tiles of level p - 1 whose 16x16 downsampled blocks cover this region
                const PyrLevel& P = a.lv[p - 1];
                const int ax0 = max(x0 - 2, 0) >> 4, ax1 = min(x0 + LT + 1, L.w - 1) >> 4;
                const int by0 = max(y0 - 2, 0) >> 4, by1 = min(y0 + LT + 1, L.h - 1) >> 4;
                const int na = ax1 - ax0 + 1, nb = by1 - by0 + 1;
                bool ok = true;
                if ((int)threadIdx.x < na * nb) {
                    const unsigned* f = P.done + (by0 + (int)threadIdx.x / na) * P.tiles_x + ax0 + (int)threadIdx.x % na;
                    uint32_t k = 0;
                    while (ld_acquire_u32(f) != mark && k < kPyrWaitPolls) {
                        __nanosleep(64);
                        k++;
                    }
                    ok = k < kPyrWaitPolls;
                }
                if (!__syncthreads_and(ok)) {
                    if (threadIdx.x == 0) atomicOr(L.nlf.err, 2u);
                    failed = true;
                    break;
                }
            }
            const T4* in = (const T4*)L.in;
            for (int i = threadIdx.x; i < LP * LP; i += kT) {
                const int r = i / LP, c = i - r * LP;
                const int gx = clampi(x0 - 2 + c, 0, L.w - 1), gy = clampi(y0 - 2 + r, 0, L.h - 1);
                stage[i] = p == 0 ? in[(size_t)gy * L.pitch + gx] : ld_cg(in + (size_t)gy * L.pitch + gx);
            }
        }
        if (L.out) level_tables(x0, y0, L.w, L.h, L.ow, L.oh, s_tx, s_ty);
        if (threadIdx.x == 0) s_item = (int)atomicAdd(&a.ctl->queue, 1u);
        __syncthreads();
        const int next = s_item;
        if constexpr (HALF) {
            for (int i = threadIdx.x; i < LP * LP; i += kT) s_wide[i] = Storage<__half>::cvt(stage[i]);
            __syncthreads();
        }
        const float4* const s_in = HALF ? s_wide : reinterpret_cast<const float4*>(stage);
        pending = next < a.items && by_tma(next);
        if (pending && threadIdx.x == 0) issue(next, buf ^ 1);
        level_tile<S>(s_in, s_tx, s_ty, x0, y0, L.w, L.h, L.out, L.ow, L.oh, L.opitch, a.th, a.stats_half, acc);
        ntiles++;
        if (L.out && p + 1 < a.nlev) {
            // publish the downsampled block to the next level's tiles: the barrier orders the
            // block's stores before thread 0's release, which is cumulative over them
            __syncthreads();
            if (threadIdx.x == 0) st_release_u32(L.done + t, mark);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        item = next;
        buf ^= 1;
    }
    if (cur >= 0 && !failed) flush();
    // the last block to leave resets the queue and advances the mark for the next launch
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&a.ctl->exits, 1u) == gridDim.x - 1) {
            __threadfence();
            // a level whose tile count is still open was not solved (a block gave up a wait and
            // recorded it in the error word): clear its count and the partial totals the other
            // blocks added, so that the next launch starts from empty sums
            for (int l = 0; l < a.nlev; l++) {
                if (atomicExch(&a.ctl->flushed[l], 0u) == 0u) continue;
                const NlfScratch& s = a.lv[l].nlf;
                for (int k = 0; k < 3 * kNlfK; k++) s.tot_limb[k] = 0ull;
                for (int k = 0; k < kNlfKF; k++) s.tot_mm[k] = 0u;
                *s.tot_nan = 0u;
                *s.ticket = 0u;
            }
            a.ctl->queue = 0u;
            a.ctl->exits = 0u;
            __threadfence();
            st_release_u32(&a.ctl->mark, mark);
        }
    }
}

// =========================================================================================
// denoise_reasm: denoiseImage (bilateral / guided fast) of a pyramid level and, below the
// coarsest level, reassembleImage with the next coarser level.  32x16 output tiles.
// =========================================================================================
constexpr int DW = 32, DH = 16;

template <class SIn, class S, int ALGO, bool REASM>
__global__ void __launch_bounds__(kT) denoise_reasm_kernel(DenoiseArgs a) {
    constexpr int PW = DW + 4, PH = DH + 4;
    __shared__ float4 s_in[PW * PH];
    const int x0 = blockIdx.x * DW, y0 = blockIdx.y * DH;
    const GImg4<SIn> gin{(const typename Storage<SIn>::T4*)a.in, a.w, a.h, a.pitch};
    for (int i = threadIdx.x; i < PW * PH; i += kT) {
        const int r = i / PW, c = i - r * PW;
        s_in[i] = gin.at(x0 - 2 + c, y0 - 2 + r);
    }
    __syncthreads();
    const SAcc4f I{s_in, x0 - 2, y0 - 2, PW};
    Nlf6 n;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        n.a[k] = a.nlf_dev[k] * a.mul[k];
        n.b[k] = a.nlf_dev[3 + k] * a.mul[3 + k];
    }
    typedef typename Storage<S>::T4 T4;
    const GImg4<S> i1{(const T4*)a.coarse_img, a.cw, a.ch, a.cpitch};
    const GImg4<S> d1{(const T4*)a.coarse_den, a.cw, a.ch, a.cpitch};
    for (int i = threadIdx.x; i < DW * DH; i += kT) {
        const int r = i / DW, c = i - r * DW, x = x0 + c, y = y0 + r;
        if (x >= a.w || y >= a.h) continue;
        float4 d = ALGO == 0 ? bilateral_px(I, x, y, n, a.chroma_boost, a.gradient_boost)
                             : guided_fast_px(I, x, y, n);
        d = round4<S>(d);
        if (REASM) d = round4<S>(reassemble_px(d, i1, d1, x, y, a.w, a.h, a.cw, a.ch, a.sharpening, n.a[0], n.b[0]));
        Storage<S>::st4((T4*)a.out + (size_t)y * a.opitch + x, d);
    }
}

// =========================================================================================
// final: level-0 denoise + reassemble over the tile, then the LTM mask, YCbCr -> camera and
// convertTosRGB.  32x24 output tiles, three positions per thread.  The local tone mapping
// samples its input bilinearly, which in general needs the denoised tile with a one-pixel
// ring (34x26).  Its sample points are the texel centres, though: when every column's and
// row's sample falls on one texel (weight 0 or 1 after the 8-bit fraction) inside the tile
// and the frame -- as it does for the bilateral denoiser at every practical frame width --
// the value is that texel's (the other weight multiplies a finite value by zero), and the
// block skips the ring (13 % of the positions it would otherwise denoise).
//
// Every bilinear sample here splits into an x part that depends only on the column and a y
// part that depends only on the row (tap1).  The block evaluates those parts once per
// column and row into tables, and stages the texels they reach -- the two half-resolution
// levels under the ring and the .x plane of the LTM guide -- in shared memory; a sample is
// then four table-indexed loads and the weights and blend of sample4, bit for bit.  The
// coordinates grow monotonically with x and y, so the first and last column (row) bound the
// texels a tile reaches: with the pyramid's sizes (w >> 1, w >> 3) that is at most
// FW / 2 + 4 half-resolution and FW / 8 + 5 guide texels across.
// =========================================================================================
// The output tile is FW x FH (a template parameter: the kernel is compiled for three
// shapes, chosen per frame size by the launch-shape tuner).
#define GLS_FINAL_TILE(FW, FH)                                                          \
    constexpr int EW = FW + 2, EH = FH + 2;           /* denoised level 0 with its ring */ \
    constexpr int HTW = EW / 2 + 6, HTH = EH / 2 + 6; /* half-resolution tile capacity */ \
    constexpr int GTW = FW / 8 + 8, GTH = FH / 8 + 8; /* guide tile capacity */

// tile origins (texels) and the table slots of one block
template <int FW, int FH>
struct FinalTabs {
    TabTap rx[3][FW + 2], ry[3][FH + 2];  // reassemble: u = ipx, ipx + nx, ipx - nx (rows likewise)
    TabTap lx[FW], ly[FH];        // LTM input sample on the denoised tile
    TabTap gx[3][FW], gy[3][FH];  // LTM guide, offsets GLS_LTM_OFFSETS + 0.5
    int org[8];                   // half-res x0, x1, y0, y1; guide x0, x1, y0, y1
};

// coordinate of table entry e of the block (the same float operations as the per-pixel
// samplers); which: 0 reassemble, 1 LTM input, 2 guide
GLS_DI float final_coord(int which, int k, int pos, float n) {
    const float off[3] = GLS_LTM_OFFSETS;
    if (which == 0) {
        const float ip = ((float)pos + 0.5f) * n;
        return k == 0 ? ip : (k == 1 ? ip + n : ip - n);
    }
    const float p = (float)pos * n;
    if (which == 1) return p + 0.5f * n;
    return p + (off[k] + 0.5f) * n;
}

// Whether an LTM input tap reads one texel of the tile's interior that phase 3 denoises:
// weight 0 or 1, the texel's offset (in units of ld) in [1, nf] and its coordinate
// org - 1 + offset inside the frame of n texels.  Taps of positions outside the frame
// (used = false) are never read.
GLS_DI bool ring_free_tap(const TabTap& u, int ld, int nf, int org, int n, bool used) {
    if (!used) return true;
    if (!(u.a == 0.0f || u.oma == 0.0f)) return false;
    const int off = (u.a == 0.0f ? u.i0 : u.i1) / ld;
    return off >= 1 && off <= nf && org - 1 + off < n;
}

template <class S, int ALGO, bool LTM, bool OUT_F32, int FW, int FH>
__global__ void __launch_bounds__(kT) final_kernel(FinalArgs a) {
    GLS_FINAL_TILE(FW, FH)
    constexpr int PW = FW + 6, PH = FH + 6;  // level 0 (binary16 values, widened), origin (x0 - 3, y0 - 3)
    constexpr int NRAW = 3 * EW + 3 * EH + FW + FH + 3 * FW + 3 * FH;
    __shared__ float4 s_l0[PW * PH];
    __shared__ float4 s_den[EW * EH];            // origin (x0 - 1, y0 - 1)
    __shared__ float4 s_i1[HTW * HTH], s_d1[HTW * HTH];
    __shared__ float s_g[GTW * GTH];
    __shared__ FinalTabs<FW, FH> T;
    __shared__ int s_ring_free;  // the LTM input reads only the tile's own texels
    // the raw table entries live only until the tables are built (phase 2); the denoised
    // tile is first written in phase 3
    static_assert(NRAW * sizeof(Tap1) <= sizeof(float4) * EW * EH, "raw table entries overflow the denoised tile");
    Tap1* const s_raw = reinterpret_cast<Tap1*>(s_den);
    const int x0 = blockIdx.x * FW, y0 = (blockIdx.y + a.tile_y0) * FH;
    const int w = a.w, h = a.h;
    const float nx = div_(1.0f, (float)w), ny = div_(1.0f, (float)h);

    // ---- phase 1: level-0 tile, raw table entries, tile origins ----
    for (int i = threadIdx.x; i < PW * PH; i += kT) {
        const int r = i / PW, c = i - r * PW;
        const int gx = clampi(x0 - 3 + c, 0, w - 1), gy = clampi(y0 - 3 + r, 0, h - 1);
        float4 v = Storage<__half>::cvt(a.level0[(size_t)gy * a.l0_pitch + gx]);
        v.w = 1.0f;  // the denoisers read only .xyz; the bilateral counts its normaliser in .w
        s_l0[i] = v;
    }
    // entry layout: rx[3][EW], ry[3][EH], lx[FW], ly[FH], gx[3][FW], gy[3][FH]
    constexpr int NRX = 3 * EW, NRY = 3 * EH, NLX = FW, NLY = FH, NGX = 3 * FW, NGY = 3 * FH;
    constexpr int NT = NRX + NRY + NLX + NLY + NGX + NGY;
    for (int e = threadIdx.x; e < NT; e += kT) {
        int q = e;
        Tap1 t;
        if (q < NRX) {
            t = tap1(final_coord(0, q / EW, x0 - 1 + q % EW, nx), a.cw);
        } else if ((q -= NRX) < NRY) {
            t = tap1(final_coord(0, q / EH, y0 - 1 + q % EH, ny), a.ch);
        } else if ((q -= NRY) < NLX) {
            t = tap1(final_coord(1, 0, x0 + q, nx), w);
        } else if ((q -= NLX) < NLY) {
            t = tap1(final_coord(1, 0, y0 + q, ny), h);
        } else if ((q -= NLY) < NGX) {
            t = tap1(final_coord(2, q / FW, x0 + q % FW, nx), a.gw);
        } else {
            q -= NGX;
            t = tap1(final_coord(2, q / FH, y0 + q % FH, ny), a.gh);
        }
        s_raw[e] = t;
    }
    if (threadIdx.x == 0) s_ring_free = ALGO == 0 || !LTM;
    if (threadIdx.x < 8) {
        // extremes: the smallest index sits at the first column (row) and smallest offset,
        // the largest at the last one and the largest offset; clamped to the image
        const int j = threadIdx.x;
        const bool guide = j >= 4, is_y = (j & 2) != 0, hi = (j & 1) != 0;
        const int n = guide ? (is_y ? a.gh : a.gw) : (is_y ? a.ch : a.cw);
        const float step = is_y ? ny : nx;
        const int pos = guide ? (is_y ? (hi ? y0 + FH - 1 : y0) : (hi ? x0 + FW - 1 : x0))
                              : (is_y ? (hi ? y0 + EH - 2 : y0 - 1) : (hi ? x0 + EW - 2 : x0 - 1));
        int v = hi ? -2147483647 : 2147483647;
        for (int k = 0; k < 3; k++) {
            const int i0 = tap1(final_coord(guide ? 2 : 0, k, pos, step), n).i0;
            v = hi ? max(v, i0 + 1) : min(v, i0);
        }
        T.org[j] = clampi(v, 0, n - 1);
    }
    __syncthreads();

    // ---- phase 2: tables against the tile origins, half-resolution and guide tiles ----
    const int hx0 = T.org[0], hy0 = T.org[2], gx0 = T.org[4], gy0 = T.org[6];
    const int htw = min(T.org[1] - hx0 + 1, HTW), hth = min(T.org[3] - hy0 + 1, HTH);
    const int gtw = min(T.org[5] - gx0 + 1, GTW), gth = min(T.org[7] - gy0 + 1, GTH);
    for (int e = threadIdx.x; e < NT; e += kT) {
        const Tap1 t = s_raw[e];
        int q = e;
        if (q < NRX) {
            T.rx[q / EW][q % EW] = tab_tap(t, a.cw, hx0, HTW, 1);
        } else if ((q -= NRX) < NRY) {
            T.ry[q / EH][q % EH] = tab_tap(t, a.ch, hy0, HTH, HTW);
        } else if ((q -= NRY) < NLX) {
            const TabTap u = tab_tap_tile(t, x0 - 1, EW, 1);
            T.lx[q] = u;
            if (LTM && !ring_free_tap(u, 1, FW, x0, w, x0 + q < w)) s_ring_free = 0;
        } else if ((q -= NLX) < NLY) {
            const TabTap u = tab_tap_tile(t, y0 - 1, EH, EW);
            T.ly[q] = u;
            if (LTM && !ring_free_tap(u, EW, FH, y0, h, y0 + q < h)) s_ring_free = 0;
        } else if ((q -= NLY) < NGX) {
            T.gx[q / FW][q % FW] = tab_tap(t, a.gw, gx0, GTW, 1);
        } else {
            q -= NGX;
            T.gy[q / FH][q % FH] = tab_tap(t, a.gh, gy0, GTH, GTW);
        }
    }
    typedef typename Storage<S>::T4 T4;
    {
        const GImg4<S> i1{(const T4*)a.pyr0, a.cw, a.ch, a.cpitch};
        const GImg4<S> d1{(const T4*)a.den1, a.cw, a.ch, a.cpitch};
        for (int i = threadIdx.x; i < htw * hth; i += kT) {
            const int r = i / htw, c = i - r * htw;
            s_i1[r * HTW + c] = i1.at(hx0 + c, hy0 + r);
            s_d1[r * HTW + c] = d1.at(hx0 + c, hy0 + r);
        }
        if (LTM) {
            const GImg4<S> guide{(const T4*)a.guide, a.gw, a.gh, a.gpitch};
            for (int i = threadIdx.x; i < gtw * gth; i += kT) {
                const int r = i / gtw, c = i - r * gtw;
                s_g[r * GTW + c] = guide.at(gx0 + c, gy0 + r).x;
            }
        }
    }
    __syncthreads();

    // ---- phase 3: denoise + reassemble over the tile and its ring ----
    const SAcc4f1 L0{{s_l0, x0 - 3, y0 - 3, PW}};
    Nlf6 n;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        n.a[k] = a.nlf_dev[k] * a.mul[k];
        n.b[k] = a.nlf_dev[3 + k] * a.mul[3 + k];
    }
    const bool ring_free = s_ring_free != 0;
    for (int i = threadIdx.x; i < (ring_free ? FW * FH : EW * EH); i += kT) {
        // position (r, c) of the denoised tile (origin x0 - 1, y0 - 1)
        const int r = ring_free ? i / FW + 1 : i / EW, c = ring_free ? i - (r - 1) * FW + 1 : i - r * EW;
        const int x = x0 - 1 + c, y = y0 - 1 + r;
        if (x < 0 || x >= w || y < 0 || y >= h) continue;
        Nlf6 nm = n;
        if (a.strength) {  // the learned stage's per-pixel multiplier of the noise model
            const float m = a.strength[(size_t)y * w + x];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                nm.a[k] = n.a[k] * m;
                nm.b[k] = n.b[k] * m;
            }
        }
        float4 d = ALGO == 0 ? bilateral_px(L0, x, y, nm, a.chroma_boost, a.gradient_boost)
                             : guided_fast_px(L0, x, y, nm);
        d = round4<S>(d);
        const float4 p1 = tab_sample4(s_i1, T.rx[0][c], T.ry[0][r]);
        const float4 pd1 = tab_sample4(s_d1, T.rx[0][c], T.ry[0][r]);
        auto sharp = [&]() {
            const float2 gx = tab_sample_x_x2(s_d1, T.rx[1][c], T.ry[0][r], T.rx[2][c], T.ry[0][r]);
            const float2 gy = tab_sample_x_x2(s_d1, T.rx[0][c], T.ry[1][r], T.rx[0][c], T.ry[2][r]);
            return make_float4(gx.x, gx.y, gy.x, gy.y);
        };
        d = round4<S>(reassemble_from(d, p1, pd1, sharp, a.sharpening, n.a[0], n.b[0]));
        s_den[r * EW + c] = d;
    }
    __syncthreads();
    if (!ring_free && (x0 - 1 < 0 || y0 - 1 < 0 || x0 + FW + 1 > w || y0 + FH + 1 > h)) {
        for (int i = threadIdx.x; i < EW * EH; i += kT) {
            const int r = i / EW, c = i - r * EW, x = x0 - 1 + c, y = y0 - 1 + r;
            if (x >= 0 && x < w && y >= 0 && y < h) continue;
            const int cx = clampi(x, 0, w - 1) - (x0 - 1), cy = clampi(y, 0, h - 1) - (y0 - 1);
            s_den[i] = s_den[cy * EW + cx];
        }
        __syncthreads();
    }

    // ---- phase 4: LTM mask, YCbCr -> camera, sRGB ----
    for (int i = threadIdx.x; i < FW * FH; i += kT) {
        const int r = i / FW, c = i - r * FW, x = x0 + c, y = y0 + r;
        if (x >= w || y >= h) continue;
        const float4 den = s_den[(r + 1) * EW + c + 1];
        if (a.tap_den) reinterpret_cast<float4*>(a.tap_den)[(size_t)y * a.tap_pitch + x] = den;
        float mask = 0.0f;
        if (LTM) {
            float gs[9];  // samples 0-7 in pairs: their sums as packed chains
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                const float2 v =
                    tab_sample1_x2(s_g, T.gx[k % 3][c], T.gy[k / 3][r], T.gx[(k + 1) % 3][c], T.gy[(k + 1) / 3][r]);
                gs[k] = v.x;
                gs[k + 1] = v.y;
            }
            gs[8] = tab_sample1(s_g, T.gx[2][c], T.gy[2][r]);
            // the input is sampled at texel centres: after the 8-bit fraction each axis sits on
            // one texel (fraction 0 or 1), and with the bilateral's finite outputs the sample is
            // that texel's value (the other weights are zero)
            const TabTap tx = T.lx[c], ty = T.ly[r];
            const bool one_x = tx.a == 0.0f || tx.oma == 0.0f, one_y = ty.a == 0.0f || ty.oma == 0.0f;
            const float4 inp = (ALGO == 0 && one_x && one_y)
                                   ? s_den[(ty.a == 0.0f ? ty.i0 : ty.i1) + (tx.a == 0.0f ? tx.i0 : tx.i1)]
                                   : tab_sample4(s_den, tx, ty);
            mask = Storage<S>::round(ltm_mask_from(gs, inp, a.ltm, a.icy));
            if (a.tap_mask) a.tap_mask[(size_t)y * a.tap_pitch + x] = mask;
        }
        const float3 cam = round3<S>(transform_px(a.icy, make_float3(den.x, den.y, den.z)));
        const float3 o = srgb_px(cam, mask, a.rgb_cam, a.rgb);
        if (OUT_F32) {
            reinterpret_cast<float4*>(a.out)[(size_t)y * a.opitch + x] = make_float4(o.x, o.y, o.z, 0.0f);
        } else {
            reinterpret_cast<uchar4*>(a.out)[(size_t)y * a.opitch + x] =
                make_uchar4(glsm::to_unorm8(o.x), glsm::to_unorm8(o.y), glsm::to_unorm8(o.z), 0);
        }
    }
}

int persistent_grid(gls_ctx* ctx, long tiles, int per_sm) {
    long g = (long)(ctx->num_sms > 0 ? ctx->num_sms : 148) * per_sm;
    if (g > kNlfMaxBlocks) g = kNlfMaxBlocks;
    if (g > tiles) g = tiles;
    return (int)(g < 1 ? 1 : g);
}

// A persistent grid of as many blocks as are resident at once: every block walks an equal
// share of the tiles, so blocks beyond the resident ones would run as a second, sparse wave.
// The count depends only on the kernel's resources, so the first query is kept (one static
// per kernel instantiation; concurrent first calls store the same value).
template <auto Kernel>
int resident_grid(gls_ctx* ctx, long tiles) {
    static int s_per_sm = 0;
    int per_sm = s_per_sm;
    if (per_sm < 1) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kernel, kT, 0) != cudaSuccess || per_sm < 1) {
            cudaGetLastError();
            per_sm = 1;
        } else {
            s_per_sm = per_sm;
        }
    }
    return persistent_grid(ctx, tiles, per_sm);
}

// Raw quads scaled on the fly, for the (rare) explicit regression passes.
template <class S>
struct RawU16SrcS {
    GRaw16 raw;
    float sm[4];
    float black;
    int bayer;
    bool half_stats;
    GLS_DI float at(int x, int y) const {
        x = clampi(x, 0, raw.w - 1);
        y = clampi(y, 0, raw.h - 1);
        return Storage<S>::round(scale_value(__ldg(raw.p + (size_t)y * raw.pitch + x), sm[((y & 1) << 1) | (x & 1)], black));
    }
    GLS_DI void stats(int qx, int qy, float* m, float* v) const {
        raw_stats_quad(*this, qx, qy, bayer, m, v);
        round_stats<4, 4>(m, v, half_stats);
    }
};

}  // namespace

#ifndef GLS_FUSED_FINAL_TU  // the final stage's launcher lives in k_fused_final.cu

// ------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------

// A 2D tensor map (elements of elem_bytes) of an image of w x h pixels of px_elems elements
// each, pitch in pixels, with a box of box_w x box_h elements; false where TMA does not apply
// (no driver entry point, an unaligned base or row, an image smaller than a box).
bool tensor_map_2d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int elem_bytes, int w_elems, int h,
                   int pitch_elems, int box_w, int box_h) {
    typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn s_encode = nullptr;
    static bool s_tried = false;
    if (!s_tried) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            s_encode = reinterpret_cast<EncodeFn>(f);
        else
            cudaGetLastError();
        s_tried = true;
    }
    const uint64_t row_bytes = (uint64_t)pitch_elems * (uint64_t)elem_bytes;
    if (!s_encode || (reinterpret_cast<uintptr_t>(base) & 15u) || (row_bytes & 15u) || w_elems < box_w || h < box_h ||
        ((uint64_t)box_w * elem_bytes) % 16u != 0)
        return false;
    const cuuint64_t dims[2] = {(cuuint64_t)w_elems, (cuuint64_t)h};
    const cuuint64_t strides[1] = {row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    const cuuint32_t estr[2] = {1, 1};
    return s_encode(map, type, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// A level (RGBA, 8 or 16 bytes per pixel) as 8-byte elements, with the 36x36-pixel box of a
// level_pass1 tile.
bool level_tensor_map(CUtensorMap* map, const void* base, int px_bytes, int w, int h, int pitch) {
    const int per = px_bytes / 8;
    return tensor_map_2d(map, base, CU_TENSOR_MAP_DATA_TYPE_UINT64, 8, w * per, h, pitch * per, LP * per, LP);
}

gls_status fused_raw_fit(gls_ctx* ctx, const RawPass1Args& args, bool half, NlfScratch s, float* out_dev) {
    RawPass1Args a = args;
    a.th = nlf_thresholds();
    a.nlf = s;
    a.nlf_out = out_dev;
    // Every scaled value is 0 or at least 2^-41 when each scale factor lies in [1/2, 2^15]
    // (unorm16 values and the black level are multiples of 2^-40, so a positive difference
    // is at least 2^-40), and at most 2^15 (finite in binary16 storage too); so a 5x5 sum is
    // 0 or in [2^-41, 2^20] and its square 0 or in [2^-82, 2^40], where x / 25 has its exact
    // shortcut.  Other scale factors take the checked path.
    a.sums_exact = 1;
    for (int k = 0; k < 4; k++)
        if (!(a.sm[k] >= 0.5f && a.sm[k] <= 32768.0f)) a.sums_exact = 0;
    const int qw = a.w / 2, qh = a.h / 2;
    const long tiles = (long)((qw + RQ - 1) / RQ) * ((qh + RQ - 1) / RQ);
    CUtensorMap map;
    memset(&map, 0, sizeof(map));
    a.tma = tensor_map_2d(&map, a.raw, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, a.w, a.h, a.pitch, RBW, RBH) ? 1 : 0;
#define GLS_RAWP1(SS, BY)                                                      \
    {                                                                          \
        const int grid = resident_grid<raw_pass1_kernel<SS, BY>>(ctx, tiles); \
        raw_pass1_kernel<SS, BY><<<grid, kT, 0, ctx->stream>>>(a, map);       \
    }
#define GLS_RAWP1_B(SS)                 \
    switch (a.bayer) {                  \
        case 0: GLS_RAWP1(SS, 0) break; \
        case 1: GLS_RAWP1(SS, 1) break; \
        case 2: GLS_RAWP1(SS, 2) break; \
        default: GLS_RAWP1(SS, 3) break; \
    }
    if (half) {
        GLS_RAWP1_B(__half)
        RawU16SrcS<__half> src{{a.raw, a.w, a.h, a.pitch}, {a.sm[0], a.sm[1], a.sm[2], a.sm[3]}, a.black, a.bayer,
                                  a.stats_half != 0};
        ctx->launches++;
        nlf_finish<4, 4>(ctx, src, qw, qh, s, out_dev);
    } else {
        GLS_RAWP1_B(float)
        RawU16SrcS<float> src{{a.raw, a.w, a.h, a.pitch}, {a.sm[0], a.sm[1], a.sm[2], a.sm[3]}, a.black, a.bayer,
                                 a.stats_half != 0};
        ctx->launches++;
        nlf_finish<4, 4>(ctx, src, qw, qh, s, out_dev);
    }
#undef GLS_RAWP1_B
#undef GLS_RAWP1
    return check_launch(ctx, "raw noise statistics (fused)");
}

// One compiled tile shape of the demosaic.
template <int TW, int TH>
void launch_demosaic(const DemosaicArgs& a, bool raw_u16, bool half, bool cnn, cudaStream_t st) {
    const dim3 grid((a.w + TW - 1) / TW, (a.h + TH - 1) / TH);
#define GLS_DEM(U16, SS)                                                           \
    if (cnn) demosaic_kernel<TW, TH, U16, SS, true><<<grid, kT, 0, st>>>(a);      \
    else demosaic_kernel<TW, TH, U16, SS, false><<<grid, kT, 0, st>>>(a);
    if (raw_u16) {
        if (half) { GLS_DEM(true, __half) } else { GLS_DEM(true, float) }
    } else {
        if (half) { GLS_DEM(false, __half) } else { GLS_DEM(false, float) }
    }
#undef GLS_DEM
}

// The learned stage's input path keeps the default shape; the plain path has three:
// 0: 44x28 (halos: green 1.25x, Sobel map 1.52x the tile; 44 KB, 5 blocks per SM),
// 1: 32x24 (more, smaller blocks: fills the GPU on small frames),
// 2: 64x32 (least halo, 67 KB, 3 blocks per SM),
// 3: split in two kernels through the green image (no green or Sobel halo recomputed).
void launch_demosaic_shape(int shape, const DemosaicArgs& a, bool raw_u16, bool half, cudaStream_t st) {
    if (a.cnn_in || shape == 0 || (shape == 3 && !a.green)) launch_demosaic<44, 28>(a, raw_u16, half, a.cnn_in != nullptr, st);
    else if (shape == 1) launch_demosaic<32, 24>(a, raw_u16, half, false, st);
    else if (shape == 2) launch_demosaic<64, 32>(a, raw_u16, half, false, st);
    else {
        const dim3 g1((a.w + SGW - 1) / SGW, (a.h + SGH - 1) / SGH), g2((a.w + 43) / 44, (a.h + 27) / 28);
#define GLS_SPLIT(U16, SS)                                        \
    green_split_kernel<U16, SS><<<g1, kT, 0, st>>>(a);            \
    rb_despeckle_kernel<U16, SS><<<g2, kT, 0, st>>>(a);
        if (raw_u16) {
            if (half) { GLS_SPLIT(true, __half) } else { GLS_SPLIT(true, float) }
        } else {
            if (half) { GLS_SPLIT(false, __half) } else { GLS_SPLIT(false, float) }
        }
#undef GLS_SPLIT
    }
}

gls_status fused_demosaic(gls_ctx* ctx, const DemosaicArgs& a, bool raw_u16, bool half) {
    const TuneKey key{kTuneDemosaic, a.w, a.h, (raw_u16 ? 1 : 0) | (half ? 2 : 0)};
    const int shape = a.cnn_in ? 0 : tune_choose(ctx, key, [&](int v) { launch_demosaic_shape(v, a, raw_u16, half, ctx->stream); });
    launch_demosaic_shape(shape, a, raw_u16, half, ctx->stream);
    ctx->launches++;
    return check_launch(ctx, "demosaic (fused)");
}

gls_status fused_post_cnn(gls_ctx* ctx, const PostCnnArgs& a, bool half) {
    const dim3 grid((a.w + PCW - 1) / PCW, (a.h + PCH - 1) / PCH);
    if (half) post_cnn_kernel<__half><<<grid, kT, 0, ctx->stream>>>(a);
    else post_cnn_kernel<float><<<grid, kT, 0, ctx->stream>>>(a);
    ctx->launches++;
    return check_launch(ctx, "after the learned stage");
}

gls_status fused_level_fit(gls_ctx* ctx, const LevelPass1Args& args, bool in_half, bool half, NlfScratch s,
                           float* out_dev) {
    LevelPass1Args a = args;
    a.th = nlf_thresholds();
    a.nlf = s;
    a.nlf_out = out_dev;
    CUtensorMap map;
    memset(&map, 0, sizeof(map));
    a.tma = level_tensor_map(&map, a.in, in_half ? 8 : 16, a.w, a.h, a.pitch) ? 1 : 0;
    const long tiles = (long)((a.w + LT - 1) / LT) * ((a.h + LT - 1) / LT);
    if (in_half) {
        if (half) level_pass1_kernel<__half, __half><<<resident_grid<level_pass1_kernel<__half, __half>>(ctx, tiles), kT, 0, ctx->stream>>>(a, map);
        else level_pass1_kernel<__half, float><<<resident_grid<level_pass1_kernel<__half, float>>(ctx, tiles), kT, 0, ctx->stream>>>(a, map);
        LevelSrc<__half> src{{(const half4*)a.in, a.w, a.h, a.pitch}, a.stats_half != 0};
        ctx->launches++;
        nlf_finish<1, 3>(ctx, src, a.w, a.h, s, out_dev);
    } else {
        level_pass1_kernel<float, float><<<resident_grid<level_pass1_kernel<float, float>>(ctx, tiles), kT, 0, ctx->stream>>>(a, map);
        LevelSrc<float> src{{(const float4*)a.in, a.w, a.h, a.pitch}, a.stats_half != 0};
        ctx->launches++;
        nlf_finish<1, 3>(ctx, src, a.w, a.h, s, out_dev);
    }
    return check_launch(ctx, "level statistics (fused)");
}

gls_status fused_wait_probe(gls_ctx* ctx, NlfScratch s, unsigned polls) {
    stage_wait_probe_kernel<<<1, kT, 0, ctx->stream>>>(s, polls);
    ctx->launches++;
    return check_launch(ctx, "statistics wait probe");
}

gls_status fused_pyramid_stats(gls_ctx* ctx, const PyramidArgs& args, bool half) {
    PyramidArgs a = args;
    a.th = nlf_thresholds();
    CUtensorMap map;
    memset(&map, 0, sizeof(map));
    a.tma = level_tensor_map(&map, a.lv[0].in, half ? 8 : 16, a.lv[0].w, a.lv[0].h, a.lv[0].pitch) ? 1 : 0;
    if (half) {
        pyramid_stats_kernel<__half><<<resident_grid<pyramid_stats_kernel<__half>>(ctx, a.items), kT, 0, ctx->stream>>>(a, map);
    } else {
        pyramid_stats_kernel<float><<<resident_grid<pyramid_stats_kernel<float>>(ctx, a.items), kT, 0, ctx->stream>>>(a, map);
    }
    ctx->launches++;
    GLS_CHECK(check_launch(ctx, "pyramid statistics (fused)"));
    // the explicit regression passes of every level, one launch each (they exit at once
    // unless a level's solve could not prove them redundant)
    auto finish = [&](auto tag) {
        typedef decltype(tag) SS;
        typedef typename Storage<SS>::T4 T4;
        LevelSet<SS> ls{};
        ls.n = a.nlev;
        for (int p = 0; p < a.nlev; p++) {
            const PyrLevel& L = a.lv[p];
            ls.src[p] = LevelSrc<SS>{{(const T4*)L.in, L.w, L.h, L.pitch}, a.stats_half != 0};
            ls.s[p] = L.nlf;
            ls.out[p] = L.nlf_out;
        }
        const int grid = grid_for(ctx, a.lv[0].w, a.lv[0].h);
        nlf_pass2_levels_kernel<SS><<<grid, kThreads, 0, ctx->stream>>>(ls, a.th);
        nlf_pass3_levels_kernel<SS><<<grid, kThreads, 0, ctx->stream>>>(ls, a.th);
        ctx->launches += 2;
    };
    if (half) finish(__half());
    else finish(float());
    return check_launch(ctx, "pyramid statistics (explicit passes)");
}

gls_status fused_denoise(gls_ctx* ctx, const DenoiseArgs& a, bool in_half, bool half, int algo, bool reasm) {
    const dim3 grid((a.w + DW - 1) / DW, (a.h + DH - 1) / DH);
    cudaStream_t st = ctx->stream;
#define GLS_DEN(SIN, SS, AL, RE) denoise_reasm_kernel<SIN, SS, AL, RE><<<grid, kT, 0, st>>>(a)
    if (in_half && half) {
        if (algo == 0) { if (reasm) GLS_DEN(__half, __half, 0, true); else GLS_DEN(__half, __half, 0, false); }
        else { if (reasm) GLS_DEN(__half, __half, 1, true); else GLS_DEN(__half, __half, 1, false); }
    } else if (in_half) {
        if (algo == 0) { if (reasm) GLS_DEN(__half, float, 0, true); else GLS_DEN(__half, float, 0, false); }
        else { if (reasm) GLS_DEN(__half, float, 1, true); else GLS_DEN(__half, float, 1, false); }
    } else {
        if (algo == 0) { if (reasm) GLS_DEN(float, float, 0, true); else GLS_DEN(float, float, 0, false); }
        else { if (reasm) GLS_DEN(float, float, 1, true); else GLS_DEN(float, float, 1, false); }
    }
#undef GLS_DEN
    ctx->launches++;
    return check_launch(ctx, "denoise/reassemble (fused)");
}

#else

template <int FW, int FH>
void launch_final(const FinalArgs& args, bool half, int algo, bool ltm, bool out_f32, int ty0, int nty, cudaStream_t st) {
    FinalArgs a = args;
    a.tile_y0 = ty0;
    const dim3 grid((a.w + FW - 1) / FW, nty);
#define GLS_FIN(SS, AL)                                                                          \
    if (ltm) {                                                                                   \
        if (out_f32) final_kernel<SS, AL, true, true, FW, FH><<<grid, kT, 0, st>>>(a);           \
        else final_kernel<SS, AL, true, false, FW, FH><<<grid, kT, 0, st>>>(a);                  \
    } else {                                                                                     \
        if (out_f32) final_kernel<SS, AL, false, true, FW, FH><<<grid, kT, 0, st>>>(a);          \
        else final_kernel<SS, AL, false, false, FW, FH><<<grid, kT, 0, st>>>(a);                 \
    }
    if (half) {
        if (algo == 0) { GLS_FIN(__half, 0) } else { GLS_FIN(__half, 1) }
    } else {
        if (algo == 0) { GLS_FIN(float, 0) } else { GLS_FIN(float, 1) }
    }
#undef GLS_FIN
}

// The bilateral path with the local tone mapping has three shapes (three, two and four
// positions per thread): 0: 32x24, 1: 32x16, 2: 64x16; the other forms keep 32x24.
int final_shape_h(int shape, int algo, bool ltm) { return (shape == 0 || algo != 0 || !ltm) ? 24 : 16; }

// tile rows [ty0, ty0 + nty) of shape `shape` (nty < 0: the whole frame)
void launch_final_shape(int shape, const FinalArgs& a, bool half, int algo, bool ltm, bool out_f32, int ty0, int nty,
                        cudaStream_t st) {
    if (nty < 0) nty = (a.h + final_shape_h(shape, algo, ltm) - 1) / final_shape_h(shape, algo, ltm);
    if (shape == 0 || algo != 0 || !ltm) launch_final<32, 24>(a, half, algo, ltm, out_f32, ty0, nty, st);
    else if (shape == 1) launch_final<32, 16>(a, half, 0, true, out_f32, ty0, nty, st);
    else launch_final<64, 16>(a, half, 0, true, out_f32, ty0, nty, st);
}

gls_status fused_final(gls_ctx* ctx, const FinalArgs& a, bool half, int algo, bool ltm, bool out_f32, int bands,
                       const FinalBandFn* band) {
    // the staged tiles are sized for the pyramid's levels 1 and 3
    if (a.cw != a.w >> 1 || a.ch != a.h >> 1 || (ltm && (a.gw != a.w >> 3 || a.gh != a.h >> 3)))
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "final stage: levels 1 and 3 must be the pyramid's");
    if (bands > 1 && !band) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "final stage: bands without a callback");
    int shape = 0;
    if (algo == 0 && ltm) {
        const TuneKey key{kTuneFinal, a.w, a.h, (half ? 1 : 0) | (out_f32 ? 2 : 0)};
        shape = tune_choose(ctx, key, [&](int v) { launch_final_shape(v, a, half, algo, ltm, out_f32, 0, -1, ctx->stream); });
    }
    const int fh = final_shape_h(shape, algo, ltm), tiles_y = (a.h + fh - 1) / fh;
    if (bands < 1) bands = 1;
    if (bands > tiles_y) bands = tiles_y;
    for (int b = 0; b < bands; b++) {
        const int ty0 = (int)((long)tiles_y * b / bands), ty1 = (int)((long)tiles_y * (b + 1) / bands);
        launch_final_shape(shape, a, half, algo, ltm, out_f32, ty0, ty1 - ty0, ctx->stream);
        ctx->launches++;
        GLS_CHECK(check_launch(ctx, "final (fused)"));
        if (band) GLS_CHECK(band->fn(band->user, ty0 * fh, ty1 * fh < a.h ? ty1 * fh : a.h));
    }
    return GLS_OK;
}

#endif  // GLS_FUSED_FINAL_TU

}  // namespace gls
