// gls_nlf.cuh -- device side of the noise-model regressions (computeNoiseStatistics /
// computeRawNoiseStatistics, CLImage/app/src/main/cpp/pyramidal_denoise.cpp:161-362):
// statistics sources, the explicit FP64 passes, the parallel deterministic solve, and
// the launcher that finishes a fit once pass-1 partial sums exist.  Included by k_nlf.cu
// (single-stage regressions) and k_fused.cu (pass 1 fused into the pyramid kernels); the
// kernels have internal linkage in each translation unit.
#ifndef GLS_NLF_CUH
#define GLS_NLF_CUH

#include "gls_internal.h"
#include "gls_pixel_ops.cuh"

namespace gls {
namespace {

constexpr int kTX = 32, kTY = 8, kThreads = kTX * kTY;

// ---- statistics sources: stats(x, y, m[MC], v[NC]) over a (sw x sh) grid ----

template <class S>
struct RawScaledSrc {
    GImg1<S> img;
    int bayer;
    GLS_DI void stats(int qx, int qy, float* m, float* v) const { raw_stats_quad(img, qx, qy, bayer, m, v); }
};

// Raw uint16 read with scaleRawData applied on the fly (and the storage rounding of the
// scaled image), so the scaled raw frame never has to be written.
struct ScaledRawAcc {
    GRaw16 raw;
    float sm[4];  // scale factor per (y & 1) * 2 + (x & 1)
    float black;
    bool half;
    GLS_DI float at(int x, int y) const {
        x = clampi(x, 0, raw.w - 1);
        y = clampi(y, 0, raw.h - 1);
        const float v = scale_value(__ldg(raw.p + (size_t)y * raw.pitch + x), sm[((y & 1) << 1) | (x & 1)], black);
        return half ? glsm::round_half(v) : v;
    }
};

struct RawU16Src {
    ScaledRawAcc acc;
    int bayer;
    GLS_DI void stats(int qx, int qy, float* m, float* v) const { raw_stats_quad(acc, qx, qy, bayer, m, v); }
};

template <class S>
struct LevelSrc {
    GImg4<S> img;
    GLS_DI void stats(int x, int y, float* m, float* v) const {
        const float4 s = noise_stats_px(img, x, y);
        m[0] = s.x;
        v[0] = s.y;
        v[1] = s.z;
        v[2] = s.w;
    }
};

// inRange (pyramidal_denoise.cpp:152-159): rejects values below or above the bounds, so a
// NaN statistic is accepted, exactly as the reference's comparisons do.
template <int MC, int NC>
GLS_DI bool in_range(const float* m, const float* v, const NlfThresholds& t) {
#pragma unroll
    for (int c = 0; c < MC; c++)
        if (m[c] < t.m_lo || m[c] > t.m_hi) return false;
#pragma unroll
    for (int c = 0; c < NC; c++)
        if (v[c] < t.v_lo || v[c] > t.v_hi) return false;
    return true;
}

// Block reduction of K doubles (fixed order), result written by threads < K.
template <int K>
GLS_DI void block_reduce_write(double (&vals)[K], double* out) {
    __shared__ double red[kThreads / 32][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const double s = warp_sum_d(vals[k]);
        if (lane == 0) red[warp][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; w++) s += red[w][threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

template <int K>
GLS_DI void block_minmax_write(float (&mn)[K], float (&mx)[K], float* out) {
    __shared__ float rmn[kThreads / 32][K], rmx[kThreads / 32][K];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float a = warp_min_f(mn[k]), b = warp_max_f(mx[k]);
        if (lane == 0) {
            rmn[warp][k] = a;
            rmx[warp][k] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < K) {
        float a = rmn[0][threadIdx.x], b = rmx[0][threadIdx.x];
        for (int w = 1; w < kThreads / 32; w++) {
            a = fminf(a, rmn[w][threadIdx.x]);
            b = fmaxf(b, rmx[w][threadIdx.x]);
        }
        out[threadIdx.x] = a;
        out[K + threadIdx.x] = b;
    }
    __syncthreads();
}

// Per-thread pass-1 accumulator.  Partial record (doubles): [0] N, then per channel c at
// 1+5c: sx, sxx, sy, sxy, syy.  Float record: [0..2NC) minimum of (m_c, v_c),
// [2NC..4NC) maximum.  All threads of the block must call write().
template <int MC, int NC>
struct Pass1Acc {
    static constexpr int NM = (MC == 1) ? 1 : NC;
    FF sx[NM], sxx[NM], sy[NC], sxy[NC], syy[NC];
    float mn[2 * NC], mx[2 * NC];
    int n;

    GLS_DI void init() {
#pragma unroll
        for (int c = 0; c < NM; c++) {
            ff_zero(sx[c]);
            ff_zero(sxx[c]);
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            ff_zero(sy[c]);
            ff_zero(sxy[c]);
            ff_zero(syy[c]);
        }
#pragma unroll
        for (int k = 0; k < 2 * NC; k++) {
            mn[k] = glsm::inf_();
            mx[k] = -glsm::inf_();
        }
        n = 0;
    }

    GLS_DI void add(const float* m, const float* v, const NlfThresholds& th) {
        if (!in_range<MC, NC>(m, v, th)) return;
        n++;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const float mc = m[MC == 1 ? 0 : c];
            if (MC != 1 || c == 0) {
                ff_add(sx[MC == 1 ? 0 : c], mc);
                ff_add_prod(sxx[MC == 1 ? 0 : c], mc, mc);
            }
            ff_add(sy[c], v[c]);
            ff_add_prod(sxy[c], mc, v[c]);
            ff_add_prod(syy[c], v[c], v[c]);
            mn[c] = fminf(mn[c], mc);
            mx[c] = fmaxf(mx[c], mc);
            mn[NC + c] = fminf(mn[NC + c], v[c]);
            mx[NC + c] = fmaxf(mx[NC + c], v[c]);
        }
    }

    GLS_DI void write(double* part_d, float* part_f) {
        double vals[1 + 5 * NC];
        vals[0] = (double)n;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int cm = MC == 1 ? 0 : c;
            vals[1 + 5 * c + 0] = ff_value(sx[cm]);
            vals[1 + 5 * c + 1] = ff_value(sxx[cm]);
            vals[1 + 5 * c + 2] = ff_value(sy[c]);
            vals[1 + 5 * c + 3] = ff_value(sxy[c]);
            vals[1 + 5 * c + 4] = ff_value(syy[c]);
        }
        block_reduce_write<1 + 5 * NC>(vals, part_d + (size_t)blockIdx.x * kNlfK);
        block_minmax_write<2 * NC>(mn, mx, part_f + (size_t)blockIdx.x * kNlfKF);
    }
};

template <int MC, int NC, class Src>
__global__ void __launch_bounds__(kThreads) nlf_pass1_kernel(Src src, int sw, int sh, NlfThresholds th,
                                                             double* part_d, float* part_f) {
    Pass1Acc<MC, NC> acc;
    acc.init();
    const int tiles_x = (sw + kTX - 1) / kTX, tiles_y = (sh + kTY - 1) / kTY;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    for (int t = blockIdx.x; t < tiles_x * tiles_y; t += gridDim.x) {
        const int x = (t % tiles_x) * kTX + tx, y = (t / tiles_x) * kTY + ty;
        if (x >= sw || y >= sh) continue;
        float m[MC], v[NC];
        src.stats(x, y, m, v);
        acc.add(m, v, th);
    }
    acc.write(part_d, part_f);
}

// Explicit pass 2 (only when solve 1 could not prove pass 3 trivial): sum of squared
// residuals per channel, FP64 per pixel as the reference computes it.
template <int MC, int NC, class Src>
__global__ void __launch_bounds__(kThreads) nlf_pass2_kernel(Src src, int sw, int sh, NlfThresholds th,
                                                             const NlfFit* fit, double* part_d) {
    if (fit->mode != 1) return;
    double acc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) acc[c] = 0.0;
    const int tiles_x = (sw + kTX - 1) / kTX, tiles_y = (sh + kTY - 1) / kTY;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    for (int t = blockIdx.x; t < tiles_x * tiles_y; t += gridDim.x) {
        const int x = (t % tiles_x) * kTX + tx, y = (t / tiles_x) * kTY + ty;
        if (x >= sw || y >= sh) continue;
        float m[MC], v[NC];
        src.stats(x, y, m, v);
        if (!in_range<MC, NC>(m, v, th)) continue;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const double d = (fit->A[c] + fit->B[c] * (double)m[MC == 1 ? 0 : c]) - (double)v[c];
            acc[c] += d * d;
        }
    }
    block_reduce_write<NC>(acc, part_d + (size_t)blockIdx.x * kNlfK);
}

// Explicit pass 3: refit on the pixels whose squared residual is <= err2 in every channel.
template <int MC, int NC, class Src>
__global__ void __launch_bounds__(kThreads) nlf_pass3_kernel(Src src, int sw, int sh, NlfThresholds th,
                                                             const NlfFit* fit, double* part_d) {
    if (fit->mode != 2) return;
    double vals[1 + 5 * NC];
#pragma unroll
    for (int k = 0; k < 1 + 5 * NC; k++) vals[k] = 0.0;
    const int tiles_x = (sw + kTX - 1) / kTX, tiles_y = (sh + kTY - 1) / kTY;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    for (int t = blockIdx.x; t < tiles_x * tiles_y; t += gridDim.x) {
        const int x = (t % tiles_x) * kTX + tx, y = (t / tiles_x) * kTY + ty;
        if (x >= sw || y >= sh) continue;
        float m[MC], v[NC];
        src.stats(x, y, m, v);
        if (!in_range<MC, NC>(m, v, th)) continue;
        bool ok = true;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const double d = (fit->A[c] + fit->B[c] * (double)m[MC == 1 ? 0 : c]) - (double)v[c];
            if (!(d * d <= fit->err2[c])) ok = false;
        }
        if (!ok) continue;
        vals[0] += 1.0;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const double mm = (double)m[MC == 1 ? 0 : c], vv = (double)v[c];
            vals[1 + 5 * c + 0] += mm;
            vals[1 + 5 * c + 1] += mm * mm;
            vals[1 + 5 * c + 2] += vv;
            vals[1 + 5 * c + 3] += mm * vv;
        }
    }
    block_reduce_write<1 + 5 * NC>(vals, part_d + (size_t)blockIdx.x * kNlfK);
}

// std::max(v, a) as gls::max(DVector, double) evaluates it (gls_linalg.hpp:238-243)
__device__ double refmax(double v, double a) { return (v < a) ? a : v; }

__device__ void neumaier(double& s, double& c, double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// One block of kSolveThreads: thread t sums (compensated) the partial rows t, t + T, ...;
// the per-thread sums are then added in a fixed tree, so the result does not depend on
// scheduling.  Thread 0 runs the FP64 regression step of the given stage.
constexpr int kSolveThreads = 256;

template <int NC>
__global__ void __launch_bounds__(kSolveThreads) nlf_solve_kernel(const double* part_d, const float* part_f,
                                                                  int nblocks, int stage, NlfFit* fit, float* out) {
    constexpr int K = 1 + 5 * NC;
    __shared__ double red[kSolveThreads];
    __shared__ float fred[kSolveThreads];
    __shared__ double tot[kNlfK];
    __shared__ float fmm[kNlfKF];
    if (stage == 2 && fit->mode != 1) return;
    if (stage == 3 && fit->mode != 2) return;
    const int nk = stage == 2 ? NC : K;
    const int t = threadIdx.x;
    double s[K], c[K];
#pragma unroll
    for (int k = 0; k < K; k++) s[k] = c[k] = 0.0;
    for (int b = t; b < nblocks; b += kSolveThreads) {
#pragma unroll
        for (int k = 0; k < K; k++)
            if (k < nk) neumaier(s[k], c[k], part_d[(size_t)b * kNlfK + k]);
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        if (k >= nk) break;
        red[t] = s[k] + c[k];
        __syncthreads();
        for (int o = kSolveThreads / 2; o > 0; o >>= 1) {
            if (t < o) red[t] += red[t + o];
            __syncthreads();
        }
        if (t == 0) tot[k] = red[0];
        __syncthreads();
    }
    if (stage == 1) {
        for (int k = 0; k < 4 * NC; k++) {
            const bool is_min = k < 2 * NC;
            float v = is_min ? glsm::inf_() : -glsm::inf_();
            for (int b = t; b < nblocks; b += kSolveThreads) {
                const float x = part_f[(size_t)b * kNlfKF + k];
                v = is_min ? fminf(v, x) : fmaxf(v, x);
            }
            fred[t] = v;
            __syncthreads();
            for (int o = kSolveThreads / 2; o > 0; o >>= 1) {
                if (t < o) fred[t] = is_min ? fminf(fred[t], fred[t + o]) : fmaxf(fred[t], fred[t + o]);
                __syncthreads();
            }
            if (t == 0) fmm[k] = fred[0];
            __syncthreads();
        }
    }
    if (threadIdx.x != 0) return;

    if (stage == 1 || stage == 3) {
        const double N = tot[0];
        double A[4], B[4];
        for (int ch = 0; ch < NC; ch++) {
            const double sx = tot[1 + 5 * ch], sxx = tot[2 + 5 * ch], sy = tot[3 + 5 * ch], sxy = tot[4 + 5 * ch];
            B[ch] = refmax((N * sxy - sx * sy) / (N * sxx - sx * sx), 1e-8);
            A[ch] = refmax((sy - B[ch] * sx) / N, 1e-8);
        }
        bool done = true;
        if (stage == 1) {
            fit->N1 = N;
            for (int ch = 0; ch < NC; ch++) {
                fit->A[ch] = A[ch];
                fit->B[ch] = B[ch];
                const double sx = tot[1 + 5 * ch], sxx = tot[2 + 5 * ch], sy = tot[3 + 5 * ch];
                const double sxy = tot[4 + 5 * ch], syy = tot[5 + 5 * ch];
                const double a = A[ch], b = B[ch];
                const double t1 = N * a * a, t2 = 2.0 * a * b * sx, t3 = b * b * sxx;
                const double t4 = -2.0 * a * sy, t5 = -2.0 * b * sxy, t6 = syy;
                const double e = t1 + t2 + t3 + t4 + t5 + t6;
                const double mag = fabs(t1) + fabs(t2) + fabs(t3) + fabs(t4) + fabs(t5) + fabs(t6);
                const double e_lo = e - 1e-12 * mag;
                bool skip = N > 0 && e_lo > 0 && a == a && b == b;
                if (skip) {
                    const double rms_lo = sqrt(e_lo / N) * (1.0 - 1e-6);
                    const double mlo = (double)fmm[ch], mhi = (double)fmm[2 * NC + ch];
                    const double vlo = (double)fmm[NC + ch], vhi = (double)fmm[3 * NC + ch];
                    const double dmax = a + b * (b >= 0 ? mhi : mlo) - vlo;
                    const double dmin = a + b * (b >= 0 ? mlo : mhi) - vhi;
                    const double mabs_ = fmax(fabs(dmax), fabs(dmin));
                    skip = mabs_ * mabs_ * (1.0 + 1e-9) <= rms_lo;
                }
                if (!skip) done = false;
            }
            fit->mode = done ? 0 : 1;
        } else {
            fit->mode = 0;
        }
        if (done) {
            for (int ch = 0; ch < NC; ch++) {
                out[ch] = (float)A[ch];
                out[NC + ch] = (float)B[ch];
            }
        }
    } else {  // stage 2: RMS of the residuals, evaluated with sqrtf as gls::sqrt(Vector) does
        for (int ch = 0; ch < NC; ch++) fit->err2[ch] = (double)sqrtf((float)(tot[ch] / fit->N1));
        fit->mode = 2;
    }
}

int grid_for(gls_ctx* ctx, int sw, int sh) {
    const long tiles = (long)((sw + kTX - 1) / kTX) * ((sh + kTY - 1) / kTY);
    long g = 4L * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    if (g > kNlfMaxBlocks) g = kNlfMaxBlocks;
    if (g > tiles) g = tiles;
    return (int)(g < 1 ? 1 : g);
}

// Everything after pass 1: solve, and the explicit error and refit passes (which exit at
// once unless solve 1 could not prove them redundant).  pass1_blocks partial rows exist.
template <int MC, int NC, class Src>
void nlf_finish(gls_ctx* ctx, const Src& src, int sw, int sh, int pass1_blocks, NlfScratch s, float* out_dev) {
    const NlfThresholds th = nlf_thresholds();
    const int grid = grid_for(ctx, sw, sh);
    cudaStream_t st = ctx->stream;
    nlf_solve_kernel<NC><<<1, kSolveThreads, 0, st>>>(s.part_d, s.part_f, pass1_blocks, 1, s.fit, out_dev);
    nlf_pass2_kernel<MC, NC, Src><<<grid, kThreads, 0, st>>>(src, sw, sh, th, s.fit, s.part_d);
    nlf_solve_kernel<NC><<<1, kSolveThreads, 0, st>>>(s.part_d, s.part_f, grid, 2, s.fit, out_dev);
    nlf_pass3_kernel<MC, NC, Src><<<grid, kThreads, 0, st>>>(src, sw, sh, th, s.fit, s.part_d);
    nlf_solve_kernel<NC><<<1, kSolveThreads, 0, st>>>(s.part_d, s.part_f, grid, 3, s.fit, out_dev);
    ctx->launches += 5;
}

template <int MC, int NC, class Src>
gls_status run_fit(gls_ctx* ctx, const Src& src, int sw, int sh, NlfScratch s, float* out_dev) {
    const NlfThresholds th = nlf_thresholds();
    const int grid = grid_for(ctx, sw, sh);
    nlf_pass1_kernel<MC, NC, Src><<<grid, kThreads, 0, ctx->stream>>>(src, sw, sh, th, s.part_d, s.part_f);
    ctx->launches += 1;
    nlf_finish<MC, NC, Src>(ctx, src, sw, sh, grid, s, out_dev);
    return check_launch(ctx, "noise model regression");
}

}  // namespace
}  // namespace gls

#endif  // GLS_NLF_CUH
