// gls_nlf.cuh -- device side of the noise-model regressions (computeNoiseStatistics /
// computeRawNoiseStatistics, CLImage/app/src/main/cpp/pyramidal_denoise.cpp:161-362):
// statistics sources, exact fixed-point partial sums, the solves run by the last block of
// each pass, the explicit FP64 passes, and the launchers.  Included by k_nlf.cu
// (single-stage regressions) and k_fused.cu (pass 1 fused into the pyramid kernels); the
// kernels have internal linkage in each translation unit.
#ifndef GLS_NLF_CUH
#define GLS_NLF_CUH

#include "gls_f32x2.cuh"
#include "gls_internal.h"
#include "gls_pixel_ops.cuh"

namespace gls {
namespace {

constexpr int kTX = 32, kTY = 8, kThreads = kTX * kTY;

// ---- statistics sources: stats(x, y, m[MC], v[NC]) over a (sw x sh) grid ----

// The statistics as the fit reads them: fp32, or (half_stats) rounded to binary16, as the
// reference's fp16 build stores its statistics images.
template <int MC, int NC>
GLS_DI void round_stats(float* m, float* v, bool half_stats) {
    if (!half_stats) return;
#pragma unroll
    for (int c = 0; c < MC; c++) m[c] = glsm::round_half(m[c]);
#pragma unroll
    for (int c = 0; c < NC; c++) v[c] = glsm::round_half(v[c]);
}

template <class S>
struct RawScaledSrc {
    GImg1<S> img;
    int bayer;
    bool half_stats;
    GLS_DI void stats(int qx, int qy, float* m, float* v) const {
        raw_stats_quad(img, qx, qy, bayer, m, v);
        round_stats<4, 4>(m, v, half_stats);
    }
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
    bool half_stats;
    GLS_DI void stats(int qx, int qy, float* m, float* v) const {
        raw_stats_quad(acc, qx, qy, bayer, m, v);
        round_stats<4, 4>(m, v, half_stats);
    }
};

template <class S>
struct LevelSrc {
    GImg4<S> img;
    bool half_stats;
    GLS_DI void stats(int x, int y, float* m, float* v) const {
        const float4 s = noise_stats_px(img, x, y);
        m[0] = s.x;
        v[0] = s.y;
        v[1] = s.z;
        v[2] = s.w;
        round_stats<1, 3>(m, v, half_stats);
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

// A float as an unsigned word with the same order (-0 below +0; NaN is never stored).
GLS_DI unsigned ord_f32(float x) {
    const unsigned b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
GLS_DI float unord_f32(unsigned u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

// The block's minima and maxima folded into the running extremes: tot[k] holds ~ord(min k)
// and tot[K + k] ord(max k), both by atomic maximum, so zero is the identity of both.
template <int K>
GLS_DI void block_minmax_atomic(float (&mn)[K], float (&mx)[K], unsigned* tot) {
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
        atomicMax(tot + threadIdx.x, ~ord_f32(a));
        atomicMax(tot + K + threadIdx.x, ord_f32(b));
    }
    __syncthreads();
}

// the running extremes back as floats (an untouched word: +inf for a minimum, -inf for a
// maximum, as the empty reductions give)
GLS_DI float tot_min(unsigned u) { return u ? unord_f32(~u) : glsm::inf_(); }
GLS_DI float tot_max(unsigned u) { return u ? unord_f32(u) : -glsm::inf_(); }

// ---- exact fixed-point partial sums ----
// Each thread sums its pixels in float-float pairs.  From there on the pass-1 and pass-3
// sums travel as 128-bit two's-complement integers in units of 2^-R, R fixed per column, so
// the block and grid reductions are exact: the totals depend neither on the order of the
// additions nor on the number of blocks, and integer adds replace FP64 ones (GB300 runs FP64
// at a small fraction of its FP32 rate).  Every selected term is bounded (0.001 <= m <= 0.5,
// 0 <= v <= 0.001), so with fewer than 2^31 selected pixels no column total reaches 2^126
// units, and the resolutions (2^-95 for sx ... 2^-114 for syy) lie far below the rounding
// of the doubles the fit uses.
struct I128 {
    unsigned long long lo, hi;  // value = hi * 2^64 + lo, two's complement
};

// R of column k of a record [N, then per channel (sx, sxx, sy, sxy, syy)]
GLS_DI int fixed_scale(int k) {
    if (k == 0) return 0;
    switch ((k - 1) % 5) {
        case 0: return 95;
        case 1: return 96;
        case 2: return 104;
        case 3: return 105;
        default: return 114;
    }
}

GLS_DI void i128_add(I128& a, const I128& b) {
    const unsigned long long lo = a.lo + b.lo;
    a.hi += b.hi + (lo < a.lo ? 1ull : 0ull);
    a.lo = lo;
}

GLS_DI I128 i128_neg(I128 a) {
    a.lo = ~a.lo + 1ull;
    a.hi = ~a.hi + (a.lo == 0ull ? 1ull : 0ull);
    return a;
}

// x * 2^R rounded to the nearest integer, ties to even.  x is finite with |x| * 2^R < 2^127
// (a larger x is clamped to that range; the column bounds rule it out).
GLS_DI I128 f32_to_fixed(float x, int R) {
    const unsigned b = __float_as_uint(x);
    const int ef = (int)((b >> 23) & 0xffu);
    unsigned long long m = b & 0x7fffffu;
    if (ef != 0) m |= 0x800000ull;
    int s = (ef == 0 ? -149 : ef - 150) + R;  // |x| * 2^R = m * 2^s, m < 2^24
    if (s > 103) s = 103;
    I128 r{0ull, 0ull};
    if (m == 0ull) return r;
    if (s >= 64) {
        r.hi = m << (s - 64);
    } else if (s > 0) {
        r.lo = m << s;
        r.hi = m >> (64 - s);
    } else if (s == 0) {
        r.lo = m;
    } else if (s > -25) {
        const int k = -s;
        unsigned long long q = m >> k;
        const unsigned long long rem = m & ((1ull << k) - 1ull), half = 1ull << (k - 1);
        if (rem > half || (rem == half && (q & 1ull))) q++;
        r.lo = q;
    }  // else m * 2^s < 1/2: rounds to 0
    return (b >> 31) ? i128_neg(r) : r;
}

GLS_DI double pow2_d(int e) { return __longlong_as_double((long long)(e + 1023) << 52); }  // |e| <= 1022

// a * 2^-R rounded once to the nearest double (ties to even)
GLS_DI double fixed_to_f64(I128 a, int R) {
    const bool neg = (long long)a.hi < 0;
    if (neg) a = i128_neg(a);
    double d;
    if (a.hi == 0ull) {
        d = __ull2double_rn(a.lo);
    } else {
        // the top 64 bits, with every lower bit folded into a sticky bit 0, round as the
        // full value does (64 bits keep the 53 of the double plus guard and round bits)
        const int lz = __clzll((long long)a.hi);
        const unsigned long long top = lz ? (a.hi << lz) | (a.lo >> (64 - lz)) : a.hi;
        const unsigned long long rest = lz ? a.lo << lz : a.lo;
        d = __ull2double_rn(top | (rest ? 1ull : 0ull)) * pow2_d(64 - lz);
    }
    d *= pow2_d(-R);
    return neg ? -d : d;
}

// A block's 128-bit sum added to a column's running total as three limbs: bits 0-39 and
// 40-79 (unsigned) and bits 80-127 (signed).  With at most kNlfMaxBlocks (2^10) blocks the
// two low limbs stay below 2^50, and the high limb's total is within one of the column total
// / 2^80 (below 2^46 in magnitude by the column bounds), so no limb overflows and the
// totals are exact whatever the order of the atomics.
GLS_DI void tot_add(unsigned long long* limb, I128 v) {
    const unsigned long long m40 = (1ull << 40) - 1ull;
    atomicAdd(limb + 0, v.lo & m40);
    atomicAdd(limb + 1, ((v.lo >> 40) | (v.hi << 24)) & m40);
    atomicAdd(limb + 2, (unsigned long long)((long long)v.hi >> 16));
}

GLS_DI I128 tot_get(const unsigned long long* limb) {
    const unsigned long long l0 = __ldcg(limb), l1 = __ldcg(limb + 1), l2 = __ldcg(limb + 2);
    I128 t{l0, 0ull};
    i128_add(t, I128{l1 << 40, l1 >> 24});
    i128_add(t, I128{0ull, l2 << 16});
    return t;
}

GLS_DI I128 warp_sum_i128(I128 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        I128 w;
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        i128_add(v, w);
    }
    return v;
}

constexpr int kWarps = kThreads / 32;

// One fixed-point column of the block's row: lane 0 of each warp leaves its warp's sum in
// red[warp][k]; a NaN or infinite pair sets bit k of nan instead of being summed.
template <int K>
GLS_DI void fixed_column(const FF& f, int k, I128 (&red)[kWarps][K], unsigned& nan) {
    const bool bad = !(isfinite(f.hi) && isfinite(f.lo));
    I128 v{0ull, 0ull};
    if (!bad) {
        const int R = fixed_scale(k);
        v = f32_to_fixed(f.hi, R);
        i128_add(v, f32_to_fixed(f.lo, R));
    }
    v = warp_sum_i128(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
    if (bad) nan |= 1u << k;
}

// Per-thread accumulator of passes 1 and 3.  Fixed-point record: [0] N, then per channel
// c at 1+5c: sx, sxx, sy, sxy, syy.  Float record (pass 1): [0..2NC) minimum of (m_c, v_c),
// [2NC..4NC) maximum.  All threads of the block must call the write functions.
template <int MC, int NC>
struct Pass1Acc {
    static constexpr int NM = (MC == 1) ? 1 : NC;
    static constexpr int K = 1 + 5 * NC;
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

    // a pixel already known to be selected
    GLS_DI void add_selected(const float* m, const float* v) {
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

    GLS_DI void add(const float* m, const float* v, const NlfThresholds& th) {
        if (in_range<MC, NC>(m, v, th)) add_selected(m, v);
    }

    // The block's fixed-point sums (threads < K) and NaN mask (thread 0) added to the totals.
    GLS_DI void write_fixed(const NlfScratch& s) const {
        __shared__ I128 red[kWarps][K];
        __shared__ unsigned nanw[kWarps];
        unsigned nan = 0;
        {
            I128 c0{(unsigned long long)n, 0ull};
            c0 = warp_sum_i128(c0);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][0] = c0;
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const int cm = MC == 1 ? 0 : c;
            fixed_column<K>(sx[cm], 1 + 5 * c + 0, red, nan);
            fixed_column<K>(sxx[cm], 1 + 5 * c + 1, red, nan);
            fixed_column<K>(sy[c], 1 + 5 * c + 2, red, nan);
            fixed_column<K>(sxy[c], 1 + 5 * c + 3, red, nan);
            fixed_column<K>(syy[c], 1 + 5 * c + 4, red, nan);
        }
        nan = __reduce_or_sync(0xffffffffu, nan);
        if ((threadIdx.x & 31) == 0) nanw[threadIdx.x >> 5] = nan;
        __syncthreads();
        if (threadIdx.x < K) {
            I128 t = red[0][threadIdx.x];
#pragma unroll
            for (int w = 1; w < kWarps; w++) i128_add(t, red[w][threadIdx.x]);
            tot_add(s.tot_limb + 3 * threadIdx.x, t);
        }
        if (threadIdx.x == 0) {
            unsigned m = 0;
#pragma unroll
            for (int w = 0; w < kWarps; w++) m |= nanw[w];
            if (m) atomicOr(s.tot_nan, m);
        }
        __syncthreads();
    }

    GLS_DI void write_minmax(const NlfScratch& s) { block_minmax_atomic<2 * NC>(mn, mx, s.tot_mm); }
};

// The raw fit's pass-1 accumulator with the four channels as two packed pairs (0, 1) and
// (2, 3): the same float-float sums as Pass1Acc<4, 4>, pixel by pixel in the same order, at
// half the instructions; unpack() hands them to Pass1Acc's writers.
struct RawPass1Acc2 {
    FF2 sx[2], sxx[2], sy[2], sxy[2], syy[2];
    float mn[8], mx[8];
    int n;

    GLS_DI void init() {
#pragma unroll
        for (int p = 0; p < 2; p++) {
            ff2_zero(sx[p]);
            ff2_zero(sxx[p]);
            ff2_zero(sy[p]);
            ff2_zero(sxy[p]);
            ff2_zero(syy[p]);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            mn[k] = glsm::inf_();
            mx[k] = -glsm::inf_();
        }
        n = 0;
    }

    // m[p], v[p]: the statistics of channels 2p, 2p + 1 of a selected quad
    GLS_DI void add_selected(const float2 (&m)[2], const float2 (&v)[2]) {
        n++;
#pragma unroll
        for (int p = 0; p < 2; p++) {
            ff2_add(sx[p], m[p]);
            ff2_add_prod(sxx[p], m[p], m[p]);
            ff2_add(sy[p], v[p]);
            ff2_add_prod(sxy[p], m[p], v[p]);
            ff2_add_prod(syy[p], v[p], v[p]);
            mn[2 * p] = fminf(mn[2 * p], m[p].x);
            mx[2 * p] = fmaxf(mx[2 * p], m[p].x);
            mn[2 * p + 1] = fminf(mn[2 * p + 1], m[p].y);
            mx[2 * p + 1] = fmaxf(mx[2 * p + 1], m[p].y);
            mn[4 + 2 * p] = fminf(mn[4 + 2 * p], v[p].x);
            mx[4 + 2 * p] = fmaxf(mx[4 + 2 * p], v[p].x);
            mn[5 + 2 * p] = fminf(mn[5 + 2 * p], v[p].y);
            mx[5 + 2 * p] = fmaxf(mx[5 + 2 * p], v[p].y);
        }
    }

    GLS_DI void unpack(Pass1Acc<4, 4>& a) const {
        auto put = [](FF& lo_ch, FF& hi_ch, const FF2& f) {
            lo_ch.hi = f.hi.x;
            lo_ch.lo = f.lo.x;
            hi_ch.hi = f.hi.y;
            hi_ch.lo = f.lo.y;
        };
#pragma unroll
        for (int p = 0; p < 2; p++) {
            put(a.sx[2 * p], a.sx[2 * p + 1], sx[p]);
            put(a.sxx[2 * p], a.sxx[2 * p + 1], sxx[p]);
            put(a.sy[2 * p], a.sy[2 * p + 1], sy[p]);
            put(a.sxy[2 * p], a.sxy[2 * p + 1], sxy[p]);
            put(a.syy[2 * p], a.syy[2 * p + 1], syy[p]);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            a.mn[k] = mn[k];
            a.mx[k] = mx[k];
        }
        a.n = n;
    }
};

// The level fits' pass-1 accumulator (one mean, three variances) with the sums packed in
// pairs of independent accumulators: (sx, sy2), (sxx, syy2), (sy0, sy1), (sxy0, sxy1),
// (syy0, syy1), and sxy2 alone -- the same float-float sums as Pass1Acc<1, 3>, pixel by
// pixel in the same order; unpack() hands them to Pass1Acc's writers.
struct LevelPass1Acc2 {
    FF2 a_sx_sy2, a_sxx_syy2, a_sy01, a_sxy01, a_syy01;
    FF sxy2;
    float mn[6], mx[6];
    int n;

    GLS_DI void init() {
        ff2_zero(a_sx_sy2);
        ff2_zero(a_sxx_syy2);
        ff2_zero(a_sy01);
        ff2_zero(a_sxy01);
        ff2_zero(a_syy01);
        ff_zero(sxy2);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            mn[k] = glsm::inf_();
            mx[k] = -glsm::inf_();
        }
        n = 0;
    }

    GLS_DI void add_selected(float m, float2 v01, float v2) {
        n++;
        const float2 mv2 = make_float2(m, v2);
        ff2_add(a_sx_sy2, mv2);
        ff2_add_prod(a_sxx_syy2, mv2, mv2);
        ff2_add(a_sy01, v01);
        ff2_add_prod(a_sxy01, make_float2(m, m), v01);
        ff2_add_prod(a_syy01, v01, v01);
        ff_add_prod(sxy2, m, v2);
        const float vv[3] = {v01.x, v01.y, v2};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            mn[c] = fminf(mn[c], m);
            mx[c] = fmaxf(mx[c], m);
            mn[3 + c] = fminf(mn[3 + c], vv[c]);
            mx[3 + c] = fmaxf(mx[3 + c], vv[c]);
        }
    }

    GLS_DI void unpack(Pass1Acc<1, 3>& a) const {
        auto lane = [](FF& d, const FF2& f, int k) {
            d.hi = k ? f.hi.y : f.hi.x;
            d.lo = k ? f.lo.y : f.lo.x;
        };
        lane(a.sx[0], a_sx_sy2, 0);
        lane(a.sy[2], a_sx_sy2, 1);
        lane(a.sxx[0], a_sxx_syy2, 0);
        lane(a.syy[2], a_sxx_syy2, 1);
        lane(a.sy[0], a_sy01, 0);
        lane(a.sy[1], a_sy01, 1);
        lane(a.sxy[0], a_sxy01, 0);
        lane(a.sxy[1], a_sxy01, 1);
        lane(a.syy[0], a_syy01, 0);
        lane(a.syy[1], a_syy01, 1);
        a.sxy[2] = sxy2;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            a.mn[k] = mn[k];
            a.mx[k] = mx[k];
        }
        a.n = n;
    }
};

// Ticket of a pass: true in the one block that finishes last, once every block's row is
// visible to it.  No block ever waits for another.
GLS_DI bool last_block(unsigned* ticket) {
    __shared__ unsigned s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    const bool last = s_last != 0u;
    if (last) __threadfence();
    return last;
}

// std::max(v, a) as gls::max(DVector, double) evaluates it (gls_linalg.hpp:238-243)
__device__ double refmax(double v, double a) { return (v < a) ? a : v; }

__device__ void neumaier(double& s, double& c, double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// The regression step (thread 0) from the column totals.  Stage 1 fits the pass-1 sums and
// decides whether the explicit passes 2 and 3 are needed: it bounds every pass-1 residual
// by the extremes of the selected statistics and, when even the largest possible squared
// residual is below a lower bound of the RMS residual (computed from the sums), pass 3
// provably keeps every pass-1 pixel and the pass-1 fit is final.  Stage 3 fits the refit sums.
template <int NC>
__device__ void fit_totals(const double* tot, const float* fmm, int stage, NlfFit* fit, float* out) {
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
}

// Solve of pass 1 (stage 1) or pass 3 (stage 3), run by the last block of the pass: exact
// column totals over the nblocks rows (warp w sums columns w, w + 8, ...), NaN masks, the
// pass-1 extremes, then the fit.  Leaves the ticket at zero for the next pass.
template <int NC>
GLS_DI void solve_fixed(const NlfScratch& s, int stage, float* out) {
    constexpr int K = 1 + 5 * NC;
    __shared__ double tot[K];
    __shared__ float fmm[4 * NC];
    __shared__ unsigned nan;
    if (threadIdx.x < K) tot[threadIdx.x] = fixed_to_f64(tot_get(s.tot_limb + 3 * threadIdx.x), fixed_scale(threadIdx.x));
    if (stage == 1 && threadIdx.x >= 32 && threadIdx.x < 32 + 4 * NC) {
        const int k = threadIdx.x - 32;
        const unsigned u = __ldcg(s.tot_mm + k);
        fmm[k] = k < 2 * NC ? tot_min(u) : tot_max(u);
    }
    if (threadIdx.x == 64) nan = __ldcg(s.tot_nan);
    __syncthreads();
    // the totals are read: leave them (and the ticket) at zero for the next pass
    if (threadIdx.x < 3 * K) s.tot_limb[threadIdx.x] = 0ull;
    if (stage == 1 && threadIdx.x >= 96 && threadIdx.x < 96 + 4 * NC) s.tot_mm[threadIdx.x - 96] = 0u;
    if (threadIdx.x == 0) {
        *s.tot_nan = 0u;
        for (int k = 0; k < K; k++)
            if (nan & (1u << k)) tot[k] = __longlong_as_double(0x7ff8000000000000ll);
        fit_totals<NC>(tot, fmm, stage, s.fit, out);
        atomicExch(s.ticket, 0u);
    }
}

// Solve of pass 2, run by its last block: RMS of the residuals per channel, evaluated with
// sqrtf as gls::sqrt(Vector) does.
template <int NC>
GLS_DI void solve_pass2(const NlfScratch& s, int nblocks) {
    __shared__ double tot[NC];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = warp; k < NC; k += kWarps) {
        double sum = 0.0, c = 0.0;
        for (int b = lane; b < nblocks; b += 32) neumaier(sum, c, __ldcg(s.part_d + (size_t)b * kNlfK + k));
        const double v = warp_sum_d(sum + c);
        if (lane == 0) tot[k] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int ch = 0; ch < NC; ch++) s.fit->err2[ch] = (double)sqrtf((float)(tot[ch] / s.fit->N1));
        s.fit->mode = 2;
        atomicExch(s.ticket, 0u);
    }
}

// End of every pass-1 kernel: the block's rows, then the solve in the last block.
template <int MC, int NC>
GLS_DI void pass1_epilogue(Pass1Acc<MC, NC>& acc, const NlfScratch& s, float* out) {
    acc.write_fixed(s);
    acc.write_minmax(s);
    if (last_block(s.ticket)) solve_fixed<NC>(s, 1, out);
}

template <int MC, int NC, class Src>
__global__ void __launch_bounds__(kThreads) nlf_pass1_kernel(Src src, int sw, int sh, NlfThresholds th,
                                                             NlfScratch s, float* out) {
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
    pass1_epilogue<MC, NC>(acc, s, out);
}

// Explicit pass 2 (only when solve 1 could not prove pass 3 trivial): sum of squared
// residuals per channel, FP64 per pixel as the reference computes it.
template <int MC, int NC, class Src>
__global__ void __launch_bounds__(kThreads) nlf_pass2_kernel(Src src, int sw, int sh, NlfThresholds th,
                                                             NlfScratch s) {
    if (s.fit->mode != 1) return;
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
            const double d = (s.fit->A[c] + s.fit->B[c] * (double)m[MC == 1 ? 0 : c]) - (double)v[c];
            acc[c] += d * d;
        }
    }
    block_reduce_write<NC>(acc, s.part_d + (size_t)blockIdx.x * kNlfK);
    if (last_block(s.ticket)) solve_pass2<NC>(s, gridDim.x);
}

// Explicit pass 3: refit on the pixels whose squared residual (FP64) is <= err2 in every
// channel.
template <int MC, int NC, class Src>
__global__ void __launch_bounds__(kThreads) nlf_pass3_kernel(Src src, int sw, int sh, NlfThresholds th,
                                                             NlfScratch s, float* out) {
    if (s.fit->mode != 2) return;
    Pass1Acc<MC, NC> acc;
    acc.init();
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
            const double d = (s.fit->A[c] + s.fit->B[c] * (double)m[MC == 1 ? 0 : c]) - (double)v[c];
            if (!(d * d <= s.fit->err2[c])) ok = false;
        }
        if (ok) acc.add_selected(m, v);
    }
    acc.write_fixed(s);
    if (last_block(s.ticket)) solve_fixed<NC>(s, 3, out);
}

// The explicit passes 2 and 3 of several level fits in one launch each: every block takes
// its share of every level whose fit needs the pass (the same per-level rows, tickets and
// solves as the one-level kernels; a level whose solve proved the pass redundant is
// skipped by every block alike).
template <class S>
struct LevelSet {
    LevelSrc<S> src[GLS_MAX_LEVELS];
    NlfScratch s[GLS_MAX_LEVELS];
    float* out[GLS_MAX_LEVELS];
    int n;
};

template <class S>
__global__ void __launch_bounds__(kThreads) nlf_pass2_levels_kernel(const __grid_constant__ LevelSet<S> ls,
                                                                    NlfThresholds th) {
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    for (int l = 0; l < ls.n; l++) {
        const NlfScratch& s = ls.s[l];
        if (s.fit->mode != 1) continue;
        const LevelSrc<S>& src = ls.src[l];
        const int sw = src.img.w, sh = src.img.h;
        double acc[3] = {0.0, 0.0, 0.0};
        const int tiles_x = (sw + kTX - 1) / kTX, tiles_y = (sh + kTY - 1) / kTY;
        for (int t = blockIdx.x; t < tiles_x * tiles_y; t += gridDim.x) {
            const int x = (t % tiles_x) * kTX + tx, y = (t / tiles_x) * kTY + ty;
            if (x >= sw || y >= sh) continue;
            float m[1], v[3];
            src.stats(x, y, m, v);
            if (!in_range<1, 3>(m, v, th)) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double d = (s.fit->A[c] + s.fit->B[c] * (double)m[0]) - (double)v[c];
                acc[c] += d * d;
            }
        }
        block_reduce_write<3>(acc, s.part_d + (size_t)blockIdx.x * kNlfK);
        if (last_block(s.ticket)) solve_pass2<3>(s, gridDim.x);
        __syncthreads();
    }
}

template <class S>
__global__ void __launch_bounds__(kThreads) nlf_pass3_levels_kernel(const __grid_constant__ LevelSet<S> ls,
                                                                    NlfThresholds th) {
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    for (int l = 0; l < ls.n; l++) {
        const NlfScratch& s = ls.s[l];
        if (s.fit->mode != 2) continue;
        const LevelSrc<S>& src = ls.src[l];
        const int sw = src.img.w, sh = src.img.h;
        Pass1Acc<1, 3> acc;
        acc.init();
        const int tiles_x = (sw + kTX - 1) / kTX, tiles_y = (sh + kTY - 1) / kTY;
        for (int t = blockIdx.x; t < tiles_x * tiles_y; t += gridDim.x) {
            const int x = (t % tiles_x) * kTX + tx, y = (t / tiles_x) * kTY + ty;
            if (x >= sw || y >= sh) continue;
            float m[1], v[3];
            src.stats(x, y, m, v);
            if (!in_range<1, 3>(m, v, th)) continue;
            bool ok = true;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double d = (s.fit->A[c] + s.fit->B[c] * (double)m[0]) - (double)v[c];
                if (!(d * d <= s.fit->err2[c])) ok = false;
            }
            if (ok) acc.add_selected(m, v);
        }
        acc.write_fixed(s);
        if (last_block(s.ticket)) solve_fixed<3>(s, 3, ls.out[l]);
        __syncthreads();
    }
}

int grid_for(gls_ctx* ctx, int sw, int sh) {
    const long tiles = (long)((sw + kTX - 1) / kTX) * ((sh + kTY - 1) / kTY);
    long g = 4L * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    if (g > kNlfMaxBlocks) g = kNlfMaxBlocks;
    if (g > tiles) g = tiles;
    return (int)(g < 1 ? 1 : g);
}

// Everything after pass 1 (whose last block already solved it): the explicit error and
// refit passes, which exit at once unless solve 1 could not prove them redundant.
template <int MC, int NC, class Src>
void nlf_finish(gls_ctx* ctx, const Src& src, int sw, int sh, NlfScratch s, float* out_dev) {
    const NlfThresholds th = nlf_thresholds();
    const int grid = grid_for(ctx, sw, sh);
    cudaStream_t st = ctx->stream;
    nlf_pass2_kernel<MC, NC, Src><<<grid, kThreads, 0, st>>>(src, sw, sh, th, s);
    nlf_pass3_kernel<MC, NC, Src><<<grid, kThreads, 0, st>>>(src, sw, sh, th, s, out_dev);
    ctx->launches += 2;
}

template <int MC, int NC, class Src>
gls_status run_fit(gls_ctx* ctx, const Src& src, int sw, int sh, NlfScratch s, float* out_dev) {
    const NlfThresholds th = nlf_thresholds();
    const int grid = grid_for(ctx, sw, sh);
    // the scratch may have held other data (the context's scratch is shared): clear the
    // ticket and the running totals
    GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(s.ticket, 0, kNlfHeaderBytes - kNlfTicketOff, ctx->stream),
                         "clear regression state"));
    nlf_pass1_kernel<MC, NC, Src><<<grid, kThreads, 0, ctx->stream>>>(src, sw, sh, th, s, out_dev);
    ctx->launches += 1;
    nlf_finish<MC, NC, Src>(ctx, src, sw, sh, s, out_dev);
    return check_launch(ctx, "noise model regression");
}

}  // namespace
}  // namespace gls

#endif  // GLS_NLF_CUH
