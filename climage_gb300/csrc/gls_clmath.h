// Copyright (c) 2026 gls-cuda authors. Licensed under the Apache License, Version 2.0.
//
// gls_clmath.h -- the OpenCL C built-in functions used by the RAW pipeline kernels,
// with their semantics fixed once for every compiler that builds this project.
//
// The reference kernels (CLImage/app/src/main/cpp/OpenCL/demosaic.cl) are built with
// -cl-fast-relaxed-math (src/gls_cl.cpp:161-165), so their transcendentals, min/max on
// signed zeros and texture filtering are implementation-defined.  This header pins one
// definition of each built-in so that the CUDA kernels and the CPU restatement produce
// bit-identical float results:
//
//   * arithmetic is IEEE-754 binary32 with round-to-nearest-even, no contraction of
//     a*b+c into fused multiply-add (nvcc --fmad=false, g++ -ffp-contract=off);
//   * sqrt and division are correctly rounded (nvcc -prec-sqrt=true -prec-div=true);
//   * atan2pi, tanh, exp2, log2 and pow are evaluated by the polynomial approximations
//     below, derived by climage_gb300/csrc/fit_clmath_coeffs.py (Lawson-refined
//     least squares on Chebyshev nodes), using only +, -, *, / and exact bit operations;
//   * min/max/clamp follow the OpenCL fmin/fmax rules (a NaN operand yields the other
//     operand) and, for equal operands, return the first one;
//   * float -> half conversion rounds to nearest even (what write_imageh / half image
//     storage does), with overflow to infinity.
//
// Accuracy of the approximations against correctly rounded results is checked by
// tests/test_clmath.py (a few ulp); nothing in this header calls the platform libm
// for a transcendental.
#ifndef GLS_CLMATH_H
#define GLS_CLMATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#include <cuda_fp16.h>
#endif

#if defined(__CUDACC__)
#define GLS_HD __host__ __device__ __forceinline__
#define GLS_HDM __host__ __device__ __forceinline__
#define GLS_HDN static __host__ __device__ __noinline__
#else
#define GLS_HD static inline
#define GLS_HDM inline
#define GLS_HDN static __attribute__((noinline))
#endif

namespace glsm {

GLS_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

GLS_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

GLS_HD bool isnan_(float x) { return x != x; }
GLS_HD float inf_() { return u2f(0x7f800000u); }
GLS_HD float nan_() { return u2f(0x7fc00000u); }
GLS_HD bool signbit_(float x) { return (f2u(x) >> 31) != 0; }
GLS_HD float fabs_(float x) { return u2f(f2u(x) & 0x7fffffffu); }
GLS_HD float copysign_(float x, float s) { return u2f((f2u(x) & 0x7fffffffu) | (f2u(s) & 0x80000000u)); }

GLS_HD float sqrt_(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return __builtin_sqrtf(x);
#endif
}

GLS_HD float div_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

GLS_HD float floor_(float x) {
#if defined(__CUDA_ARCH__)
    return floorf(x);
#else
    return __builtin_floorf(x);
#endif
}

GLS_HD float rint_(float x) {
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return __builtin_rintf(x);
#endif
}

// OpenCL fmax/fmin: a NaN argument yields the other argument; ties keep the first.
GLS_HD float fmax_(float a, float b) { return isnan_(a) ? b : (isnan_(b) ? a : (a < b ? b : a)); }
GLS_HD float fmin_(float a, float b) { return isnan_(a) ? b : (isnan_(b) ? a : (b < a ? b : a)); }

// OpenCL clamp(x, lo, hi) == fmin(fmax(x, lo), hi)
GLS_HD float clamp_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }

// OpenCL mix(x, y, a) == x + (y - x) * a
GLS_HD float mix_(float x, float y, float a) { return x + (y - x) * a; }

// OpenCL step(edge, x): 0 when x < edge, else 1 -- evaluated as x >= edge ? 1 : 0, which is
// the same function for every non-NaN x.  The reference is compiled with
// -cl-finite-math-only, so its result for a NaN x is undefined; this reading (NaN -> 0)
// keeps the bilateral weights finite where the fitted noise model gives a negative
// variance or a zero raw sample gives 0/0 (demosaic.cl:757, 940).
GLS_HD float step_(float edge, float x) { return x >= edge ? 1.0f : 0.0f; }

// OpenCL smoothstep(e0, e1, x): t = clamp((x - e0) / (e1 - e0), 0, 1); t * t * (3 - 2 * t)
GLS_HD float smoothstep_ref(float e0, float e1, float x) {
    float t = clamp_(div_(x - e0, e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// ---- exact shortcuts (results identical to the literal expressions) ----

GLS_HD float fma_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}

GLS_HD float rcp_(float d) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(d);
#else
    return 1.0f / d;
#endif
}

// the literal division, out of line (the rare paths of the shortcuts below)
GLS_HDN float div_slow(float a, float b) { return div_(a, b); }

// RN(1/d) for |d| in [2^-60, 2^30]: the hardware's reciprocal approximation refined by one
// Newton-Raphson step, r + r (1 - d r) with both operations fused.  Equal to the correctly
// rounded reciprocal for every d in that range (checked exhaustively against __frcp_rn on the
// GPU by gls_selftest_reciprocal), at three instructions.
GLS_HD float rcp_fast(float d) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(d));
    return __fmaf_rn(__fmaf_rn(-d, r, 1.0f), r, r);
#else
    return 1.0f / d;
#endif
}

// Division by a value shared by many numerators.  With y = RN(1/d) and q0 = RN(x*y), the
// residual r = x - q0*d is exact and RN(q0 + r*y) is the correctly rounded x/d
// (Markstein's correction, P. Markstein, "IA-64 and Elementary Functions", 2000); the
// shortcut is taken only where no intermediate can overflow or underflow, and zero, NaN
// and infinite numerators take the literal division.
struct FastDiv {
    float d, y;
    bool ok;
    // divisor range [2^-60, 2^30] and numerator range {0} u [2^-83, 2^60] keep the quotient
    // in [2^-113, 2^120] and the residual above 2^-107: every intermediate is normal
    GLS_HDM void init(float den) {
        d = den;
        const float ad = fabs_(den);
        ok = ad >= 8.67361738e-19f && ad <= 1073741824.0f;
        y = ok ? rcp_fast(den) : 0.0f;
    }
    // a divisor known in advance: y = RN(1/den) and ok as init() computes them
    GLS_HDM static FastDiv of(float den, float rcp, bool in_range) {
        FastDiv f;
        f.d = den;
        f.y = rcp;
        f.ok = in_range;
        return f;
    }
    GLS_HDM float operator()(float x) const {
        if (!ok || !in_range(x)) return div_slow(x, d);
        return fast(x);
    }
    // the shortcut alone: exact when ok and in_range(x) (x == 0 gives a zero of either sign)
    GLS_HDM float fast(float x) const {
        const float q0 = x * y;
        const float r = fma_(-q0, d, x);
        return fma_(r, y, q0);
    }
    GLS_HDM static bool in_range(float x) {
        const float ax = fabs_(x);
        return ax <= 1.15292150e18f && (ax >= 1.03397577e-25f || ax == 0.0f);
    }
};

// smoothstep with the interpolation denominator e1 - e0 shared by many evaluations: the
// division is only evaluated where the clamp does not decide the result by itself
// (num <= 0 or NaN clamps to 0, num >= den > 0 clamps to 1, exactly as the literal form).
// out-of-line literal operations for the rare paths (keeps the unrolled loops compact)
GLS_HDN float sqrt_slow(float a) { return sqrt_(a); }
GLS_HDN float smoothstep_slow(float num, float den) {
    const float t = clamp_(div_(num, den), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

GLS_HD float smoothstep_den(float e0, const FastDiv& den, float x) {
    const float num = x - e0;
    if (!(den.ok && den.d > 0.0f)) return smoothstep_slow(num, den.d);
    // 0 < num < den <= 2^60: num >= 2^-60 makes the shortcut exact
    const float t = !(num > 0.0f) ? 0.0f
                    : (num >= den.d ? 1.0f : (num >= 8.67361738e-19f ? den.fast(num) : div_slow(num, den.d)));
    return t * t * (3.0f - 2.0f * t);
}

// smoothstep(e0, e1, x), identical to smoothstep_ref, skipping the division when the
// clamp decides the value.
GLS_HD float smoothstep_(float e0, float e1, float x) {
    const float den = e1 - e0;
    const float num = x - e0;
    if (!(den > 0.0f && den <= 3.4e38f)) return smoothstep_slow(num, den);
    const float t = !(num > 0.0f) ? 0.0f : (num >= den ? 1.0f : div_slow(num, den));
    return t * t * (3.0f - 2.0f * t);
}

// sqrt_rn(q) >= e decided without the square root when q is clearly on one side of e^2
// (|q - e^2| > 2^-20 e^2); e must be positive and moderate, otherwise the literal test.
struct SqrtGe {
    float e, lo, hi;
    bool ok;
    GLS_HDM void init(float edge) {
        e = edge;
        ok = edge > 1e-15f && edge < 1e15f;
        const float t = edge * edge;
        lo = t * (1.0f - 9.5367431640625e-07f);  // 1 - 2^-20, exact
        hi = t * (1.0f + 9.5367431640625e-07f);  // 1 + 2^-20, exact
    }
    // returns sqrt_rn(q) >= e (false for NaN q)
    GLS_HDM bool operator()(float q) const {
        if (ok) {
            if (q < lo) return false;
            if (q > hi) return true;
        }
        return sqrt_slow(q) >= e;
    }
    // true when q is close enough to e^2 that only the literal test decides
    GLS_HDM bool ambiguous(float q) const { return q >= lo && q <= hi; }
};

// The reference's own min/max/abs macros (demosaic.cl:56-65): plain selects.
GLS_HD float mmin(float a, float b) { return a < b ? a : b; }
GLS_HD float mmax(float a, float b) { return a > b ? a : b; }
GLS_HD float mabs(float a) { return a > 0 ? a : -a; }

// OpenCL length(): square root of the dot product, summed left to right.
GLS_HD float length2_(float x, float y) { return sqrt_(x * x + y * y); }
GLS_HD float length3_(float x, float y, float z) { return sqrt_(x * x + y * y + z * z); }
GLS_HD float length4_(float x, float y, float z, float w) { return sqrt_(x * x + y * y + z * z + w * w); }

// ---- binary16 storage rounding ----

// float -> IEEE binary16 bits, round to nearest even; NaN -> quiet NaN, overflow -> inf.
GLS_HD uint16_t f32_to_f16_bits(float f) {
    const uint32_t b = f2u(f);
    const uint32_t sign = (b >> 16) & 0x8000u;
    const uint32_t a = b & 0x7fffffffu;
    if (a >= 0x7f800000u) return (uint16_t)(sign | (a > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (a >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // >= 65520 rounds to inf
    if (a < 0x38800000u) {                                     // below 2^-14: subnormal half
        // |f| * 2^24 is exact and < 2^10; rint rounds to nearest even.
        const uint32_t r = (uint32_t)rint_(fabs_(f) * 16777216.0f);
        return (uint16_t)(sign | r);
    }
    uint32_t h = ((((a >> 23) - 112u) << 10) | ((a >> 13) & 0x3ffu));
    const uint32_t rem = a & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
    return (uint16_t)(sign | h);
}

GLS_HD float f16_bits_to_f32(uint16_t h) {
    const uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    const uint32_t e = ((uint32_t)h >> 10) & 0x1fu;
    const uint32_t m = (uint32_t)h & 0x3ffu;
    if (e == 0) {
        // subnormal or zero: m * 2^-24, exact in float
        const float v = (float)m * 5.9604644775390625e-8f;
        return u2f(f2u(v) | sign);
    }
    if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

// Round a float to the nearest binary16 value (as a float).
GLS_HD float round_half(float f) {
#if defined(__CUDA_ARCH__)
    return __half2float(__float2half_rn(f));
#else
    return f16_bits_to_f32(f32_to_f16_bits(f));
#endif
}

// ---- transcendentals ----

// atan2(y, x) / pi with the C99 special values.
GLS_HD float atan2pi_(float y, float x) {
    if (isnan_(x) || isnan_(y)) return x + y;
    const float ax = fabs_(x), ay = fabs_(y);
    const bool xneg = signbit_(x);
    float r;
    if (ay == 0.0f) {
        r = xneg ? 1.0f : 0.0f;
    } else if (ax == 0.0f) {
        r = 0.5f;
    } else if (ax == inf_() && ay == inf_()) {
        r = xneg ? 0.75f : 0.25f;
    } else if (ax == inf_()) {
        r = xneg ? 1.0f : 0.0f;
    } else if (ay == inf_()) {
        r = 0.5f;
    } else {
        const bool swap = ay > ax;
        const float a = swap ? div_(ax, ay) : div_(ay, ax);
        const float s = a * a;
        float p = -5.582857679e-04f;
        p = p * s + 3.414458497e-03f;
        p = p * s + -9.805344525e-03f;
        p = p * s + 1.831933928e-02f;
        p = p * s + -2.666578585e-02f;
        p = p * s + 3.482955246e-02f;
        p = p * s + -4.539714054e-02f;
        p = p * s + 6.365645763e-02f;
        p = p * s + -1.061031372e-01f;
        p = p * s + 3.183098854e-01f;
        r = a * p;
        if (swap) r = 0.5f - r;
        if (xneg) r = 1.0f - r;
    }
    return copysign_(r, y);
}

// 2^x on (-126, 126), where no special case applies: n = x rounded to an integer, the
// polynomial on the fraction, and an exact scaling by 2^n (the general form below, bit for bit)
GLS_HD float exp2_core(float x) {
    const float n = floor_(x + 0.5f);
    const float f = x - n;  // [-0.5, 0.5], exact
    float p = 1.534580750e-04f;
    p = p * f + 1.339993118e-03f;
    p = p * f + 9.618488974e-03f;
    p = p * f + 5.550328777e-02f;
    p = p * f + 2.402264689e-01f;
    p = p * f + 6.931472057e-01f;
    p = p * f + 1.000000001e+00f;
    return p * u2f((uint32_t)((int)n + 127) << 23);
}

// 2^x
// the special cases and the edge of the range, out of line (the kernels rarely reach them)
GLS_HDN float exp2_slow(float x) {
    if (isnan_(x)) return x;
    if (x >= 128.0f) return inf_();
    if (x < -150.0f) return 0.0f;
    const float n = floor_(x + 0.5f);
    const float f = x - n;  // [-0.5, 0.5], exact
    float p = 1.534580750e-04f;
    p = p * f + 1.339993118e-03f;
    p = p * f + 9.618488974e-03f;
    p = p * f + 5.550328777e-02f;
    p = p * f + 2.402264689e-01f;
    p = p * f + 6.931472057e-01f;
    p = p * f + 1.000000001e+00f;
    int e = (int)n;
    if (e > 127) {
        p = p * 2.0f;
        e -= 1;
    }
    if (e < -126) {
        // scale in two exact steps to reach the subnormal range
        p = p * u2f((uint32_t)(e + 126 + 127) << 23);
        return p * u2f((uint32_t)(-126 + 127) << 23);
    }
    return p * u2f((uint32_t)(e + 127) << 23);
}

GLS_HD float exp2_(float x) {
    if (fabs_(x) < 126.0f) return exp2_core(x);  // NaN goes on
    return exp2_slow(x);
}

// true for a positive, normal, finite x (one unsigned compare on the bits)
GLS_HD bool is_pos_normal_(float x) { return f2u(x) - 0x00800000u < 0x7f000000u; }

// log2 of a positive normal finite x: the general form below with k = 0 (e + 0.0f == e)
GLS_HD float log2_core(float x) {
    uint32_t b = f2u(x);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = u2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float z = div_(m - 1.0f, m + 1.0f);
    const float s = z * z;
    float p = 2.381667258e-02f;
    p = p * s + 3.386064467e-01f;
    p = p * s + 4.117443166e-01f;
    p = p * s + 5.770824732e-01f;
    p = p * s + 9.617966808e-01f;
    p = p * s + 2.885390082e+00f;
    return (float)e + z * p;
}

// log2 of what is not a positive normal finite x, out of line
GLS_HDN float log2_slow(float x) {
    if (isnan_(x)) return x;
    if (x < 0.0f) return nan_();
    if (x == 0.0f) return -inf_();
    if (x == inf_()) return x;
    float k = 0.0f;
    if (x < 1.17549435e-38f) {  // subnormal: scale by 2^24 (exact)
        x = x * 16777216.0f;
        k = -24.0f;
    }
    uint32_t b = f2u(x);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = u2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float z = div_(m - 1.0f, m + 1.0f);
    const float s = z * z;
    float p = 2.381667258e-02f;
    p = p * s + 3.386064467e-01f;
    p = p * s + 4.117443166e-01f;
    p = p * s + 5.770824732e-01f;
    p = p * s + 9.617966808e-01f;
    p = p * s + 2.885390082e+00f;
    return ((float)e + k) + z * p;
}

// log2(x)
GLS_HD float log2_(float x) {
    if (is_pos_normal_(x)) return log2_core(x);
    return log2_slow(x);
}

GLS_HD bool is_integer_(float y) { return floor_(y) == y; }

// pow's special cases, out of line
GLS_HDN float pow_slow(float x, float y) {
    if (isnan_(x) || isnan_(y)) return x + y;
    if (x == 0.0f) return y < 0.0f ? inf_() : 0.0f;
    if (x < 0.0f) {
        if (!is_integer_(y)) return nan_();
        const float r = exp2_(y * log2_(-x));
        const float half_y = y * 0.5f;
        return is_integer_(half_y) ? r : -r;
    }
    if (x == inf_()) return y < 0.0f ? 0.0f : x;
    return exp2_(y * log2_(x));
}

// OpenCL pow(x, y) for the cases the pipeline meets: finite or infinite x, finite y.
GLS_HD float pow_(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    // positive normal x and finite y: the general case, without its special-case tests
    if (is_pos_normal_(x) && fabs_(y) < inf_()) return exp2_(y * log2_core(x));
    return pow_slow(x, y);
}

// OpenCL powr(x, y): defined for x >= 0 only.
GLS_HD float powr_(float x, float y) {
    if (x < 0.0f || isnan_(x) || isnan_(y)) return nan_();
    if (x == 0.0f) return y == 0.0f ? nan_() : (y < 0.0f ? inf_() : 0.0f);
    if (x == 1.0f) return 1.0f;
    if (y == 0.0f) return 1.0f;
    return exp2_(y * log2_(x));
}

// tanh(x)
GLS_HD float tanh_(float x) {
    if (isnan_(x)) return x;
    const float ax = fabs_(x);
    float r;
    if (ax < 0.625f) {
        const float s = ax * ax;
        float p = 6.422573784e-04f;
        p = p * s + 1.535835834e-03f;
        p = p * s + -8.009078423e-03f;
        p = p * s + 2.170054290e-02f;
        p = p * s + -5.395293793e-02f;
        p = p * s + 1.333328214e-01f;
        p = p * s + -3.333333306e-01f;
        r = ax + ax * (s * p);
    } else if (ax < 9.01f) {
        const float e = exp2_(ax * 2.88539008f);  // e^(2|x|)
        r = 1.0f - div_(2.0f, e + 1.0f);
    } else {
        r = 1.0f;
    }
    return copysign_(r, x);
}

// UNORM8 image write (write_imagef on CL_UNORM_INT8): convert_uchar_sat_rte(x * 255)
GLS_HD uint8_t to_unorm8(float x) {
    const float v = x * 255.0f;
    if (!(v > 0.0f)) return 0;  // NaN and negatives
    if (v >= 255.0f) return 255;
    return (uint8_t)rint_(v);
}

// UNORM16 image read (read_imagef on CL_UNORM_INT16)
GLS_HD float from_unorm16(uint16_t v) { return div_((float)v, 65535.0f); }

}  // namespace glsm

#endif  // GLS_CLMATH_H
