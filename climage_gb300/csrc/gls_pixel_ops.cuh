// gls_pixel_ops.cuh -- the per-pixel arithmetic of every stage of CLImage's RAW->RGB
// pipeline, written once and shared by the single-stage kernels (global-memory
// accessors) and the fused pipeline kernels (shared-memory tiles).
//
// Each function follows the reference kernel named in its comment operation by
// operation, in the same order, so that the result is bit-identical to the CPU
// restatement under the conventions of gls_clmath.h.  An accessor (Acc) is any type with
// `float at(int x, int y)` (single channel) or `float4 at(int x, int y)` (RGBA) that
// clamps to the image edge.
#ifndef GLS_PIXEL_OPS_CUH
#define GLS_PIXEL_OPS_CUH

#include "gls_device.cuh"
#include "gls_f32x2.cuh"

namespace gls {

using glsm::clamp_;
using glsm::div_;
using glsm::length2_;
using glsm::length3_;
using glsm::length4_;
using glsm::mabs;
using glsm::mix_;
using glsm::mmax;
using glsm::mmin;
using glsm::smoothstep_;
using glsm::sqrt_;
using glsm::step_;

#define GLS_SQRT2_F 1.41421356237309504880f
#define GLS_SQRT3_F 1.7320508f

using glsm::FastDiv;
using glsm::SqrtGe;

// x / 25 (the 5x5 box normalisation): 0.04f is RN(1/25)
GLS_DI FastDiv div25() {
    FastDiv f;
    f.d = 25.0f;
    f.y = 0.04f;
    f.ok = true;
    return f;
}

// UNORM16 read, (float)raw / 65535 correctly rounded: with y = RN(1/65535) (0x37800080) and
// q0 = RN(x * y), one Markstein correction RN(q0 + RN(x - q0 * 65535) * y) is the quotient of
// the division for every one of the 65536 inputs (checked exhaustively, on the GPU by
// test_unorm16_read_is_the_division), at three instructions instead of a division.
GLS_DI float unorm16(uint16_t raw) {
    const float x = (float)raw;
    const float y = __uint_as_float(0x37800080u);
    const float q0 = x * y;
    return glsm::fma_(glsm::fma_(-q0, 65535.0f, x), y, q0);
}

// ---- a4: scaleRawData (demosaic.cl:69-78) ----
GLS_DI float scale_value(uint16_t raw, float scale_mul, float black) {
    const float v = unorm16(raw);
    const float r = scale_mul * (v - black);
    return r > 0.0f ? r : 0.0f;
}

// ---- a5: rawNoiseStatistics + readRAWQuad (demosaic.cl:1288-1324) ----
template <class Acc>
GLS_DI void raw_stats_quad(const Acc& raw, int qx, int qy, int bayer, float mean[4], float var[4]) {
    float sum[4] = {0.0f, 0.0f, 0.0f, 0.0f}, sq[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int y = -2; y <= 2; y++) {
#pragma unroll
        for (int x = -2; x <= 2; x++) {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const float s = raw.at(2 * (qx + x) + bayer_dx(bayer, c), 2 * (qy + y) + bayer_dy(bayer, c));
                sum[c] = sum[c] + s;
                sq[c] = sq[c] + s * s;
            }
        }
    }
    const FastDiv d25 = div25();
#pragma unroll
    for (int c = 0; c < 4; c++) {
        mean[c] = d25(sum[c]);
        var[c] = d25(sq[c] - d25(sum[c] * sum[c]));
    }
}

// ---- a13: noiseStatistics (demosaic.cl:1267-1286): (mean Y, var Y, var Cb, var Cr) ----
template <class Acc>
GLS_DI float4 noise_stats_px(const Acc& im, int px, int py) {
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, q0 = 0.0f, q1 = 0.0f, q2 = 0.0f;
#pragma unroll
    for (int y = -2; y <= 2; y++) {
#pragma unroll
        for (int x = -2; x <= 2; x++) {
            const float4 s = im.at(px + x, py + y);
            s0 = s0 + s.x;
            q0 = q0 + s.x * s.x;
            s1 = s1 + s.y;
            q1 = q1 + s.y * s.y;
            s2 = s2 + s.z;
            q2 = q2 + s.z * s.z;
        }
    }
    const FastDiv d25 = div25();
    float4 r;
    r.x = d25(s0);
    r.y = d25(q0 - d25(s0 * s0));
    r.z = d25(q1 - d25(s1 * s1));
    r.w = d25(q2 - d25(s2 * s2));
    return r;
}

// ---- a7: sobel / bilateralSobel / interpolateGreen (demosaic.cl:96-129, 160-227) ----
struct SobelVal {
    float gx, gy, len;  // |sobel| components and their length
};

// FINITE: the samples are finite (the fused pipeline's scaled raw tile), so each zero tap
// of the kernels adds a zero to the sum and the taps of weight +-1 and +-2 add +-s and +-2s
// exactly; the sums are evaluated with those taps only, in the kernels' order.  This can
// change only the sign of a zero sum (and so of a zero |gradient| component), which no
// value of interpolateGreen depends on: the gradient components are non-negative, a zero
// luma direction is taken where the gradient vanishes and there the direction is mixed
// away (lgt = 0).
template <bool FINITE = false, class Acc>
GLS_DI SobelVal sobel_abs(const Acc& im, int x, int y) {
    float vx = 0.0f, vy = 0.0f;
    if (FINITE) {
        const float a = im.at(x - 1, y - 1), b = im.at(x, y - 1), c = im.at(x + 1, y - 1);
        const float d = im.at(x - 1, y), f = im.at(x + 1, y);
        const float g = im.at(x - 1, y + 1), h = im.at(x, y + 1), k = im.at(x + 1, y + 1);
        vx = ((((a - c) + 2.0f * d) - 2.0f * f) + g) - k;
        vy = ((((a + 2.0f * b) + c) - g) - 2.0f * h) - k;
    } else {
        const float kx[3][3] = {{1.0f, 0.0f, -1.0f}, {2.0f, 0.0f, -2.0f}, {1.0f, 0.0f, -1.0f}};
        const float ky[3][3] = {{1.0f, 2.0f, 1.0f}, {0.0f, 0.0f, 0.0f}, {-1.0f, -2.0f, -1.0f}};
#pragma unroll
        for (int j = -1; j <= 1; j++) {
#pragma unroll
            for (int i = -1; i <= 1; i++) {
                const float s = im.at(x + i, y + j);
                vx = vx + kx[j + 1][i + 1] * s;
                vy = vy + ky[j + 1][i + 1] * s;
            }
        }
    }
    // division by sqrt(4.5) (the Sobel normalisation): 0x4007c3b6 = RN(sqrt(4.5)) and
    // 0x3ef15bf0 = RN(1 / that), the values init(sqrt_(4.5f)) computes
    const FastDiv r = FastDiv::of(__uint_as_float(0x4007c3b6u), __uint_as_float(0x3ef15bf0u), true);
    SobelVal o;
    o.gx = mabs(r(vx));
    o.gy = mabs(r(vy));
    o.len = length2_(o.gx, o.gy);
    return o;
}

// Signed sobel of a single channel (used by denoiseImage's gradient boost).
template <class Acc>
GLS_DI float2 sobel_signed(const Acc& im, int x, int y) {
    const float kx[3][3] = {{1.0f, 0.0f, -1.0f}, {2.0f, 0.0f, -2.0f}, {1.0f, 0.0f, -1.0f}};
    const float ky[3][3] = {{1.0f, 2.0f, 1.0f}, {0.0f, 0.0f, 0.0f}, {-1.0f, -2.0f, -1.0f}};
    float vx = 0.0f, vy = 0.0f;
#pragma unroll
    for (int j = -1; j <= 1; j++) {
#pragma unroll
        for (int i = -1; i <= 1; i++) {
            const float s = im.at(x + i, y + j);
            vx = vx + kx[j + 1][i + 1] * s;
            vy = vy + ky[j + 1][i + 1] * s;
        }
    }
    const FastDiv r = FastDiv::of(__uint_as_float(0x4007c3b6u), __uint_as_float(0x3ef15bf0u), true);
    return make_float2(r(vx), r(vy));
}

// sob(i, j) returns the SobelVal at offset (i, j) from the centre.
// The literal evaluation (rare: sigma outside the ranges the fast forms cover).
template <class SobF>
__device__ __noinline__ float2 bilateral_sobel_literal(const SobF& sob, float e0, float e1) {
    const SobelVal c = sob(0, 0);
    float sx = 0.0f, sy = 0.0f, ws = 0.0f;
    for (int j = -2; j <= 2; j++) {
        for (int i = -2; i <= 2; i++) {
            const SobelVal g = sob(i, j);
            const float w = 1.0f - glsm::smoothstep_ref(e0, e1, 0.05f * mabs(g.len - c.len));
            sx = sx + w * g.gx;
            sy = sy + w * g.gy;
            ws = ws + w;
        }
    }
    return make_float2(div_(sx, ws), div_(sy, ws));
}

// The weight 1 - smoothstep(e0, e1, x) of every tap is evaluated in one of two exact forms,
// chosen once per pixel:
//  - e0 >= 2^-36 and e1 - e0 in the shortcut's divisor range: x and e0 are floats, so a
//    positive x - e0 is at least 2^-60 and the shared-divisor division is exact for it;
//  - sigma = 0 (a black neighbourhood): e0 = e1 = 0 and x >= 0, so (x - 0) / 0 clamps to
//    1 for x > 0 and 0/0 to 0 (the clamp returns the bound for NaN): the weight is x == 0.
// Any other sigma (NaN, subnormal) takes the literal evaluation.
template <class SobF>
GLS_DI float2 bilateral_sobel(const SobF& sob, float sigma) {
    const float e0 = 4.0f * sigma, e1 = 16.0f * sigma;
    FastDiv den;
    den.init(e1 - e0);
    const bool fast = den.ok && den.d > 0.0f && e0 >= 1.4551915228366852e-11f;  // 2^-36
    const bool zero = e0 == 0.0f && e1 == 0.0f;
    if (!(fast || zero)) return bilateral_sobel_literal(sob, e0, e1);
    const SobelVal c = sob(0, 0);
    float2 sxy = make_float2(0.0f, 0.0f);  // (sx, sy): the products are scalar, the sums packed
    float ws = 0.0f;
    auto acc = [&](const SobelVal& g, float w) {
        sxy = add2(sxy, mul2s(make_float2(w, w), make_float2(g.gx, g.gy)));
        ws = ws + w;
    };
    if (fast) {
        // the weights of two taps at a time as packed lanes (t from the shared-divisor
        // shortcut, then 1 - t * t * (3 - 2 t) with 3 - 2 t = fma(-2, t, 3): 2 t is exact),
        // accumulated tap by tap in the reference's order (rows, then columns)
        const float2 e0v = make_float2(e0, e0), yv = make_float2(den.y, den.y), ndv = make_float2(-den.d, -den.d);
#pragma unroll
        for (int k = 0; k < 25; k += 2) {
            const bool two = k + 1 < 25;
            const SobelVal ga = sob(k % 5 - 2, k / 5 - 2);
            const SobelVal gb = two ? sob((k + 1) % 5 - 2, (k + 1) / 5 - 2) : ga;
            const float2 num = sub2(make_float2(0.05f * mabs(ga.len - c.len), 0.05f * mabs(gb.len - c.len)), e0v);
            const float2 q0 = mul2(num, yv);
            const float2 q = fma2(fma2(q0, ndv, num), yv, q0);
            const float2 t = make_float2(!(num.x > 0.0f) ? 0.0f : (num.x >= den.d ? 1.0f : q.x),
                                         !(num.y > 0.0f) ? 0.0f : (num.y >= den.d ? 1.0f : q.y));
            const float2 w = sub2(make_float2(1.0f, 1.0f),
                                  mul2s(mul2(t, t), fma2(t, make_float2(-2.0f, -2.0f), make_float2(3.0f, 3.0f))));
            acc(ga, w.x);
            if (two) acc(gb, w.y);
        }
    } else {
#pragma unroll
        for (int j = -2; j <= 2; j++) {
#pragma unroll
            for (int i = -2; i <= 2; i++) {
                const SobelVal g = sob(i, j);
                const float x = 0.05f * mabs(g.len - c.len);
                acc(g, x > 0.0f ? 0.0f : 1.0f);
            }
        }
    }
    return make_float2(div_(sxy.x, ws), div_(sxy.y, ws));
}

// True when (x, y) is a red or blue site, where green has to be interpolated.
GLS_DI bool green_needs_interp(int x, int y, int bayer) {
    const int gx = bayer_dx(bayer, raw_green), gy = bayer_dy(bayer, raw_green);
    const int x0 = (y & 1) == (gy & 1) ? gx + 1 : gx;
    return (x0 & 1) == (x & 1);
}

// Green at a red/blue site; lumaVariance already clamped to >= 1e-4.
template <class Acc, class SobF>
GLS_DI float green_at(const Acc& raw, int x, int y, float lumaVariance, const SobF& sob) {
    const float g_left = raw.at(x - 1, y), g_right = raw.at(x + 1, y);
    const float g_up = raw.at(x, y - 1), g_down = raw.at(x, y + 1);
    const float c_xy = raw.at(x, y);
    const float c_left = raw.at(x - 2, y), c_right = raw.at(x + 2, y);
    const float c_up = raw.at(x, y - 2), c_down = raw.at(x, y + 2);
    const float c2_tl = raw.at(x - 1, y - 1), c2_tr = raw.at(x + 1, y - 1);
    const float c2_bl = raw.at(x - 1, y + 1), c2_br = raw.at(x + 1, y + 1);
    const float c2_ave = ((c2_tl + c2_tr + c2_bl + c2_br) * 0.25f);

    const float g_ave = ((g_left + g_right + g_up + g_down) * 0.25f);
    const float lumaStdDev = sqrt_(lumaVariance * g_ave);
    const float2 grad = bilateral_sobel(sob, lumaStdDev);

    const float g_lf_x = ((g_left + g_right) * 0.5f), g_lf_y = ((g_up + g_down) * 0.5f);
    const float g_hf_x = ((2.0f * c_xy - (c_left + c_right)) * 0.25f);
    const float g_hf_y = ((2.0f * c_xy - (c_up + c_down)) * 0.25f);

    const float glen = length2_(grad.x, grad.y);
    const float lgt = smoothstep_(lumaStdDev, 4.0f * lumaStdDev, glen);
    if (lgt == 0.0f && glen <= 3.40282347e38f) {
        // Flat (lgt a zero of either sign) with a finite gradient: hf_gain below is lgt times a
        // value in [+0, 1] (the clamped whiteness halved plus a smoothstep, capped at 1), so a
        // zero of lgt's sign, and the direction is mix(0.5, d, lgt) with a finite d, which is
        // 0.5; the whiteness, the angle and its smoothsteps do not change the result.
        const float hf0 = lgt * 0.0f;
        return mix_(g_lf_y + hf0 * g_hf_y, g_lf_x + hf0 * g_hf_x, 0.5f);
    }
    const float whiteness =
        clamp_(div_(mmin(c_xy, mmin(g_ave, c2_ave)), mmax(c_xy, mmax(g_ave, c2_ave))), 0.0f, 1.0f);
    const float hf_gain = lgt * mmin(0.5f * whiteness + smoothstep_(0.0f, 0.3f, div_(glen, GLS_SQRT2_F)), 1.0f);
    const float g_est_x = g_lf_x + hf_gain * g_hf_x;
    const float g_est_y = g_lf_y + hf_gain * g_hf_y;

    float direction = 2.0f * glsm::atan2pi_(grad.y, grad.x);
    direction = direction < 0.5f
                    ? mix_(direction, 0.0f, 1.0f - smoothstep_(0.3f * lgt, 0.45f * lgt, direction))
                    : mix_(direction, 1.0f, smoothstep_((1.0f - 0.45f) * lgt, (1.0f - 0.3f) * lgt, direction));
    direction = mix_(0.5f, direction, lgt);
    return mix_(g_est_y, g_est_x, direction);
}

// ---- a8: interpolateRedBlue (demosaic.cl:229-318) -> (red, green, blue) ----
template <class AccR, class AccG>
GLS_DI float3 red_blue_at(const AccR& raw, const AccG& gi, int x, int y, int bayer, float chromaVariance) {
    const int rx = bayer_dx(bayer, raw_red), ry = bayer_dy(bayer, raw_red);
    const int gx = bayer_dx(bayer, raw_green), gy = bayer_dy(bayer, raw_green);
    const int bx = bayer_dx(bayer, raw_blue), by = bayer_dy(bayer, raw_blue);
    const int color = ((rx & 1) == (x & 1) && (ry & 1) == (y & 1))   ? raw_red
                      : ((gx & 1) == (x & 1) && (gy & 1) == (y & 1)) ? raw_green
                      : ((bx & 1) == (x & 1) && (by & 1) == (y & 1)) ? raw_blue
                                                                     : raw_green2;
    const float green = gi.at(x, y);
    float red, blue;
    if (color == raw_red || color == raw_blue) {
        const float c1 = raw.at(x, y);
        const float g_tl = gi.at(x - 1, y - 1), g_tr = gi.at(x + 1, y - 1);
        const float g_bl = gi.at(x - 1, y + 1), g_br = gi.at(x + 1, y + 1);
        const float c2_tl = g_tl - raw.at(x - 1, y - 1), c2_tr = g_tr - raw.at(x + 1, y - 1);
        const float c2_bl = g_bl - raw.at(x - 1, y + 1), c2_br = g_br - raw.at(x + 1, y + 1);
        const float chromaStdDev = sqrt_(chromaVariance * green);
        const float dvx = glsm::fabs_(c2_tl - c2_br), dvy = glsm::fabs_(c2_tr - c2_bl);
        const float flatness = 1.0f - smoothstep_(0.25f * chromaStdDev, chromaStdDev, length2_(dvx, dvy));
        const float alpha = mix_(2.0f * glsm::atan2pi_(dvy, dvx), 0.5f, flatness);
        const float c2 = green - mix_(((c2_tr + c2_bl) * 0.5f), ((c2_tl + c2_br) * 0.5f), alpha);
        if (color == raw_red) {
            red = c1;
            blue = c2;
        } else {
            blue = c1;
            red = c2;
        }
    } else {
        const float g_left = gi.at(x - 1, y), g_right = gi.at(x + 1, y);
        const float g_up = gi.at(x, y - 1), g_down = gi.at(x, y + 1);
        const float c1_left = g_left - raw.at(x - 1, y), c1_right = g_right - raw.at(x + 1, y);
        const float c2_up = g_up - raw.at(x, y - 1), c2_down = g_down - raw.at(x, y + 1);
        const float c1 = green - ((c1_left + c1_right) * 0.5f);
        const float c2 = green - ((c2_up + c2_down) * 0.5f);
        const int red_row_green = (bayer == bggr || bayer == grbg) ? raw_green : raw_green2;
        if (color == red_row_green) {
            red = c1;
            blue = c2;
        } else {
            blue = c1;
            red = c2;
        }
    }
    return make_float3(red, green, blue);
}

// ---- a9: blendHighlightsImage (demosaic.cl:338-380) ----
GLS_DI float3 blend_highlights_px(float3 p, float clip) {
    if (p.x > clip || p.y > clip || p.z > clip) {
        const float S3 = GLS_SQRT3_F;
        const float h3 = S3 / 2.0f;
        float c0[3] = {p.x, p.y, p.z};
        float c1[3] = {mmin(p.x, clip), mmin(p.y, clip), mmin(p.z, clip)};
        // lab = trans * cam, trans = {{1,1,1},{S3,-S3,0},{-1,-1,2}}
        float l0[3], l1[3];
        l0[0] = 1.0f * c0[0] + 1.0f * c0[1] + 1.0f * c0[2];
        l0[1] = S3 * c0[0] + -S3 * c0[1] + 0.0f * c0[2];
        l0[2] = -1.0f * c0[0] + -1.0f * c0[1] + 2.0f * c0[2];
        l1[0] = 1.0f * c1[0] + 1.0f * c1[1] + 1.0f * c1[2];
        l1[1] = S3 * c1[0] + -S3 * c1[1] + 0.0f * c1[2];
        l1[2] = -1.0f * c1[0] + -1.0f * c1[1] + 2.0f * c1[2];
        const float sum0 = l0[1] * l0[1] + l0[2] * l0[2];
        const float sum1 = l1[1] * l1[1] + l1[2] * l1[2];
        const float chratio = sum0 > 0.0f ? sqrt_(div_(sum1, sum0)) : 1.0f;
        l0[1] = l0[1] * chratio;
        l0[2] = l0[2] * chratio;
        // itrans = {{1, S3/2, -0.5}, {1, -S3/2, -0.5}, {1, 0, 1}}
        p.x = div_(1.0f * l0[0] + h3 * l0[1] + -0.5f * l0[2], 3.0f);
        p.y = div_(1.0f * l0[0] + -h3 * l0[1] + -0.5f * l0[2], 3.0f);
        p.z = div_(1.0f * l0[0] + 0.0f * l0[1] + 1.0f * l0[2], 3.0f);
    }
    return p;
}

// ---- a10: transformImage (demosaic.cl:728-733) ----
struct Mat3 {
    float m[9];
};

GLS_DI float3 transform_px(const Mat3& t, float3 v) {
    return make_float3(t.m[0] * v.x + t.m[1] * v.y + t.m[2] * v.z, t.m[3] * v.x + t.m[4] * v.y + t.m[5] * v.z,
                       t.m[6] * v.x + t.m[7] * v.y + t.m[8] * v.z);
}

// ---- a11: despeckleLumaMedianChromaImage (demosaic.cl:444-489), bound by the host
// function despeckleImage (demosaic_cl.cpp:270-291).  Reads through read_imageh (values
// rounded to binary16); every half-precision operation rounds to binary16. ----
GLS_DI void cswap(float& a, float& b) {
    const float t = a;
    a = mmin(a, b);
    b = mmax(t, b);
}

// the compare-exchange of the median network on (Cb, Cr) pairs: the hardware's half2
// minimum and maximum.  For finite values it agrees with cswap's selects as values; on a
// (-0, +0) tie it may keep the other zero, which no later value depends on (the chroma feeds
// differences, squares, sums and products; the parity tests compare values).
GLS_DI void cswap2(__half2& a, __half2& b) {
    const __half2 lo = __hmin2(a, b), hi = __hmax2(a, b);
    a = lo;
    b = hi;
}

// HALF_EXACT: the accessor returns binary16 values already (a half4 tile of the fused
// pipeline, finite by construction), so the rounding of every read to binary16 is the
// identity and is skipped, and the chroma median runs on half2 pairs (cswap2).  Otherwise
// (the single-stage entry point, any input) the reference's selects are evaluated as written.
template <bool HALF_EXACT = false, class Acc4>
GLS_DI float4 despeckle_px(const Acc4& im, int px, int py, float va0, float vb0) {
    using glsm::round_half;
    float sample = 0.0f, firstMax = 0.0f, secMax = 0.0f;
    const float hinf = glsm::inf_();  // (half)(float)0xffff overflows to +inf
    float firstMin = hinf, secMin = hinf;
    float acb[6], acr[6];
    __half2 ac[6];  // HALF_EXACT: (acb, acr) pairs
    auto rd = [&](int dx, int dy, int k) {
        const float4 p = im.at(px + dx, py + dy);
        const float v = HALF_EXACT ? p.x : round_half(p.x);
        if (HALF_EXACT) {
            ac[k] = __floats2half2_rn(p.y, p.z);
        } else {
            acb[k] = round_half(p.y);
            acr[k] = round_half(p.z);
        }
        secMax = (v <= firstMax && v > secMax) ? v : secMax;
        secMax = v > firstMax ? firstMax : secMax;
        firstMax = v > firstMax ? v : firstMax;
        secMin = (v >= firstMin && v < secMin) ? v : secMin;
        secMin = v < firstMin ? firstMin : secMin;
        firstMin = v < firstMin ? v : firstMin;
        if (dx == 0 && dy == 0) sample = v;
    };
    auto cs = [&](int a, int b) {
        if (HALF_EXACT) {
            cswap2(ac[a], ac[b]);
        } else {
            cswap(acb[a], acb[b]);
            cswap(acr[a], acr[b]);
        }
    };
    rd(0, -1, 0);
    rd(1, -1, 1);
    rd(0, 0, 2);
    rd(1, 0, 3);
    rd(0, 1, 4);
    rd(1, 1, 5);
    // minMax6
    cs(0, 1); cs(2, 3); cs(4, 5);
    cs(0, 2); cs(1, 3); cs(0, 4); cs(3, 5);
    rd(-1, 1, 0);
    // minMax5
    cs(0, 1); cs(2, 3); cs(0, 2);
    cs(1, 3); cs(0, 4); cs(3, 4);
    rd(-1, 0, 0);
    // minMax4
    cs(0, 1); cs(2, 3); cs(0, 2); cs(1, 3);
    rd(-1, -1, 0);
    // minMax3
    cs(0, 1); cs(0, 2); cs(1, 2);

    const float sigma = round_half(sqrt_(va0 + vb0 * sample));
    const float four_sigma = round_half(4.0f * sigma);
    auto hsmooth = [&](float e0, float e1, float x) {
        const float t = clamp_(round_half(div_(round_half(x - e0), round_half(e1 - e0))), 0.0f, 1.0f);
        return round_half(round_half(t * t) * round_half(3.0f - round_half(2.0f * t)));
    };
    auto hmix = [&](float x, float y, float t) { return round_half(x + round_half(round_half(y - x) * t)); };
    const float minVal = hmix(secMin, firstMin, hsmooth(sigma, four_sigma, round_half(secMin - firstMin)));
    const float maxVal = hmix(secMax, firstMax, hsmooth(sigma, four_sigma, round_half(firstMax - secMax)));
    sample = clamp_(sample, minVal, maxVal);
    if (HALF_EXACT) return make_float4(sample, __low2float(ac[1]), __high2float(ac[1]), 0.0f);
    return make_float4(sample, acb[1], acr[1], 0.0f);
}

// ---- a12: downsampleImage (demosaic.cl:853-865) ----
template <class Acc4>
GLS_DI float4 downsample_px(const Acc4& in, int x, int y, int ow, int oh, int iw, int ih) {
    const float nx = div_(1.0f, (float)ow), ny = div_(1.0f, (float)oh);
    const float px = ((float)x + 0.5f) * nx, py = ((float)y + 0.5f) * ny;
    const float sx = 0.5f * nx, sy = 0.5f * ny;
    const float4 t0 = sample4(in, px + -sx, py + -sy, iw, ih);
    const float4 t1 = sample4(in, px + sx, py + -sy, iw, ih);
    const float4 t2 = sample4(in, px + -sx, py + sy, iw, ih);
    const float4 t3 = sample4(in, px + sx, py + sy, iw, ih);
    float4 r;
    r.x = 0.25f * (t0.x + t1.x + t2.x + t3.x);
    r.y = 0.25f * (t0.y + t1.y + t2.y + t3.y);
    r.z = 0.25f * (t0.z + t1.z + t2.z + t3.z);
    r.w = 0.25f * (t0.w + t1.w + t2.w + t3.w);
    return r;
}

// ---- a14: denoiseImage, bilateral (demosaic.cl:735-765) ----
struct Nlf6 {
    float a[3], b[3];
};

// Luma channel of an RGBA accessor, for the sobel of the gradient boost.
template <class Acc4>
struct LumaOf {
    const Acc4& im;
    GLS_DI float at(int x, int y) const { return im.at(x, y).x; }
};

// The bilateral sum with the literal divisions and square roots (rare path).
template <class Acc4>
__device__ __noinline__ float4 bilateral_literal(const Acc4& im, int px, int py, float sig0, float sig1, float sig2,
                                                 float e0, float e1) {
    const float4 c = im.at(px, py);
    // the two chroma channels share their weights, so their normalisers are one sum
    float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, n0 = 0.0f, n1 = 0.0f;
    for (int y = -2; y <= 2; y++) {
        for (int x = -2; x <= 2; x++) {
            const float4 s = im.at(px + x, py + y);
            const float d0 = div_(s.x - c.x, sig0), d1 = div_(s.y - c.y, sig1), d2 = div_(s.z - c.z, sig2);
            const float l = length3_(d0, d1, d2);
            const float w0 = 1.0f - step_(e0, l), w1 = 1.0f - step_(e1, l);
            f0 = f0 + w0 * s.x;
            n0 = n0 + w0;
            f1 = f1 + w1 * s.y;
            n1 = n1 + w1;
            f2 = f2 + w1 * s.z;
        }
    }
    return make_float4(div_(f0, n0), div_(f1, n1), div_(f2, n1), 0.0f);
}

// Accessors whose samples all have .w == 1 (a staged tile whose alpha the kernel set) declare
// `static constexpr bool kUnitW = true`; the bilateral then counts its normaliser in the
// packed (z, w) accumulation instead of a separate add.
template <class A, class = void>
struct unit_w {
    static constexpr bool value = false;
};
template <class A>
struct unit_w<A, decltype((void)A::kUnitW)> {
    static constexpr bool value = A::kUnitW;
};

// 1 / v to within one unit in the last place (the hardware reciprocal approximation): the
// bilateral's decision proxy needs 1 / sigma^2 to a few 2^-23 only.
GLS_DI float rcp_approx(float v) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}

template <class Acc4>
__device__ __noinline__ float4 bilateral_literal_v(const Acc4& im, int px, int py, float v0, float v1, float v2,
                                                   float e0, float e1) {
    return bilateral_literal(im, px, py, sqrt_(v0), sqrt_(v1), sqrt_(v2), e0, e1);
}

template <class Acc4>
GLS_DI float4 bilateral_px(const Acc4& im, int px, int py, const Nlf6& n, float chromaBoost, float gradientBoost) {
    constexpr bool UW = unit_w<Acc4>::value;
    const float4 c = im.at(px, py);
    // sigma_k = sqrt(v_k) (demosaic.cl:741-743); the fast path below needs only 1 / v_k
    const float v0 = n.a[0] + n.b[0] * c.x;
    const float v1 = n.a[1] + n.b[1] * c.x;
    const float v2 = n.a[2] + n.b[2] * c.x;
    float lumaBoost = 1.0f;
    if (gradientBoost > 1.0f) {
        const float sig0 = sqrt_(v0);
        LumaOf<Acc4> l{im};
        const float2 g = sobel_signed(l, px, py);
        lumaBoost = gradientBoost -
                    (gradientBoost - 1.0f) * smoothstep_(0.5f, 2.0f, length2_(div_(g.x, sig0), div_(g.y, sig0)));
    }
    // weight = 1 - step(edge, length(diff / sigma)) = !(sqrt_rn(q) >= edge), where
    // q = RN(RN(d0^2) + RN(d1^2)) + RN(d2^2) with d_k = RN(diff_k / sigma_k).  Each tap is
    // decided on qa = sum diff_k^2 * r_k instead, r_k = 1 / v_k to one ulp (1 / sigma_k^2 to
    // about 2^-21.4, sigma_k being the rounded square root): all terms are non-negative, so
    // qa and q both lie within about 2^-20 of the exact sum of (diff_k / sigma_k)^2, and a tap
    // whose qa clears the square-root band of the edge (2^-20) widened by 2^-16 has the same
    // weight either way.  The fast path keeps edges below 2^20 and 2^-120 <= v_k <= 2^60 (the
    // sigmas in [2^-60, 2^30]), so an overflowing diff^2 (or product) means d^2 > 2^68 and
    // weight 0 on both sides, and qa is never NaN for finite samples.  A tap inside the band,
    // or a NaN qa (the literal weight of a NaN sample is 1), is counted by !(qa > hi) but not
    // by qa < lo: when the two counts differ the pixel takes the literal evaluation.  The
    // weights are 0 or 1, so w * s is exact and the multiply-adds can be fused without
    // changing a bit; channel pairs go through the packed fp32x2 operations, each lane
    // rounded exactly as the scalar one.
    SqrtGe ge0, ge1;
    ge0.init(lumaBoost * GLS_SQRT2_F);
    ge1.init(chromaBoost * GLS_SQRT2_F);
    auto v_ok = [](float v) { return v >= 7.52316384526264e-37f && v <= 1.152921504606847e18f; };  // 2^-120, 2^60
    if (!(v_ok(v0) && v_ok(v1) && v_ok(v2) && ge0.ok && ge1.ok && ge0.e < 1048576.0f && ge1.e < 1048576.0f))
        return bilateral_literal_v(im, px, py, v0, v1, v2, ge0.e, ge1.e);
    constexpr float kWiden = 1.52587890625e-05f;  // 2^-16
    const float r0 = rcp_approx(v0), r1 = rcp_approx(v1), r2 = rcp_approx(v2);
    const float lo0 = ge0.lo * (1.0f - kWiden), hi0 = ge0.hi * (1.0f + kWiden);
    const float lo1 = ge1.lo * (1.0f - kWiden), hi1 = ge1.hi * (1.0f + kWiden);
    const float2 nc = make_float2(-c.x, -c.y);  // s - c == s + (-c), bit for bit
    float2 fxy = make_float2(0.0f, 0.0f);       // (f0, f1)
    float2 fzn = make_float2(0.0f, 0.0f);       // (f2, n1): the two chroma channels share their normaliser
    if (ge0.e == ge1.e) {
        // one edge for luma and chroma: one weight per tap, n0 == n1
        float nhi = 0.0f;
#pragma unroll 1
        for (int y = -2; y <= 2; y++) {
#pragma unroll
            for (int x = -2; x <= 2; x++) {
                const float4 s = im.at(px + x, py + y);
                const float2 dxy = add2(make_float2(s.x, s.y), nc);
                const float2 qxy = mul2(dxy, dxy);  // feeds multiplicands only
                const float d2 = s.z - c.z;
                const float qa = glsm::fma_(qxy.x, r0, glsm::fma_(qxy.y, r1, (d2 * d2) * r2));
                const float w = qa < lo0 ? 1.0f : 0.0f;
                nhi = nhi + (qa > hi0 ? 0.0f : 1.0f);
                const float2 ww = make_float2(w, w);
                fxy = fma2(ww, make_float2(s.x, s.y), fxy);
                fzn = fma2(ww, make_float2(s.z, UW ? s.w : 1.0f), fzn);
            }
        }
        if (nhi != fzn.y) return bilateral_literal_v(im, px, py, v0, v1, v2, ge0.e, ge1.e);
        return make_float4(div_(fxy.x, fzn.y), div_(fxy.y, fzn.y), div_(fzn.x, fzn.y), 0.0f);
    }
    float n0 = 0.0f, nhi0 = 0.0f, nhi1 = 0.0f;
#pragma unroll 1
    for (int y = -2; y <= 2; y++) {
#pragma unroll
        for (int x = -2; x <= 2; x++) {
            const float4 s = im.at(px + x, py + y);
            const float2 dxy = add2(make_float2(s.x, s.y), nc);
            const float2 qxy = mul2(dxy, dxy);
            const float d2 = s.z - c.z;
            const float qa = glsm::fma_(qxy.x, r0, glsm::fma_(qxy.y, r1, (d2 * d2) * r2));
            const float w0 = qa < lo0 ? 1.0f : 0.0f, w1 = qa < lo1 ? 1.0f : 0.0f;
            nhi0 = nhi0 + (qa > hi0 ? 0.0f : 1.0f);
            nhi1 = nhi1 + (qa > hi1 ? 0.0f : 1.0f);
            n0 = n0 + w0;
            fxy = fma2(make_float2(w0, w1), make_float2(s.x, s.y), fxy);
            fzn = fma2(make_float2(w1, w1), make_float2(s.z, UW ? s.w : 1.0f), fzn);
        }
    }
    if (nhi0 != n0 || nhi1 != fzn.y) return bilateral_literal_v(im, px, py, v0, v1, v2, ge0.e, ge1.e);
    return make_float4(div_(fxy.x, n0), div_(fxy.y, fzn.y), div_(fzn.x, fzn.y), 0.0f);
}

// ---- a15: denoiseImageGuided / denoiseLumaChromaGuided (demosaic.cl:767-851) ----
template <class Acc4>
GLS_DI float4 guided_fast_px(const Acc4& im, int px, int py, const Nlf6& n) {
    const float4 I = im.at(px, py);
    const float eps0 = n.a[0] + n.b[0] * I.x, eps1 = n.a[1] + n.b[1] * I.x, eps2 = n.a[2] + n.b[2] * I.x;
    const float norm = div_(1.0f, 25.0f);
    float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f, rr = 0.0f, rg = 0.0f, rb = 0.0f, gg = 0.0f, gb = 0.0f, bb = 0.0f;
#pragma unroll
    for (int y = -2; y <= 2; y++) {
#pragma unroll
        for (int x = -2; x <= 2; x++) {
            const float4 s = im.at(px + x, py + y);
            m0 = m0 + s.x;
            m1 = m1 + s.y;
            m2 = m2 + s.z;
            rr = rr + s.x * s.x;
            rg = rg + s.x * s.y;
            rb = rb + s.x * s.z;
            gg = gg + s.y * s.y;
            gb = gb + s.y * s.z;
            bb = bb + s.z * s.z;
        }
    }
    m0 = m0 * norm; m1 = m1 * norm; m2 = m2 * norm;
    rr = rr * norm; rg = rg * norm; rb = rb * norm; gg = gg * norm; gb = gb * norm; bb = bb * norm;
    const float vrr = rr - m0 * m0, vrg = rg - m0 * m1, vrb = rb - m0 * m2;
    const float vgg = gg - m1 * m1, vgb = gb - m1 * m2, vbb = bb - m2 * m2;
    const float vrre = vrr + eps0, vgge = vgg + eps1, vbbe = vbb + eps2;
    float invrr = vgge * vbbe - vgb * vgb;
    float invrg = vgb * vrb - vrg * vbbe;
    float invrb = vrg * vgb - vgge * vrb;
    float invgg = vrre * vbbe - vrb * vrb;
    float invgb = vrb * vrg - vrre * vgb;
    float invbb = vrre * vgge - vrg * vrg;
    const float det = div_(1.0f, invrr * vrre + invrg * vrg + invrb * vrb);
    invrr = invrr * det; invrg = invrg * det; invrb = invrb * det;
    invgg = invgg * det; invgb = invgb * det; invbb = invbb * det;
    const float cr[3] = {vrr, vrg, vrb}, cg[3] = {vrg, vgg, vgb}, cb[3] = {vrb, vgb, vbb};
    const float mI[3] = {m0, m1, m2};
    const float In[3] = {I.x, I.y, I.z};
    float out[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float ar = invrr * cr[k] + invrg * cg[k] + invrb * cb[k];
        const float ag = invrg * cr[k] + invgg * cg[k] + invgb * cb[k];
        const float ab = invrb * cr[k] + invgb * cg[k] + invbb * cb[k];
        const float b = mI[k] - ar * mI[0] - ag * mI[1] - ab * mI[2];
        out[k] = ar * In[0] + ag * In[1] + ab * In[2] + b;
    }
    return make_float4(out[0], out[1], out[2], 0.0f);
}

// ---- a17: reassembleImage (demosaic.cl:867-896) ----
// d0: the denoised fine pixel; i1/d1: the coarse level before/after denoise; (w, h) the
// fine level's size, (w1, h1) the coarse level's.
// The arithmetic of reassembleImage once its samples are known: p1, pd1 are the coarse
// image and its denoised version at the pixel; sharp() returns the .x of the denoised coarse
// level one fine pixel to the right, left, below and above (asked for only when sharpening).
template <class SharpF>
GLS_DI float4 reassemble_from(float4 d0, float4 p1, float4 pd1, const SharpF& sharp, float sharpening, float nlf0,
                              float nlf1) {
    // dp = d0 - (p1 - pd1) per channel, the channel pairs packed
    const float2 dxy = sub2(f2(d0.x, d0.y), sub2(f2(p1.x, p1.y), f2(pd1.x, pd1.y)));
    const float2 dzw = sub2(f2(d0.z, d0.w), sub2(f2(p1.z, p1.w), f2(pd1.z, pd1.w)));
    float4 dp = make_float4(dxy.x, dxy.y, dzw.x, dzw.y);
    if (sharpening > 1.0f) {
        const float4 g = sharp();
        const float dx = ((g.x - g.y) * 0.5f);
        const float dy = ((g.z - g.w) * 0.5f);
        const float threshold = 0.25f * sqrt_(nlf0 + nlf1 * pd1.x);
        const float detail = smoothstep_(0.25f * threshold, threshold, length2_(dx, dy)) *
                             (1.0f - smoothstep_(0.95f, 1.0f, dp.x)) * (0.6f + 0.4f * smoothstep_(0.0f, 0.1f, dp.x));
        sharpening = 1.0f + (sharpening - 1.0f) * detail;
    }
    dp.x = mix_(pd1.x, dp.x, sharpening);
    return dp;
}

template <class AccI, class AccD>
GLS_DI float4 reassemble_px(float4 d0, const AccI& i1, const AccD& d1, int x, int y, int w, int h, int w1, int h1,
                            float sharpening, float nlf0, float nlf1) {
    const float nx = div_(1.0f, (float)w), ny = div_(1.0f, (float)h);
    const float ipx = ((float)x + 0.5f) * nx, ipy = ((float)y + 0.5f) * ny;
    const float4 p1 = sample4(i1, ipx, ipy, w1, h1);
    const float4 pd1 = sample4(d1, ipx, ipy, w1, h1);
    auto sharp = [&]() {
        return make_float4(sample4(d1, ipx + nx, ipy + 0.0f * ny, w1, h1).x,
                           sample4(d1, ipx - nx, ipy - 0.0f * ny, w1, h1).x,
                           sample4(d1, ipx + 0.0f * nx, ipy + ny, w1, h1).x,
                           sample4(d1, ipx - 0.0f * nx, ipy - ny, w1, h1).x);
    };
    return reassemble_from(d0, p1, pd1, sharp, sharpening, nlf0, nlf1);
}

// ---- a18: localToneMappingMask (demosaic.cl:1026-1107) ----
struct LtmParams {
    float eps, shadows, highlights, detail;
};

// Guide sample offsets of localToneMappingMask, in fine pixels: sample i sits at
// (kLtmOff[i % 3], kLtmOff[i / 3]) + 0.5 from the pixel, with weight kLtmW[i].
#define GLS_LTM_OFFSETS {-1.5f, 0.5f, 2.0f}

// The arithmetic of localToneMappingMask once its samples are known: gs[i] the guide's .x at
// the nine offsets, inp the denoised image at the pixel.
GLS_DI float ltm_mask_from(const float (&gs)[9], float4 inp, const LtmParams& lp, const Mat3& m) {
    const float bw[9] = {0.16f, 0.16f, 0.08f, 0.16f, 0.16f, 0.08f, 0.08f, 0.08f, 0.04f};
    float2 ss = f2(0.0f, 0.0f);  // (sum, sumSq) as one packed chain of scalar products
#pragma unroll
    for (int i = 0; i < 9; i++) {
        const float s = __fmul_rn(bw[i], gs[i]);
        ss = add2(ss, f2(s, __fmul_rn(s, s)));
    }
    const float sum = ss.x, sumSq = ss.y;
    const float mean = sum, var = sumSq - sum * sum;
    const float luma = inp.x;
    float filtered = 0.0f, knorm = 0.0f;
    const float den = var + lp.eps;
    FastDiv dv;
    dv.init(den);
    // The numerators (gs_i - mean) * (luma - mean): when the samples and the luma are finite
    // with magnitudes summing to at most 2^20, every numerator is below 2^42, inside the
    // shortcut's range; a numerator under its lower bound (2^-83) gives, with den >= 2^-20, a
    // quotient below 2^-62 either way, and 1 + q rounds to 1 for both.  So the shortcut gives
    // every tap its literal weight and the per-tap range test is dropped.
    float mag = glsm::fabs_(luma);
#pragma unroll
    for (int i = 0; i < 9; i++) mag = mag + glsm::fabs_(gs[i]);
    const bool fast = dv.ok && den >= 9.5367431640625e-07f && mag <= 1048576.0f;  // 2^-20, 2^20; NaN fails
    if (fast) {
        // two taps per step: the numerators and the shortcut's quotients as packed lanes
        // (num feeds a multiply and an fma only), the weights and the products that are
        // summed as scalar multiplies, (filtered, knorm) as one packed chain
        const float lm = luma - mean;
        const float2 mv = f2(mean, mean), lmv = f2(lm, lm), yv = f2(dv.y, dv.y), ndv = f2(-dv.d, -dv.d);
        float2 fk = f2(0.0f, 0.0f);
#pragma unroll
        for (int i = 0; i < 9; i += 2) {
            const bool two = i + 1 < 9;
            const float2 g = f2(gs[i], two ? gs[i + 1] : gs[i]);
            const float2 num = mul2(sub2(g, mv), lmv);
            const float2 q0 = mul2(num, yv);
            const float2 opq = add2(f2(1.0f, 1.0f), fma2(fma2(q0, ndv, num), yv, q0));
            const float wa = __fmul_rn(bw[i], opq.x);
            fk = add2(fk, f2(__fmul_rn(wa, g.x), wa));
            if (two) {
                const float wb = __fmul_rn(bw[i + 1], opq.y);
                fk = add2(fk, f2(__fmul_rn(wb, g.y), wb));
            }
        }
        filtered = fk.x;
        knorm = fk.y;
    } else {
#pragma unroll
        for (int i = 0; i < 9; i++) {
            const float num = (gs[i] - mean) * (luma - mean);
            const float wgt = bw[i] * (1.0f + dv(num));
            filtered = filtered + wgt * gs[i];
            knorm = knorm + wgt;
        }
    }
    const float illuminance = div_(filtered, knorm);
    const float reflectance = div_(luma, illuminance);
    const float3 rgb = transform_px(m, make_float3(inp.x, inp.y, inp.z));
    // hc = min(length(sqrt(2r), sqrt(2g), sqrt(2b)), 1), which is 1 without the square roots
    // when a channel is negative or NaN (the length is NaN, and min(NaN, 1) selects 1) or
    // when 2 (r + g + b) >= 1 + 2^-18 (each rounded sqrt(2c)^2 is within 2^-22 of 2c, so the
    // rounded length is at least 1)
    float hc = 1.0f;
    if (rgb.x >= 0.0f && rgb.y >= 0.0f && rgb.z >= 0.0f &&
        2.0f * ((rgb.x + rgb.y) + rgb.z) < 1.000003814697265625f)
        hc = mmin(length3_(sqrt_(2.0f * rgb.x), sqrt_(2.0f * rgb.y), sqrt_(2.0f * rgb.z)), 1.0f);
    const float tc = mix_(lp.shadows, lp.highlights, hc);
    return div_(glsm::pow_(illuminance, div_(1.0f, tc)) * glsm::pow_(reflectance, lp.detail), luma);
}

template <class AccIn, class AccG>
GLS_DI float ltm_mask_px(const AccIn& in, const AccG& guide, int x, int y, int w, int h, int gw, int gh,
                         const LtmParams& lp, const Mat3& m) {
    const float off[3] = GLS_LTM_OFFSETS;
    const float nx = div_(1.0f, (float)w), ny = div_(1.0f, (float)h);
    const float px = (float)x * nx, py = (float)y * ny;
    float gs[9];
#pragma unroll
    for (int i = 0; i < 9; i++)
        gs[i] = sample4(guide, px + (off[i % 3] + 0.5f) * nx, py + (off[i / 3] + 0.5f) * ny, gw, gh).x;
    const float4 inp = sample4(in, px + 0.5f * nx, py + 0.5f * ny, w, h);
    return ltm_mask_from(gs, inp, lp, m);
}

// ---- a19: convertTosRGB + toneCurve & co (demosaic.cl:1380-1474) ----
struct RgbParams {
    float contrast, saturation, toneCurveSlope, exposureBias, blacks;
    int localToneMapping;
    // per-frame constants of convertTosRGB, evaluated once (rgb_params_init): the exposure
    // factor powr(2, exposureBias) and the tone curve's sigmoid(0, s), sigmoid(1, s) - sigmoid(0, s)
    // with its reciprocal RN(1 / that) and whether the shared-divisor shortcut applies to it
    float eb, sig0, sig_den, sig_rcp;
    int sig_ok;
};

__host__ __device__ inline float sigmoid_(float x, float s) { return 0.5f * (glsm::tanh_(s * x - 0.3f * s) + 1.0f); }

__host__ __device__ inline RgbParams rgb_params_init(float contrast, float saturation, float toneCurveSlope,
                                                     float exposureBias, float blacks, int localToneMapping) {
    RgbParams r;
    r.contrast = contrast;
    r.saturation = saturation;
    r.toneCurveSlope = toneCurveSlope;
    r.exposureBias = exposureBias;
    r.blacks = blacks;
    r.localToneMapping = localToneMapping;
    r.eb = exposureBias != 0.0f ? glsm::powr_(2.0f, exposureBias) : 1.0f;
    r.sig0 = sigmoid_(0.0f, toneCurveSlope);
    r.sig_den = sigmoid_(1.0f, toneCurveSlope) - r.sig0;
    FastDiv f;
    f.init(r.sig_den);
    r.sig_rcp = f.y;
    r.sig_ok = f.ok ? 1 : 0;
    return r;
}

GLS_DI float tone_curve_(float x, float s, float sig0, const FastDiv& den) {
    return den(sigmoid_(sqrt_(0.95f * x), s) - sig0);
}

GLS_DI float3 srgb_px(float3 in, float ltm, const Mat3& m, const RgbParams& rp) {
    float p[3] = {in.x, in.y, in.z};
    const float eb = rp.eb;
#pragma unroll
    for (int k = 0; k < 3; k++) p[k] = p[k] * eb;
    if (rp.saturation != 1.0f) {
        const float luma = 0.2126f * p[0] + 0.7152f * p[1] + 0.0722f * p[2];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float clip = smoothstep_(0.75f, 2.0f, p[k]);
            p[k] = mix_(luma, p[k], mix_(rp.saturation, 1.0f, clip));
        }
    }
    if (rp.contrast != 1.0f) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float clip = smoothstep_(0.9f, 2.0f, p[k]);
            p[k] = mix_(0.2f, p[k], mix_(rp.contrast, 1.0f, clip));
        }
    }
    const float3 t = transform_px(m, make_float3(p[0], p[1], p[2]));
    float rgb[3] = {t.x, t.y, t.z};
    const FastDiv tden = FastDiv::of(rp.sig_den, rp.sig_rcp, rp.sig_ok != 0);
#pragma unroll
    for (int k = 0; k < 3; k++) rgb[k] = clamp_(tone_curve_(rgb[k], rp.toneCurveSlope, rp.sig0, tden), 0.0f, 1.0f);
    if (rp.localToneMapping) {
        const float boost = ltm;
        if (boost > 1.0f) {
            const float luma = 0.2126f * rgb[0] + 0.7152f * rgb[1] + 0.0722f * rgb[2];
            const float tt = glsm::pow_(luma, 0.5f);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float a = rgb[k] * boost;
                const float b = luma < 1.0f ? 1.0f - div_((1.0f - rgb[k]) * (1.0f - boost * luma), 1.0f - luma) : rgb[k];
                rgb[k] = mix_(a, b, tt);
            }
        } else if (boost < 1.0f) {
#pragma unroll
            for (int k = 0; k < 3; k++) rgb[k] = rgb[k] * boost;
        }
    }
    if (rp.blacks > 0.0f) {
#pragma unroll
        for (int k = 0; k < 3; k++) rgb[k] = div_(rgb[k] - rp.blacks, 1.0f - rp.blacks);
    }
    return make_float3(rgb[0], rgb[1], rgb[2]);
}

// ---- a6: high-noise raw branch (demosaic.cl:530-553, 930-949, 1187-1201) ----
template <class Acc4>
GLS_DI float4 despeckle_rgba_px(const Acc4& im, int px, int py) {
    float s[4] = {0, 0, 0, 0}, fmx[4] = {0, 0, 0, 0}, smx[4] = {0, 0, 0, 0};
    float fmn[4] = {65535.0f, 65535.0f, 65535.0f, 65535.0f}, smn[4] = {65535.0f, 65535.0f, 65535.0f, 65535.0f};
#pragma unroll
    for (int x = -1; x <= 1; x++) {
#pragma unroll
        for (int y = -1; y <= 1; y++) {
            const float4 v4 = im.at(px + x, py + y);
            const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float v = vv[k];
                smx[k] = (v <= fmx[k] && v > smx[k]) ? v : smx[k];
                smx[k] = v > fmx[k] ? fmx[k] : smx[k];
                fmx[k] = v > fmx[k] ? v : fmx[k];
                smn[k] = (v >= fmn[k] && v < smn[k]) ? v : smn[k];
                smn[k] = v < fmn[k] ? fmn[k] : smn[k];
                fmn[k] = v < fmn[k] ? v : fmn[k];
                if (x == 0 && y == 0) s[k] = v;
            }
        }
    }
    return make_float4(clamp_(s[0], smn[0], smx[0]), clamp_(s[1], smn[1], smx[1]), clamp_(s[2], smn[2], smx[2]),
                       clamp_(s[3], smn[3], smx[3]));
}

// The literal evaluation of denoiseRawRGBA (divisions and the square root per tap).
template <class Acc4>
__device__ __noinline__ float4 denoise_rgba_literal(const Acc4& im, int px, int py, const float sg[4]) {
    const float4 c = im.at(px, py);
    const float in[4] = {c.x, c.y, c.z, c.w};
    float f[4] = {0, 0, 0, 0}, nrm[4] = {0, 0, 0, 0};
    for (int y = -2; y <= 2; y++) {
        for (int x = -2; x <= 2; x++) {
            const float4 s4 = im.at(px + x, py + y);
            const float s[4] = {s4.x, s4.y, s4.z, s4.w};
            float d[4];
            for (int k = 0; k < 4; k++) d[k] = div_(s[k] - in[k], sg[k]);
            const float w = 1.0f - step_(1.0f, length4_(d[0], d[1], d[2], d[3]));
            for (int k = 0; k < 4; k++) {
                f[k] = f[k] + w * s[k];
                nrm[k] = nrm[k] + w;
            }
        }
    }
    return make_float4(div_(f[0], nrm[0]), div_(f[1], nrm[1]), div_(f[2], nrm[2]), div_(f[3], nrm[3]));
}

// denoiseRawRGBA: weight = 1 - step(1, length(diff / sigma)).  Channels with sigma > 0 enter
// qa = sum diff_k^2 * RN(1/sigma_k)^2, decided against 1 +- 2^-20 widened by 2^-18 as in
// bilateral_px.  A channel with sigma = 0 (a zero plane value) has diff / 0 = NaN for
// diff == 0 and +-inf otherwise, and NaN outranks inf in the sum: when such channels exist
// the weight is 1 exactly if one of them has diff == 0.  Non-finite samples, sigma outside
// the shortcut's range and taps inside the band take the literal evaluation.
template <class Acc4>
GLS_DI float4 denoise_rgba_px(const Acc4& im, int px, int py, const float rv[4]) {
    const float4 c = im.at(px, py);
    const float in[4] = {c.x, c.y, c.z, c.w};
    float sg[4], r[4];
    unsigned zmask = 0;
    bool lit = false;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        sg[k] = sqrt_(rv[k] * in[k]);
        FastDiv d;
        d.init(sg[k]);
        if (sg[k] == 0.0f) zmask |= 1u << k;
        else if (!d.ok) lit = true;
        r[k] = sg[k] == 0.0f ? 0.0f : d.y * d.y;
    }
    if (lit) return denoise_rgba_literal(im, px, py, sg);
    SqrtGe ge;
    ge.init(1.0f);
    constexpr float kWiden = 3.814697265625e-06f;  // 2^-18
    const float lo = ge.lo * (1.0f - kWiden), hi = ge.hi * (1.0f + kWiden);
    float f[4] = {0, 0, 0, 0}, n = 0.0f;
    bool redo = false;
#pragma unroll 1
    for (int y = -2; y <= 2; y++) {
#pragma unroll
        for (int x = -2; x <= 2; x++) {
            const float4 s4 = im.at(px + x, py + y);
            const float s[4] = {s4.x, s4.y, s4.z, s4.w};
            float xs[4];
#pragma unroll
            for (int k = 0; k < 4; k++) xs[k] = s[k] - in[k];
            float w;
            if (zmask) {
                bool nan = false;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (zmask & (1u << k)) nan |= xs[k] == 0.0f;
                redo |= !(fabsf(xs[0]) + fabsf(xs[1]) + fabsf(xs[2]) + fabsf(xs[3]) <= 3.402823466e38f);
                w = nan ? 1.0f : 0.0f;
            } else {
                const float qa = glsm::fma_(xs[0] * xs[0], r[0],
                                            glsm::fma_(xs[1] * xs[1], r[1],
                                                       glsm::fma_(xs[2] * xs[2], r[2], (xs[3] * xs[3]) * r[3])));
                const bool in1 = qa < lo;
                redo |= !(in1 || qa > hi);
                w = in1 ? 1.0f : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) f[k] = glsm::fma_(w, s[k], f[k]);
            n = n + w;
        }
    }
    if (redo) return denoise_rgba_literal(im, px, py, sg);
    return make_float4(div_(f[0], n), div_(f[1], n), div_(f[2], n), div_(f[3], n));
}

}  // namespace gls

#endif  // GLS_PIXEL_OPS_CUH
