// gls_device.cuh -- device-side building blocks shared by every kernel of the RAW pipeline:
// storage types (fp32 / fp16 images), clamp-to-edge accessors over global or shared
// memory, the linear sampler, and compensated (float-float) accumulators for the
// noise-model regressions.
#ifndef GLS_DEVICE_CUH
#define GLS_DEVICE_CUH

#include <cuda_fp16.h>
#include <stdint.h>

#include "gls_clmath.h"
#include "gls_f32x2.cuh"

namespace gls {

#define GLS_DI __device__ __forceinline__

// Kernel CFA offsets (x, y) per {red, green, blue, green2}, demosaic.cl:29-34.
__host__ __device__ constexpr int bayer_dx(int pattern, int c) {
    return (pattern == 0) ? (c == 0 ? 1 : c == 3 ? 1 : 0)
         : (pattern == 1) ? (c == 2 ? 1 : c == 3 ? 1 : 0)
         : (pattern == 2) ? (c == 2 ? 1 : c == 3 ? 1 : 0)
                          : (c == 0 ? 1 : c == 3 ? 1 : 0);
}
__host__ __device__ constexpr int bayer_dy(int pattern, int c) {
    return (pattern == 0) ? (c == 2 ? 1 : c == 3 ? 1 : 0)
         : (pattern == 1) ? (c == 0 ? 1 : c == 3 ? 1 : 0)
         : (pattern == 2) ? (c == 1 ? 1 : c == 2 ? 1 : 0)
                          : (c == 0 ? 1 : c == 1 ? 1 : 0);
}

enum { raw_red = 0, raw_green = 1, raw_blue = 2, raw_green2 = 3 };
enum { grbg = 0, gbrg = 1, rggb = 2, bggr = 3 };

// ---------------------------------------------------------------------------------------
// Storage: fp32 or fp16 images.  Values are always computed in fp32; a store to an fp16
// image rounds to nearest even, exactly like a half-float OpenCL image write.
// ---------------------------------------------------------------------------------------
struct __align__(8) half4 {
    __half2 xy, zw;
};

template <class S>
struct Storage;

template <>
struct Storage<float> {
    typedef float T1;
    typedef float4 T4;
    static GLS_DI float ld(const float* p) { return *p; }
    static GLS_DI float ldg(const float* p) { return __ldg(p); }
    static GLS_DI float4 ld4(const float4* p) { return *p; }
    static GLS_DI float4 ldg4(const float4* p) { return __ldg(p); }
    static GLS_DI void st(float* p, float v) { *p = v; }
    static GLS_DI void st4(float4* p, float4 v) { *p = v; }
    static GLS_DI float round(float v) { return v; }
};

template <>
struct Storage<__half> {
    typedef __half T1;
    typedef half4 T4;
    static GLS_DI float ld(const __half* p) { return __half2float(*p); }
    static GLS_DI float ldg(const __half* p) { return __half2float(__ldg(p)); }
    static GLS_DI float4 cvt(half4 h) {
        const float2 a = __half22float2(h.xy), b = __half22float2(h.zw);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    static GLS_DI float4 ld4(const half4* p) { return cvt(*p); }
    static GLS_DI float4 ldg4(const half4* p) {
        const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
        half4 h;
        *reinterpret_cast<uint2*>(&h) = u;
        return cvt(h);
    }
    static GLS_DI void st(__half* p, float v) { *p = __float2half_rn(v); }
    static GLS_DI void st4(half4* p, float4 v) {
        half4 h;
        h.xy = __halves2half2(__float2half_rn(v.x), __float2half_rn(v.y));
        h.zw = __halves2half2(__float2half_rn(v.z), __float2half_rn(v.w));
        *p = h;
    }
    static GLS_DI float round(float v) { return __half2float(__float2half_rn(v)); }
};

GLS_DI int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Single-channel image in global memory, clamp-to-edge reads.
template <class S>
struct GImg1 {
    const S* p;
    int w, h, pitch;  // pitch in elements
    GLS_DI float at(int x, int y) const {
        x = clampi(x, 0, w - 1);
        y = clampi(y, 0, h - 1);
        return Storage<S>::ldg(p + (size_t)y * pitch + x);
    }
};

// RGBA image in global memory (4 elements per pixel), clamp-to-edge reads.
template <class S>
struct GImg4 {
    const typename Storage<S>::T4* p;
    int w, h, pitch;  // pitch in pixels
    GLS_DI float4 at(int x, int y) const {
        x = clampi(x, 0, w - 1);
        y = clampi(y, 0, h - 1);
        return Storage<S>::ldg4(p + (size_t)y * pitch + x);
    }
};

// Raw uint16 image read through the UNORM16 convention.
struct GRaw16 {
    const uint16_t* p;
    int w, h, pitch;
    GLS_DI uint16_t at(int x, int y) const {
        x = clampi(x, 0, w - 1);
        y = clampi(y, 0, h - 1);
        return __ldg(p + (size_t)y * pitch + x);
    }
};

// ---------------------------------------------------------------------------------------
// Linear sampler (normalised coordinates, CLAMP_TO_EDGE, FILTER_LINEAR): fractions
// computed in float and quantised to 8 fractional bits, texels blended in float in the
// order w00, w10, w01, w11.  Acc must provide float4 at(int, int) with clamping.
// ---------------------------------------------------------------------------------------
struct BilinearTap {
    int i0, j0;
    float w00, w10, w01, w11;
};

// One axis of the sampler: texel index below the (texel-centred) coordinate u * n - 0.5 and
// the fraction above it, quantized to 8 bits as the hardware sampler does.
struct Tap1 {
    int i0;
    float a;
};

GLS_DI Tap1 tap1(float u, int n) {
    const float fu = u * (float)n - 0.5f;
    const float f = floorf(fu);
    float a = fu - f;
    a = floorf(a * 256.0f + 0.5f) * 0.00390625f;
    return Tap1{(int)f, a};
}

GLS_DI BilinearTap bilinear_tap(float u, float v, int w, int h) {
    const Tap1 tx = tap1(u, w), ty = tap1(v, h);
    const float a = tx.a, b = ty.a;
    BilinearTap t;
    t.i0 = tx.i0;
    t.j0 = ty.i0;
    t.w00 = (1.0f - a) * (1.0f - b);
    t.w10 = a * (1.0f - b);
    t.w01 = (1.0f - a) * b;
    t.w11 = a * b;
    return t;
}

template <class Acc>
GLS_DI float4 sample4(const Acc& im, const BilinearTap& t) {
    const float4 p00 = im.at(t.i0, t.j0), p10 = im.at(t.i0 + 1, t.j0);
    const float4 p01 = im.at(t.i0, t.j0 + 1), p11 = im.at(t.i0 + 1, t.j0 + 1);
    // per channel w00 p00 + w10 p10 + w01 p01 + w11 p11, the channel pairs (x, y) and (z, w)
    // as packed sums of scalar products
    auto pair = [&](float2 a00, float2 a10, float2 a01, float2 a11) {
        return add2(add2(add2(mul2s(f2(t.w00, t.w00), a00), mul2s(f2(t.w10, t.w10), a10)),
                         mul2s(f2(t.w01, t.w01), a01)),
                    mul2s(f2(t.w11, t.w11), a11));
    };
    const float2 xy = pair(f2(p00.x, p00.y), f2(p10.x, p10.y), f2(p01.x, p01.y), f2(p11.x, p11.y));
    const float2 zw = pair(f2(p00.z, p00.w), f2(p10.z, p10.w), f2(p01.z, p01.w), f2(p11.z, p11.w));
    return make_float4(xy.x, xy.y, zw.x, zw.y);
}

template <class Acc>
GLS_DI float4 sample4(const Acc& im, float u, float v, int w, int h) {
    return sample4(im, bilinear_tap(u, v, w, h));
}

// One axis of a tap resolved against a tile staged in shared memory: i0, i1 are the texel
// positions of the two taps relative to the tile (for a row axis already multiplied by the
// tile's row length), oma = 1 - a.  sample over the tile then forms the weights and the
// blend exactly as sample4 does.
struct TabTap {
    int i0, i1;
    float a, oma;
};

// taps clamped to an image of n texels (clamp-to-edge), then made relative to the tile
// origin org; cap bounds the result to the tile for memory safety
GLS_DI TabTap tab_tap(Tap1 t, int n, int org, int cap, int ld) {
    TabTap r;
    r.i0 = clampi(clampi(t.i0, 0, n - 1) - org, 0, cap - 1) * ld;
    r.i1 = clampi(clampi(t.i0 + 1, 0, n - 1) - org, 0, cap - 1) * ld;
    r.a = t.a;
    r.oma = 1.0f - t.a;
    return r;
}

// taps into a tile that already holds the clamped image around its edges
GLS_DI TabTap tab_tap_tile(Tap1 t, int org, int cap, int ld) {
    TabTap r;
    r.i0 = clampi(t.i0 - org, 0, cap - 1) * ld;
    r.i1 = clampi(t.i0 + 1 - org, 0, cap - 1) * ld;
    r.a = t.a;
    r.oma = 1.0f - t.a;
    return r;
}

GLS_DI float4 tab_sample4(const float4* s, const TabTap& tx, const TabTap& ty) {
    const float w00 = tx.oma * ty.oma, w10 = tx.a * ty.oma, w01 = tx.oma * ty.a, w11 = tx.a * ty.a;
    const float4 p00 = s[ty.i0 + tx.i0], p10 = s[ty.i0 + tx.i1];
    const float4 p01 = s[ty.i1 + tx.i0], p11 = s[ty.i1 + tx.i1];
    // the channel pairs (x, y) and (z, w) as packed sums of scalar products, each lane summed
    // in the order of w00 p00 + w10 p10 + w01 p01 + w11 p11
    auto pair = [&](float2 a00, float2 a10, float2 a01, float2 a11) {
        return add2(add2(add2(mul2s(f2(w00, w00), a00), mul2s(f2(w10, w10), a10)), mul2s(f2(w01, w01), a01)),
                    mul2s(f2(w11, w11), a11));
    };
    const float2 xy = pair(f2(p00.x, p00.y), f2(p10.x, p10.y), f2(p01.x, p01.y), f2(p11.x, p11.y));
    const float2 zw = pair(f2(p00.z, p00.w), f2(p10.z, p10.w), f2(p01.z, p01.w), f2(p11.z, p11.w));
    return make_float4(xy.x, xy.y, zw.x, zw.y);
}

GLS_DI float tab_sample_x(const float4* s, const TabTap& tx, const TabTap& ty) {
    const float w00 = tx.oma * ty.oma, w10 = tx.a * ty.oma, w01 = tx.oma * ty.a, w11 = tx.a * ty.a;
    return w00 * s[ty.i0 + tx.i0].x + w10 * s[ty.i0 + tx.i1].x + w01 * s[ty.i1 + tx.i0].x +
           w11 * s[ty.i1 + tx.i1].x;
}

GLS_DI float tab_sample1(const float* s, const TabTap& tx, const TabTap& ty) {
    const float w00 = tx.oma * ty.oma, w10 = tx.a * ty.oma, w01 = tx.oma * ty.a, w11 = tx.a * ty.a;
    return w00 * s[ty.i0 + tx.i0] + w10 * s[ty.i0 + tx.i1] + w01 * s[ty.i1 + tx.i0] + w11 * s[ty.i1 + tx.i1];
}

// Two samples at once (a at (ax, ay), b at (bx, by)), each lane the value of tab_sample1 /
// tab_sample_x: scalar weights and products, the sums as one packed chain.
template <class V>
GLS_DI float2 tab_sample_pair(V v, const TabTap& ax, const TabTap& ay, const TabTap& bx, const TabTap& by) {
    const float a00 = ax.oma * ay.oma, a10 = ax.a * ay.oma, a01 = ax.oma * ay.a, a11 = ax.a * ay.a;
    const float b00 = bx.oma * by.oma, b10 = bx.a * by.oma, b01 = bx.oma * by.a, b11 = bx.a * by.a;
    return add2(add2(add2(mul2s(f2(a00, b00), f2(v(ay.i0 + ax.i0), v(by.i0 + bx.i0))),
                          mul2s(f2(a10, b10), f2(v(ay.i0 + ax.i1), v(by.i0 + bx.i1)))),
                     mul2s(f2(a01, b01), f2(v(ay.i1 + ax.i0), v(by.i1 + bx.i0)))),
                mul2s(f2(a11, b11), f2(v(ay.i1 + ax.i1), v(by.i1 + bx.i1))));
}

GLS_DI float2 tab_sample1_x2(const float* s, const TabTap& ax, const TabTap& ay, const TabTap& bx, const TabTap& by) {
    return tab_sample_pair([s](int i) { return s[i]; }, ax, ay, bx, by);
}

GLS_DI float2 tab_sample_x_x2(const float4* s, const TabTap& ax, const TabTap& ay, const TabTap& bx,
                              const TabTap& by) {
    return tab_sample_pair([s](int i) { return s[i].x; }, ax, ay, bx, by);
}

// ---------------------------------------------------------------------------------------
// Float-float accumulator: TwoSum on the high part, rounding errors collected in the low
// part; products enter exactly through an FMA-based TwoProduct.  Relative error after k
// terms is about k * 2^-48, far below the fp32 rounding of the fitted noise model.
// ---------------------------------------------------------------------------------------
struct FF {
    float hi, lo;
};

GLS_DI void ff_zero(FF& a) {
    a.hi = 0.0f;
    a.lo = 0.0f;
}

GLS_DI void ff_add(FF& a, float x) {
    const float s = __fadd_rn(a.hi, x);
    const float bb = __fsub_rn(s, a.hi);
    const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, err);
}

GLS_DI void ff_add_prod(FF& a, float x, float y) {
    const float p = __fmul_rn(x, y);
    const float e = __fmaf_rn(x, y, -p);
    ff_add(a, p);
    a.lo = __fadd_rn(a.lo, e);
}

GLS_DI double ff_value(const FF& a) { return (double)a.hi + (double)a.lo; }

GLS_DI double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

GLS_DI float warp_min_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

GLS_DI float warp_max_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace gls

#endif  // GLS_DEVICE_CUH
