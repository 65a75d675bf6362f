// gls_device.cuh -- device-side building blocks shared by every kernel of the RAW pipeline:
// storage types (fp32 / fp16 images), clamp-to-edge accessors over global or shared
// memory, the linear sampler, and compensated (float-float) accumulators for the
// noise-model regressions.
#ifndef GLS_DEVICE_CUH
#define GLS_DEVICE_CUH

#include <cuda_fp16.h>
#include <stdint.h>

#include "gls_clmath.h"

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

GLS_DI BilinearTap bilinear_tap(float u, float v, int w, int h) {
    const float fu = u * (float)w - 0.5f;
    const float fv = v * (float)h - 0.5f;
    const float i0f = floorf(fu), j0f = floorf(fv);
    float a = fu - i0f, b = fv - j0f;
    a = floorf(a * 256.0f + 0.5f) * 0.00390625f;
    b = floorf(b * 256.0f + 0.5f) * 0.00390625f;
    BilinearTap t;
    t.i0 = (int)i0f;
    t.j0 = (int)j0f;
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
    float4 r;
    r.x = t.w00 * p00.x + t.w10 * p10.x + t.w01 * p01.x + t.w11 * p11.x;
    r.y = t.w00 * p00.y + t.w10 * p10.y + t.w01 * p01.y + t.w11 * p11.y;
    r.z = t.w00 * p00.z + t.w10 * p10.z + t.w01 * p01.z + t.w11 * p11.z;
    r.w = t.w00 * p00.w + t.w10 * p10.w + t.w01 * p01.w + t.w11 * p11.w;
    return r;
}

template <class Acc>
GLS_DI float4 sample4(const Acc& im, float u, float v, int w, int h) {
    return sample4(im, bilinear_tap(u, v, w, h));
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
