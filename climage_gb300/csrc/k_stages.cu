// k_stages.cu -- one CUDA kernel per stage of the reference pipeline, and the C-ABI entry
// points that bind them (demosaic_cl.hpp:23-129 in the reference).  These kernels read
// their inputs through clamp-to-edge global accessors; the fused pipeline kernels in
// k_fused.cu run the same per-pixel arithmetic (gls_pixel_ops.cuh) out of shared memory.
#include <cstring>

#include "gls_internal.h"
#include "gls_pixel_ops.cuh"
#include "gls_stages.h"

namespace gls {

namespace {

constexpr int BX = 32, BY = 8;

inline dim3 grid2(int w, int h) { return dim3((w + BX - 1) / BX, (h + BY - 1) / BY); }

#define PIXEL_XY                                      \
    const int x = blockIdx.x * BX + threadIdx.x;      \
    const int y = blockIdx.y * BY + threadIdx.y;

// ---- a4 ----
template <class SO>
__global__ void scale_raw_kernel(GRaw16 raw, SO* out, int opitch, int bayer, float4 sm4, float black) {
    const int qx = blockIdx.x * BX + threadIdx.x, qy = blockIdx.y * BY + threadIdx.y;
    if (qx >= raw.w / 2 || qy >= raw.h / 2) return;
    const float sm[4] = {sm4.x, sm4.y, sm4.z, sm4.w};
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int x = 2 * qx + bayer_dx(bayer, c), y = 2 * qy + bayer_dy(bayer, c);
        Storage<SO>::st(out + (size_t)y * opitch + x, scale_value(raw.p[(size_t)y * raw.pitch + x], sm[c], black));
    }
}

// ---- a5 ----
template <class S>
__global__ void raw_stats_kernel(GImg1<S> raw, int bayer, float4* mean, int mpitch, float4* var, int vpitch) {
    const int qx = blockIdx.x * BX + threadIdx.x, qy = blockIdx.y * BY + threadIdx.y;
    if (qx >= raw.w / 2 || qy >= raw.h / 2) return;
    float m[4], v[4];
    raw_stats_quad(raw, qx, qy, bayer, m, v);
    mean[(size_t)qy * mpitch + qx] = make_float4(m[0], m[1], m[2], m[3]);
    var[(size_t)qy * vpitch + qx] = make_float4(v[0], v[1], v[2], v[3]);
}

// ---- a7 ----
template <class Acc>
struct DirectSobel {
    const Acc& im;
    int x, y;
    GLS_DI SobelVal operator()(int i, int j) const { return sobel_abs(im, x + i, y + j); }
};

template <class S>
__global__ void green_kernel(GImg1<S> raw, S* out, int opitch, int bayer, float lv_host, const float* lv_dev) {
    PIXEL_XY
    if (x >= raw.w || y >= raw.h) return;
    float g;
    if (green_needs_interp(x, y, bayer)) {
        const float lv = mmax(lv_dev ? *lv_dev : lv_host, 1e-4f);
        DirectSobel<GImg1<S>> sob{raw, x, y};
        g = green_at(raw, x, y, lv, sob);
    } else {
        g = raw.at(x, y);
    }
    Storage<S>::st(out + (size_t)y * opitch + x, g);
}

// ---- a8 ----
// With rotate_180 the reference writes pixel (x, y) at (w - x, h - y) (demosaic.cl:310-313):
// here each thread computes the output pixel (x, y) from the source pixel (w - x, h - y), and
// row 0 and column 0 of the output, which the reference never writes, are zero.
template <class S>
__global__ void red_blue_kernel(GImg1<S> raw, GImg1<S> green, typename Storage<S>::T4* out, int opitch, int bayer,
                                float cv_host, const float* rawB_dev, int rotate_180) {
    PIXEL_XY
    if (x >= raw.w || y >= raw.h) return;
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!rotate_180 || (x > 0 && y > 0)) {
        float cv = rawB_dev ? div_(rawB_dev[0] + rawB_dev[2], 2.0f) : cv_host;
        cv = mmax(cv, 1e-6f);
        const float3 p = rotate_180 ? red_blue_at(raw, green, raw.w - x, raw.h - y, bayer, cv)
                                    : red_blue_at(raw, green, x, y, bayer, cv);
        o = make_float4(p.x, p.y, p.z, 0.0f);
    }
    Storage<S>::st4(out + (size_t)y * opitch + x, o);
}

// ---- a9, a10 ----
template <class S>
__global__ void highlights_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, float clip) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    const float4 p = in.at(x, y);
    const float3 r = blend_highlights_px(make_float3(p.x, p.y, p.z), clip);
    Storage<S>::st4(out + (size_t)y * opitch + x, make_float4(r.x, r.y, r.z, 0.0f));
}

template <class S>
__global__ void transform_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, Mat3 m) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    const float4 p = in.at(x, y);
    const float3 r = transform_px(m, make_float3(p.x, p.y, p.z));
    Storage<S>::st4(out + (size_t)y * opitch + x, make_float4(r.x, r.y, r.z, 0.0f));
}

// ---- a11 ----
template <class S>
__global__ void despeckle_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, float va0, float vb0) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    Storage<S>::st4(out + (size_t)y * opitch + x, despeckle_px(in, x, y, va0, vb0));
}

// ---- a12, a13 ----
template <class S>
__global__ void downsample_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, int ow, int oh) {
    PIXEL_XY
    if (x >= ow || y >= oh) return;
    Storage<S>::st4(out + (size_t)y * opitch + x, downsample_px(in, x, y, ow, oh, in.w, in.h));
}

template <class S>
__global__ void noise_stats_kernel(GImg4<S> in, float4* out, int opitch) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    out[(size_t)y * opitch + x] = noise_stats_px(in, x, y);
}

// ---- a14, a15: the noise model either from host values or from a fitted device slot ----
GLS_DI Nlf6 nlf_get(const NlfArg& a) {
    Nlf6 n;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        n.a[k] = (a.dev ? a.dev[k] : a.host[k]) * a.mul[k];
        n.b[k] = (a.dev ? a.dev[3 + k] : a.host[3 + k]) * a.mul[3 + k];
    }
    return n;
}

template <class S>
__global__ void bilateral_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, NlfArg nlf, float cb,
                                 float gb) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    Storage<S>::st4(out + (size_t)y * opitch + x, bilateral_px(in, x, y, nlf_get(nlf), cb, gb));
}

template <class S>
__global__ void guided_fast_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, NlfArg nlf) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    Storage<S>::st4(out + (size_t)y * opitch + x, guided_fast_px(in, x, y, nlf_get(nlf)));
}

// ---- a17 ----
template <class S>
__global__ void reassemble_kernel(GImg4<S> d0, GImg4<S> i1, GImg4<S> d1, typename Storage<S>::T4* out, int opitch,
                                  float sharpening, NlfArg nlf) {
    PIXEL_XY
    if (x >= d0.w || y >= d0.h) return;
    const Nlf6 n = nlf_get(nlf);
    const float4 r = reassemble_px(d0.at(x, y), i1, d1, x, y, d0.w, d0.h, i1.w, i1.h, sharpening, n.a[0], n.b[0]);
    Storage<S>::st4(out + (size_t)y * opitch + x, r);
}

// ---- a18 ----
template <class S>
__global__ void ltm_kernel(GImg4<S> in, GImg4<S> guide, S* out, int opitch, LtmParams lp, Mat3 m) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    Storage<S>::st(out + (size_t)y * opitch + x, ltm_mask_px(in, guide, x, y, in.w, in.h, guide.w, guide.h, lp, m));
}

// ---- a19 ----
template <class S>
__global__ void srgb_kernel(GImg4<S> in, GImg1<S> mask, uchar4* out8, float4* outf, int opitch, Mat3 m, RgbParams rp) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    const float4 p = in.at(x, y);
    const float lv = rp.localToneMapping ? mask.at(x, y) : 0.0f;
    const float3 r = srgb_px(make_float3(p.x, p.y, p.z), lv, m, rp);
    if (out8) {
        out8[(size_t)y * opitch + x] = make_uchar4(glsm::to_unorm8(r.x), glsm::to_unorm8(r.y), glsm::to_unorm8(r.z), 0);
    } else {
        outf[(size_t)y * opitch + x] = make_float4(r.x, r.y, r.z, 0.0f);
    }
}

// ---- a6 and fastDebayer ----
template <class S>
__global__ void bayer_to_rgba_kernel(GImg1<S> raw, typename Storage<S>::T4* out, int opitch, int bayer) {
    const int qx = blockIdx.x * BX + threadIdx.x, qy = blockIdx.y * BY + threadIdx.y;
    if (qx >= raw.w / 2 || qy >= raw.h / 2) return;
    float v[4];
#pragma unroll
    for (int c = 0; c < 4; c++) v[c] = raw.at(2 * qx + bayer_dx(bayer, c), 2 * qy + bayer_dy(bayer, c));
    Storage<S>::st4(out + (size_t)qy * opitch + qx, make_float4(v[0], v[1], v[2], v[3]));
}

template <class S>
__global__ void rgba_to_bayer_kernel(GImg4<S> rgba, S* raw, int rpitch, int bayer) {
    const int qx = blockIdx.x * BX + threadIdx.x, qy = blockIdx.y * BY + threadIdx.y;
    if (qx >= rgba.w || qy >= rgba.h) return;
    const float4 p = rgba.at(qx, qy);
    const float v[4] = {p.x, p.y, p.z, p.w};
#pragma unroll
    for (int c = 0; c < 4; c++)
        Storage<S>::st(raw + (size_t)(2 * qy + bayer_dy(bayer, c)) * rpitch + 2 * qx + bayer_dx(bayer, c), v[c]);
}

template <class S>
__global__ void despeckle_rgba_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    Storage<S>::st4(out + (size_t)y * opitch + x, despeckle_rgba_px(in, x, y));
}

template <class S>
__global__ void denoise_rgba_kernel(GImg4<S> in, typename Storage<S>::T4* out, int opitch, float4 rv_host,
                                    const float* rawB_dev) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    float rv[4] = {rv_host.x, rv_host.y, rv_host.z, rv_host.w};
    if (rawB_dev) {
#pragma unroll
        for (int k = 0; k < 4; k++) rv[k] = rawB_dev[k];
    }
    Storage<S>::st4(out + (size_t)y * opitch + x, denoise_rgba_px(in, x, y, rv));
}

template <class S>
__global__ void fast_debayer_kernel(GImg1<S> raw, typename Storage<S>::T4* out, int opitch, int bayer) {
    const int qx = blockIdx.x * BX + threadIdx.x, qy = blockIdx.y * BY + threadIdx.y;
    if (qx >= raw.w / 2 || qy >= raw.h / 2) return;
    float v[4];
#pragma unroll
    for (int c = 0; c < 4; c++) v[c] = raw.at(2 * qx + bayer_dx(bayer, c), 2 * qy + bayer_dy(bayer, c));
    Storage<S>::st4(out + (size_t)qy * opitch + qx, make_float4(v[0], div_(v[1] + v[3], 2.0f), v[2], 0.0f));
}

// ---- a16: GuidedFilter (guided_filter.cl) ----
// boxBlurX: sum over the row window, divided by the filter size, written transposed.
template <int C, class SI, class SO>
__global__ void box_blur_x_kernel(const SI* in, int w, int h, int ipitch, SO* out, int opitch, int fs) {
    PIXEL_XY
    if (x >= w || y >= h) return;
    float sum[C];
#pragma unroll
    for (int k = 0; k < C; k++) sum[k] = 0.0f;
    for (int i = -fs / 2; i <= fs / 2; i++) {
        const int xx = clampi(x + i, 0, w - 1);
#pragma unroll
        for (int k = 0; k < C; k++) sum[k] = sum[k] + Storage<SI>::ld(in + ((size_t)y * ipitch + xx) * C + k);
    }
#pragma unroll
    for (int k = 0; k < C; k++) Storage<SO>::st(out + ((size_t)x * opitch + y) * C + k, div_(sum[k], (float)fs));
}

template <class S>
__global__ void gf_products_kernel(GImg4<S> in, float4* p1, float2* p2, float4* ipr, float4* ipg, float4* ipb) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    const float4 s = in.at(x, y);
    const size_t o = (size_t)y * in.w + x;
    p1[o] = make_float4(s.x * s.x, s.x * s.y, s.x * s.z, s.y * s.y);
    p2[o] = make_float2(s.y * s.z, s.z * s.z);
    ipr[o] = make_float4(s.x * s.x, s.x * s.y, s.x * s.z, 0.0f);
    ipg[o] = make_float4(s.y * s.x, s.y * s.y, s.y * s.z, 0.0f);
    ipb[o] = make_float4(s.z * s.x, s.z * s.y, s.z * s.z, 0.0f);
}

template <class S>
__global__ void gf_inv_sigma_kernel(const typename Storage<S>::T4* meanI, const float4* p1, const float2* p2, int w,
                                    int h, NlfArg eps, float4* inv1, float2* inv2) {
    PIXEL_XY
    if (x >= w || y >= h) return;
    const Nlf6 en = nlf_get(eps);
    const float e0 = en.b[0], e1 = en.b[1], e2 = en.b[2];
    const size_t o = (size_t)y * w + x;
    const float4 m = Storage<S>::ld4(meanI + o);
    const float4 a = p1[o];
    const float2 b = p2[o];
    const float vrr = a.x - m.x * m.x + e0 * m.x;
    const float vrg = a.y - m.x * m.y;
    const float vrb = a.z - m.x * m.z;
    const float vgg = a.w - m.y * m.y + e1;
    const float vgb = b.x - m.y * m.z;
    const float vbb = b.y - m.z * m.z + e2;
    const float irr = vgg * vbb - vgb * vgb;
    const float irg = vgb * vrb - vrg * vbb;
    const float irb = vrg * vgb - vgg * vrb;
    const float igg = vrr * vbb - vrb * vrb;
    const float igb = vrb * vrg - vrr * vgb;
    const float ibb = vrr * vgg - vrg * vrg;
    const float det = irr * vrr + irg * vrg + irb * vrb;
    inv1[o] = make_float4(div_(irr, det), div_(irg, det), div_(irb, det), div_(igg, det));
    inv2[o] = make_float2(div_(igb, det), div_(ibb, det));
}

template <class S>
__global__ void gf_ab_kernel(const typename Storage<S>::T4* meanI, float4* ipr, float4* ipg, float4* ipb,
                             const float4* inv1, const float2* inv2, int w, int h) {
    PIXEL_XY
    if (x >= w || y >= h) return;
    const size_t o = (size_t)y * w + x;
    const float4 mp4 = Storage<S>::ld4(meanI + o);
    const float mp[3] = {mp4.x, mp4.y, mp4.z};
    const float4 r4 = ipr[o], g4 = ipg[o], b4 = ipb[o];
    const float rr[3] = {r4.x, r4.y, r4.z}, gg[3] = {g4.x, g4.y, g4.z}, bb[3] = {b4.x, b4.y, b4.z};
    float cr[3], cg[3], cb[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        cr[k] = rr[k] - mp[0] * mp[k];
        cg[k] = gg[k] - mp[1] * mp[k];
        cb[k] = bb[k] - mp[2] * mp[k];
    }
    const float4 i1 = inv1[o];
    const float2 i2 = inv2[o];
    const float irr = i1.x, irg = i1.y, irb = i1.z, igg = i1.w, igb = i2.x, ibb = i2.y;
    float ar[3], ag[3], ab[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        ar[k] = irr * cr[k] + irg * cg[k] + irb * cb[k];
        ag[k] = irg * cr[k] + igg * cg[k] + igb * cb[k];
        ab[k] = irb * cr[k] + igb * cg[k] + ibb * cb[k];
    }
    ipr[o] = make_float4(ar[0], ar[1], ar[2], mp[0] - ar[0] * mp[0] - ag[0] * mp[1] - ab[0] * mp[2]);
    ipg[o] = make_float4(ag[0], ag[1], ag[2], mp[1] - ar[1] * mp[0] - ag[1] * mp[1] - ab[1] * mp[2]);
    ipb[o] = make_float4(ab[0], ab[1], ab[2], mp[2] - ar[2] * mp[0] - ag[2] * mp[1] - ab[2] * mp[2]);
}

template <class S>
__global__ void gf_result_kernel(GImg4<S> in, const float4* abr, const float4* abg, const float4* abb,
                                 typename Storage<S>::T4* out, int opitch) {
    PIXEL_XY
    if (x >= in.w || y >= in.h) return;
    const size_t o = (size_t)y * in.w + x;
    const float4 I = in.at(x, y);
    const float4 r = abr[o], g = abg[o], b = abb[o];
    float4 res;
    res.x = r.x * I.x + g.x * I.y + b.x * I.z + r.w;
    res.y = r.y * I.x + g.y * I.y + b.y * I.z + g.w;
    res.z = r.z * I.x + g.z * I.y + b.z * I.z + b.w;
    res.w = 0.0f;
    Storage<S>::st4(out + (size_t)y * opitch + x, res);
}

// ---- packed raw unpack (src/gls_image_tiff.cpp:53-87; 10-bit by the same bit order) ----
__global__ void unpack_kernel(const uint8_t* in, size_t n_bytes, int bits, uint16_t* out, size_t n) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const size_t bit0 = k * (size_t)bits;
    const size_t byte0 = bit0 >> 3;
    // up to 3 bytes hold a <= 16-bit sample starting at any bit offset
    uint32_t w = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) w = (w << 8) | (byte0 + i < n_bytes ? in[byte0 + i] : 0u);
    const int shift = 24 - (int)(bit0 & 7) - bits;
    out[k] = (uint16_t)((w >> shift) & ((1u << bits) - 1u));
}

}  // namespace

// ------------------------------------------------------------------------------------------
// Launch wrappers used by the C ABI and by the pipeline (gls_stages.h)
// ------------------------------------------------------------------------------------------
#define DISPATCH_S(half, ...)      \
    if (half) {                    \
        using S = __half;          \
        __VA_ARGS__;               \
    } else {                       \
        using S = float;           \
        __VA_ARGS__;               \
    }

template <class S>
static GImg1<S> g1(const ImgRef& r) {
    return GImg1<S>{(const S*)r.ptr, r.w, r.h, r.pitch};
}
template <class S>
static GImg4<S> g4(const ImgRef& r) {
    return GImg4<S>{(const typename Storage<S>::T4*)r.ptr, r.w, r.h, r.pitch};
}
template <class S>
static S* o1(const ImgRef& r) {
    return (S*)r.ptr;
}
template <class S>
static typename Storage<S>::T4* o4(const ImgRef& r) {
    return (typename Storage<S>::T4*)r.ptr;
}

void launch_scale_raw(gls_ctx* ctx, const uint16_t* raw, int w, int h, int rpitch, const ImgRef& out, int bayer,
                      const float sm[4], float black) {
    GRaw16 r{raw, w, h, rpitch};
    const float4 s4 = make_float4(sm[0], sm[1], sm[2], sm[3]);
    DISPATCH_S(out.half, (scale_raw_kernel<S><<<grid2(w / 2, h / 2), dim3(BX, BY), 0, ctx->stream>>>(
                             r, o1<S>(out), out.pitch, bayer, s4, black)));
    ctx->launches++;
}

void launch_raw_stats(gls_ctx* ctx, const ImgRef& scaled, int bayer, float4* mean, int mpitch, float4* var,
                      int vpitch) {
    DISPATCH_S(scaled.half, (raw_stats_kernel<S><<<grid2(scaled.w / 2, scaled.h / 2), dim3(BX, BY), 0, ctx->stream>>>(
                                g1<S>(scaled), bayer, mean, mpitch, var, vpitch)));
    ctx->launches++;
}

void launch_green(gls_ctx* ctx, const ImgRef& scaled, const ImgRef& green, int bayer, float lv, const float* lv_dev) {
    DISPATCH_S(scaled.half, (green_kernel<S><<<grid2(scaled.w, scaled.h), dim3(BX, BY), 0, ctx->stream>>>(
                                g1<S>(scaled), o1<S>(green), green.pitch, bayer, lv, lv_dev)));
    ctx->launches++;
}

void launch_red_blue(gls_ctx* ctx, const ImgRef& scaled, const ImgRef& green, const ImgRef& rgb, int bayer, float cv,
                     const float* rawB_dev, int rotate_180) {
    DISPATCH_S(scaled.half, (red_blue_kernel<S><<<grid2(scaled.w, scaled.h), dim3(BX, BY), 0, ctx->stream>>>(
                                g1<S>(scaled), g1<S>(green), o4<S>(rgb), rgb.pitch, bayer, cv, rawB_dev, rotate_180)));
    ctx->launches++;
}

void launch_highlights(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, float clip) {
    DISPATCH_S(in.half, (highlights_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, clip)));
    ctx->launches++;
}

void launch_transform(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const float m[9]) {
    Mat3 t;
    memcpy(t.m, m, sizeof(t.m));
    DISPATCH_S(in.half, (transform_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, t)));
    ctx->launches++;
}

void launch_despeckle(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, float va0, float vb0) {
    DISPATCH_S(in.half, (despeckle_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, va0, vb0)));
    ctx->launches++;
}

void launch_downsample(gls_ctx* ctx, const ImgRef& in, const ImgRef& out) {
    DISPATCH_S(in.half, (downsample_kernel<S><<<grid2(out.w, out.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, out.w, out.h)));
    ctx->launches++;
}

void launch_noise_stats(gls_ctx* ctx, const ImgRef& in, float4* out, int opitch) {
    DISPATCH_S(in.half, (noise_stats_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), out, opitch)));
    ctx->launches++;
}

void launch_bilateral(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const NlfArg& nlf, float cb, float gb) {
    DISPATCH_S(in.half, (bilateral_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, nlf, cb, gb)));
    ctx->launches++;
}

void launch_guided_fast(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const NlfArg& nlf) {
    DISPATCH_S(in.half, (guided_fast_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, nlf)));
    ctx->launches++;
}

void launch_reassemble(gls_ctx* ctx, const ImgRef& d0, const ImgRef& i1, const ImgRef& d1, const ImgRef& out,
                       float sharpening, const NlfArg& nlf) {
    DISPATCH_S(d0.half, (reassemble_kernel<S><<<grid2(d0.w, d0.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(d0), g4<S>(i1), g4<S>(d1), o4<S>(out), out.pitch, sharpening, nlf)));
    ctx->launches++;
}

void launch_ltm(gls_ctx* ctx, const ImgRef& in, const ImgRef& guide, const ImgRef& out, const LtmParams& lp,
                const float m[9]) {
    Mat3 t;
    memcpy(t.m, m, sizeof(t.m));
    DISPATCH_S(in.half, (ltm_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), g4<S>(guide), o1<S>(out), out.pitch, lp, t)));
    ctx->launches++;
}

void launch_srgb(gls_ctx* ctx, const ImgRef& in, const ImgRef* mask, void* out, bool out_float, int opitch,
                 const float m[9], const RgbParams& rp) {
    Mat3 t;
    memcpy(t.m, m, sizeof(t.m));
    DISPATCH_S(in.half, {
        GImg1<S> mk{nullptr, 1, 1, 1};
        if (mask) mk = g1<S>(*mask);
        srgb_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
            g4<S>(in), mk, out_float ? nullptr : (uchar4*)out, out_float ? (float4*)out : nullptr, opitch, t, rp);
    });
    ctx->launches++;
}

void launch_bayer_to_rgba(gls_ctx* ctx, const ImgRef& raw, const ImgRef& rgba, int bayer) {
    DISPATCH_S(raw.half, (bayer_to_rgba_kernel<S><<<grid2(raw.w / 2, raw.h / 2), dim3(BX, BY), 0, ctx->stream>>>(
                             g1<S>(raw), o4<S>(rgba), rgba.pitch, bayer)));
    ctx->launches++;
}

void launch_rgba_to_bayer(gls_ctx* ctx, const ImgRef& rgba, const ImgRef& raw, int bayer) {
    DISPATCH_S(rgba.half, (rgba_to_bayer_kernel<S><<<grid2(rgba.w, rgba.h), dim3(BX, BY), 0, ctx->stream>>>(
                              g4<S>(rgba), o1<S>(raw), raw.pitch, bayer)));
    ctx->launches++;
}

void launch_despeckle_rgba(gls_ctx* ctx, const ImgRef& in, const ImgRef& out) {
    DISPATCH_S(in.half, (despeckle_rgba_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch)));
    ctx->launches++;
}

void launch_denoise_rgba(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const float rv[4], const float* rawB_dev) {
    const float4 r4 = make_float4(rv[0], rv[1], rv[2], rv[3]);
    DISPATCH_S(in.half, (denoise_rgba_kernel<S><<<grid2(in.w, in.h), dim3(BX, BY), 0, ctx->stream>>>(
                            g4<S>(in), o4<S>(out), out.pitch, r4, rawB_dev)));
    ctx->launches++;
}

void launch_fast_debayer(gls_ctx* ctx, const ImgRef& raw, const ImgRef& rgb, int bayer) {
    DISPATCH_S(raw.half, (fast_debayer_kernel<S><<<grid2(raw.w / 2, raw.h / 2), dim3(BX, BY), 0, ctx->stream>>>(
                             g1<S>(raw), o4<S>(rgb), rgb.pitch, bayer)));
    ctx->launches++;
}

size_t guided_filter_scratch_bytes(int w, int h) {
    const size_t n = (size_t)w * h;
    // meanI (+ transposed temp) in storage precision (<= 16 B/px each), p1, p2, ipr, ipg,
    // ipb, inv1, inv2 and an fp32 transposed temp; each of the 10 buffers starts on a
    // 256-byte boundary, so up to 255 bytes of padding follow each one
    return n * (16 + 16 + 16 + 8 + 16 * 3 + 16 + 8 + 16) + 10 * 256;
}

void launch_guided_filter(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, int fs, const NlfArg& eps, void* scratch) {
    const int w = in.w, h = in.h;
    const size_t n = (size_t)w * h;
    char* p = (char*)scratch;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~(size_t)255;
        return r;
    };
    void* meanI = take(n * 16);
    void* tmpS = take(n * 16);
    float4* p1 = (float4*)take(n * 16);
    float2* p2 = (float2*)take(n * 8);
    float4* ipr = (float4*)take(n * 16);
    float4* ipg = (float4*)take(n * 16);
    float4* ipb = (float4*)take(n * 16);
    float4* inv1 = (float4*)take(n * 16);
    float2* inv2 = (float2*)take(n * 8);
    float4* tmpF = (float4*)take(n * 16);
    cudaStream_t st = ctx->stream;
    const dim3 B(BX, BY);
    DISPATCH_S(in.half, {
        typedef typename Storage<S>::T1 T1;
        // mean_I = boxBlur(input) in storage precision, through a transposed temporary
        {
            // the input may have a pitch: blur rows of the (pitched) input image
            const T1* src = (const T1*)in.ptr;
            box_blur_x_kernel<4, T1, T1><<<grid2(w, h), B, 0, st>>>(src, w, h, in.pitch, (T1*)tmpS, h, fs);
            box_blur_x_kernel<4, T1, T1><<<grid2(h, w), B, 0, st>>>((const T1*)tmpS, h, w, h, (T1*)meanI, w, fs);
        }
        gf_products_kernel<S><<<grid2(w, h), B, 0, st>>>(g4<S>(in), p1, p2, ipr, ipg, ipb);
        auto blur4 = [&](float4* buf) {
            box_blur_x_kernel<4, float, float><<<grid2(w, h), B, 0, st>>>((const float*)buf, w, h, w, (float*)tmpF, h, fs);
            box_blur_x_kernel<4, float, float><<<grid2(h, w), B, 0, st>>>((const float*)tmpF, h, w, h, (float*)buf, w, fs);
        };
        auto blur2 = [&](float2* buf) {
            box_blur_x_kernel<2, float, float><<<grid2(w, h), B, 0, st>>>((const float*)buf, w, h, w, (float*)tmpF, h, fs);
            box_blur_x_kernel<2, float, float><<<grid2(h, w), B, 0, st>>>((const float*)tmpF, h, w, h, (float*)buf, w, fs);
        };
        blur4(p1);
        blur2(p2);
        gf_inv_sigma_kernel<S><<<grid2(w, h), B, 0, st>>>((const typename Storage<S>::T4*)meanI, p1, p2, w, h, eps,
                                                           inv1, inv2);
        blur4(ipr);
        blur4(ipg);
        blur4(ipb);
        gf_ab_kernel<S><<<grid2(w, h), B, 0, st>>>((const typename Storage<S>::T4*)meanI, ipr, ipg, ipb, inv1, inv2, w, h);
        blur4(ipr);
        blur4(ipg);
        blur4(ipb);
        gf_result_kernel<S><<<grid2(w, h), B, 0, st>>>(g4<S>(in), ipr, ipg, ipb, o4<S>(out), out.pitch);
    });
    ctx->launches += 2 + 1 + 2 + 2 + 1 + 6 + 1 + 6 + 1;
}

void launch_unpack(gls_ctx* ctx, const void* packed, size_t n_bytes, int bits, uint16_t* out, size_t n) {
    const int T = 256;
    unpack_kernel<<<(unsigned)((n + T - 1) / T), T, 0, ctx->stream>>>((const uint8_t*)packed, n_bytes, bits, out, n);
    ctx->launches++;
}

}  // namespace gls

// ------------------------------------------------------------------------------------------
// Self-test of the exact shortcuts against the literal operations (gls_selftest).
// ------------------------------------------------------------------------------------------
namespace gls {
namespace {

__device__ uint32_t hash32(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return (uint32_t)x;
}

// a float with a random sign, mantissa and an exponent in [emin, emax]
__device__ float rand_float(uint64_t key, int emin, int emax) {
    const uint32_t h = hash32(key);
    const uint32_t h2 = hash32(key ^ 0x9e3779b97f4a7c15ULL);
    const int e = emin + (int)(h2 % (uint32_t)(emax - emin + 1));
    const uint32_t bits = ((uint32_t)(e + 127) << 23) | (h & 0x7fffffu) | (h2 & 0x80000000u);
    return __uint_as_float(bits);
}

__global__ void selftest_kernel(uint64_t n, uint64_t seed, unsigned long long* bad) {
    unsigned long long b0 = 0, b1 = 0, b2 = 0, b3 = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = seed * 0x100000001b3ULL + 4 * i;
        // division: random and near-halfway numerators
        const float d = fabsf(rand_float(k, -40, 40)) * ((i & 1) ? 1.0f : -1.0f);
        float x = rand_float(k + 1, -40, 40);
        if (i & 2) x = __fmul_rn(d, 1.0f + (float)(hash32(k + 2) & 0xffff) * 1.1920929e-07f);
        FastDiv fd;
        fd.init(d);
        const float q1 = fd(x), q2 = div_(x, d);
        if (__float_as_uint(q1) != __float_as_uint(q2) && !(q1 != q1 && q2 != q2)) b0++;
        // smoothstep: edges and samples of the magnitudes the kernels see
        const float e0 = fabsf(rand_float(k + 3, -20, 2)), e1 = e0 * (1.0f + (float)(hash32(k) & 15));
        const float xs = rand_float(k + 2, -22, 3);
        const float s1 = glsm::smoothstep_(e0, e1, xs), s2 = glsm::smoothstep_ref(e0, e1, xs);
        FastDiv den;
        den.init(e1 - e0);
        const float s3 = glsm::smoothstep_den(e0, den, xs);
        if (__float_as_uint(s1) != __float_as_uint(s2) || __float_as_uint(s3) != __float_as_uint(s2)) b1++;
        // squared-length edge test, including q within a few ulps of e^2
        const float e = fabsf(rand_float(k + 4, -10, 10));
        SqrtGe ge;
        ge.init(e);
        float qv = e * e;
        const int off = (int)(hash32(k + 5) % 64) - 32;
        qv = __uint_as_float(__float_as_uint(qv) + off);
        if ((i & 7) == 0) qv = fabsf(rand_float(k + 6, -25, 25));
        if (ge(qv) != (sqrt_(qv) >= e)) b2++;
        // float -> half rounding
        const float hv = rand_float(k + 7, -26, 16);
        const float h1 = glsm::round_half(hv);
        const float h2 = glsm::f16_bits_to_f32(glsm::f32_to_f16_bits(hv));
        if (__float_as_uint(h1) != __float_as_uint(h2)) b3++;
    }
    if (b0) atomicAdd(&bad[0], b0);
    if (b1) atomicAdd(&bad[1], b1);
    if (b2) atomicAdd(&bad[2], b2);
    if (b3) atomicAdd(&bad[3], b3);
}

// every divisor magnitude of the shared-divisor range [2^-60, 2^31), both signs: rcp_fast
// against the correctly rounded reciprocal
__global__ void selftest_reciprocal_kernel(unsigned long long* bad) {
    constexpr uint64_t kCount = (uint64_t)(158 - 67) << 24;  // exponent fields 67..157, 2^23 mantissas, 2 signs
    unsigned long long b = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kCount; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t bits = ((uint32_t)(67 + (i >> 24)) << 23) | (uint32_t)(i & 0x7fffffu) | ((uint32_t)(i >> 23) & 1u) << 31;
        const float d = __uint_as_float(bits);
        if (__float_as_uint(glsm::rcp_fast(d)) != __float_as_uint(__frcp_rn(d))) b++;
    }
    if (b) atomicAdd(bad, b);
}

}  // namespace
}  // namespace gls

extern "C" gls_status gls_selftest_reciprocal(gls_ctx* ctx, uint64_t* mismatches) {
    using namespace gls;
    if (!ctx || !mismatches) return GLS_ERR_INVALID_ARGUMENT;
    unsigned long long* d = nullptr;
    GLS_CHECK(check_cuda(ctx, cudaMalloc(&d, sizeof(unsigned long long)), "cudaMalloc(selftest)"));
    cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream);
    selftest_reciprocal_kernel<<<8 * (ctx->num_sms > 0 ? ctx->num_sms : 148), 256, 0, ctx->stream>>>(d);
    ctx->launches++;
    unsigned long long h = 0;
    gls_status s = check_cuda(ctx, cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "selftest copy");
    if (s == GLS_OK) s = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "selftest");
    cudaFree(d);
    *mismatches = h;
    return s;
}

extern "C" gls_status gls_selftest(gls_ctx* ctx, uint64_t n, uint64_t seed, uint64_t mismatches[4]) {
    using namespace gls;
    if (!ctx || !mismatches) return GLS_ERR_INVALID_ARGUMENT;
    unsigned long long* d = nullptr;
    GLS_CHECK(check_cuda(ctx, cudaMalloc(&d, 4 * sizeof(unsigned long long)), "cudaMalloc(selftest)"));
    cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), ctx->stream);
    selftest_kernel<<<4 * (ctx->num_sms > 0 ? ctx->num_sms : 148), 256, 0, ctx->stream>>>(n, seed, d);
    ctx->launches++;
    unsigned long long h[4] = {0, 0, 0, 0};
    gls_status s = check_cuda(ctx, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "selftest copy");
    if (s == GLS_OK) s = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "selftest");
    cudaFree(d);
    for (int i = 0; i < 4; i++) mismatches[i] = h[i];
    return s;
}
