// clref_driver.cpp -- runs single kernels of the reference's own demosaic.cl (compiled as C++
// against cl_shim.h) over images in host memory, with the global sizes the reference's host
// binding uses (demosaic_cl.cpp).  TEST INFRASTRUCTURE ONLY: it checks the oracle's
// restatement against the kernel source it restates; the product never loads it.
//
// Images are float32, interleaved, 1 or 4 channels (the raw frame uint16), as the oracle's
// per-stage entry points take them, so the two can be compared directly.
#include <cstdint>
#include <cstring>

#include <vector>

#include "cl_shim.h"
#include CLREF_SOURCE
#include CLREF_GF_SOURCE

namespace {

// runs f for every work item; -1 when a vector condition had disagreeing components
template <class F>
int run2d(int gw, int gh, F&& f) {
    clshim::mixed_condition = false;
    for (int y = 0; y < gh; y++)
        for (int x = 0; x < gw; x++) {
            clshim::gid[0] = x;
            clshim::gid[1] = y;
            f();
        }
    return clshim::mixed_condition ? -1 : 0;
}

cl_image img(const void* p, int w, int h, int ch, int kind) { return cl_image{w, h, ch, kind, const_cast<void*>(p)}; }

Matrix3x3 mat(const float m[9]) {
    Matrix3x3 r;
    for (int i = 0; i < 3; i++) r.m[i] = float3(m[3 * i], m[3 * i + 1], m[3 * i + 2]);
    return r;
}

const sampler_t kLinear = CLK_NORMALIZED_COORDS_TRUE | CLK_ADDRESS_CLAMP_TO_EDGE | CLK_FILTER_LINEAR;

}  // namespace

extern "C" {

int clref_scale_raw(const uint16_t* raw, int w, int h, int bayer, const float sm[4], float black, float* out) {
    cl_image in = img(raw, w, h, 1, CLSHIM_U16), o = img(out, w, h, 1, CLSHIM_F32);
    return run2d(w / 2, h / 2, [&] { scaleRawData(&in, &o, bayer, float4(sm[0], sm[1], sm[2], sm[3]), black); });
}

int clref_interpolate_green(const float* scaled, int w, int h, int bayer, float luma_variance, float* out) {
    cl_image in = img(scaled, w, h, 1, CLSHIM_F32), o = img(out, w, h, 1, CLSHIM_F32);
    return run2d(w, h, [&] { interpolateGreen(&in, &o, bayer, luma_variance); });
}

int clref_interpolate_red_blue(const float* scaled, const float* green, int w, int h, int bayer, float chroma_variance,
                               int rotate_180, float* out) {
    cl_image in = img(scaled, w, h, 1, CLSHIM_F32), g = img(green, w, h, 1, CLSHIM_F32),
             o = img(out, w, h, 4, CLSHIM_F32);
    return run2d(w, h, [&] { interpolateRedBlue(&in, &g, &o, bayer, chroma_variance, rotate_180); });
}

int clref_blend_highlights(const float* in_p, int w, int h, float clip, float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    return run2d(w, h, [&] { blendHighlightsImage(&in, clip, &o); });
}

int clref_transform(const float* in_p, int w, int h, const float m[9], float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    const Matrix3x3 t = mat(m);
    return run2d(w, h, [&] { transformImage(&in, &o, t); });
}

int clref_noise_statistics(const float* in_p, int w, int h, float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    return run2d(w, h, [&] { noiseStatistics(&in, &o); });
}

int clref_raw_noise_statistics(const float* scaled, int w, int h, int bayer, float* mean, float* var) {
    cl_image in = img(scaled, w, h, 1, CLSHIM_F32), m = img(mean, w / 2, h / 2, 4, CLSHIM_F32),
             v = img(var, w / 2, h / 2, 4, CLSHIM_F32);
    return run2d(w / 2, h / 2, [&] { rawNoiseStatistics(&in, bayer, &m, &v); });
}

int clref_denoise_bilateral(const float* in_p, int w, int h, const float var_a[3], const float var_b[3],
                            float chroma_boost, float gradient_boost, float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    const float3 a(var_a[0], var_a[1], var_a[2]), b(var_b[0], var_b[1], var_b[2]);
    return run2d(w, h, [&] { denoiseImage(&in, a, b, chroma_boost, gradient_boost, &o); });
}

int clref_downsample(const float* in_p, int w, int h, int ow, int oh, float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, ow, oh, 4, CLSHIM_F32);
    return run2d(ow, oh, [&] { downsampleImage(&in, &o, kLinear); });
}

int clref_reassemble(const float* den0, int w, int h, const float* img1, const float* den1, int w1, int h1,
                     float sharpening, const float nlf[2], float* out) {
    cl_image d0 = img(den0, w, h, 4, CLSHIM_F32), i1 = img(img1, w1, h1, 4, CLSHIM_F32),
             d1 = img(den1, w1, h1, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    return run2d(w, h, [&] { reassembleImage(&d0, &i1, &d1, sharpening, float2(nlf[0], nlf[1]), &o, kLinear); });
}

int clref_ltm_mask(const float* in_p, int w, int h, const float* guide, int gw, int gh, const float ltm[4],
                   const float m[9], float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), g = img(guide, gw, gh, 4, CLSHIM_F32),
             o = img(out, w, h, 1, CLSHIM_F32);
    LTMParameters p;
    p.guidedFilterEps = ltm[0];
    p.shadows = ltm[1];
    p.highlights = ltm[2];
    p.detail = ltm[3];
    const Matrix3x3 t = mat(m);
    return run2d(w, h, [&] { localToneMappingMaskImage(&in, &g, p, t, &o, kLinear); });
}

// out: RGBA8 (out_u8) or RGBA fp32 (out_f32), whichever is not null
int clref_convert_to_srgb(const float* in_p, const float* mask, int w, int h, const float m[9], const float rgb[5],
                          int local_tone_mapping, uint8_t* out_u8, float* out_f32) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), k = img(mask, w, h, 1, CLSHIM_F32);
    cl_image o = out_u8 ? img(out_u8, w, h, 4, CLSHIM_U8) : img(out_f32, w, h, 4, CLSHIM_F32);
    RGBConversionParameters p;
    p.contrast = rgb[0];
    p.saturation = rgb[1];
    p.toneCurveSlope = rgb[2];
    p.exposureBias = rgb[3];
    p.blacks = rgb[4];
    p.localToneMapping = local_tone_mapping;
    const Matrix3x3 t = mat(m);
    return run2d(w, h, [&] { convertTosRGB(&in, &k, &o, t, p); });
}

int clref_fast_debayer(const float* scaled, int w, int h, int bayer, float* out) {
    cl_image in = img(scaled, w, h, 1, CLSHIM_F32), o = img(out, w / 2, h / 2, 4, CLSHIM_F32);
    return run2d(w / 2, h / 2, [&] { fastDebayer(&in, &o, bayer); });
}

int clref_bayer_to_rgba(const float* scaled, int w, int h, int bayer, float* out) {
    cl_image in = img(scaled, w, h, 1, CLSHIM_F32), o = img(out, w / 2, h / 2, 4, CLSHIM_F32);
    return run2d(w / 2, h / 2, [&] { bayerToRawRGBA(&in, &o, bayer); });
}

int clref_rgba_to_bayer(const float* rgba, int qw, int qh, int bayer, float* out) {
    cl_image in = img(rgba, qw, qh, 4, CLSHIM_F32), o = img(out, 2 * qw, 2 * qh, 1, CLSHIM_F32);
    return run2d(qw, qh, [&] { rawRGBAToBayer(&in, &o, bayer); });
}

int clref_denoise_rgba(const float* in_p, int w, int h, const float raw_variance[4], float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    const float4 rv(raw_variance[0], raw_variance[1], raw_variance[2], raw_variance[3]);
    return run2d(w, h, [&] { denoiseRawRGBAImage(&in, rv, &o); });
}

int clref_denoise_guided(const float* in_p, int w, int h, const float var_a[3], const float var_b[3], float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    const float3 a(var_a[0], var_a[1], var_a[2]), b(var_b[0], var_b[1], var_b[2]);
    return run2d(w, h, [&] { denoiseImageGuided(&in, a, b, &o); });
}

int clref_despeckle(const float* in_p, int w, int h, const float var_a[3], const float var_b[3], float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    const float3 a(var_a[0], var_a[1], var_a[2]), b(var_b[0], var_b[1], var_b[2]);
    return run2d(w, h, [&] { despeckleLumaMedianChromaImage(&in, a, b, &o); });
}

int clref_despeckle_rgba(const float* in_p, int w, int h, float* out) {
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    return run2d(w, h, [&] { despeckleRawRGBAImage(&in, &o); });
}

// GuidedFilter::filter (guided_filter.cpp:195-225): the reference's host sequence of
// guided_filter.cl kernels, every BoxBlur::blur (guided_filter.cpp:25-48) two boxBlurX passes
// through a transposed temporary; fp32 intermediates, mean_I in the input's storage (fp32).
int clref_guided_filter(const float* in_p, int w, int h, int filter_size, const float eps_p[3], float* out) {
    const size_t n = (size_t)w * h;
    std::vector<float> mean_I(4 * n), inv1(4 * n), inv2(2 * n), cr(4 * n), cg(4 * n), cb(4 * n), tmp(4 * n);
    cl_image in = img(in_p, w, h, 4, CLSHIM_F32), o = img(out, w, h, 4, CLSHIM_F32);
    cl_image mI = img(mean_I.data(), w, h, 4, CLSHIM_F32), s1 = img(inv1.data(), w, h, 4, CLSHIM_F32),
             s2 = img(inv2.data(), w, h, 2, CLSHIM_F32), r = img(cr.data(), w, h, 4, CLSHIM_F32),
             g = img(cg.data(), w, h, 4, CLSHIM_F32), b = img(cb.data(), w, h, 4, CLSHIM_F32);
    int rc = 0;
    auto blur = [&](cl_image* src, cl_image* dst) {
        cl_image t = img(tmp.data(), src->h, src->w, src->ch, CLSHIM_F32);
        rc |= run2d(src->w, src->h, [&] { boxBlurX(src, filter_size, &t); });
        rc |= run2d(t.w, t.h, [&] { boxBlurX(&t, filter_size, dst); });
    };
    const float3 eps(eps_p[0], eps_p[1], eps_p[2]);
    blur(&in, &mI);
    rc |= run2d(w, h, [&] { covMatrixProducts(&in, &s1, &s2); });
    blur(&s1, &s1);
    blur(&s2, &s2);
    rc |= run2d(w, h, [&] { invSigma(&mI, &s1, &s2, eps, &s1, &s2); });
    rc |= run2d(w, h, [&] { meanIpProducts(&in, &r, &g, &b); });
    blur(&r, &r);
    blur(&g, &g);
    blur(&b, &b);
    rc |= run2d(w, h, [&] { computeAb(&mI, &r, &g, &b, &s1, &s2, &r, &g, &b); });
    blur(&r, &r);
    blur(&g, &g);
    blur(&b, &b);
    rc |= run2d(w, h, [&] { computeResult(&in, &r, &g, &b, &o); });
    return rc;
}

}  // extern "C"
