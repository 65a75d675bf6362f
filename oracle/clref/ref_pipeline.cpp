// ref_pipeline.cpp -- the reference's own RawConverter::demosaicImage (raw_converter.cpp and
// pyramidal_denoise.cpp, compiled from the reference's sources against host_stub/) run on the
// CPU: its OpenCL host bindings (demosaic_cl.hpp) are supplied here, each running the
// reference's own kernel from demosaic.cl (compiled as C++ against cl_shim.h) over the
// stand-in images with the global size and arguments the reference's binding
// (demosaic_cl.cpp) passes.  TEST INFRASTRUCTURE ONLY: a checker of the oracle's pipeline.
#include <cstring>
#include <type_traits>

#include "raw_converter.hpp"
// the shim and the kernel file after the host headers (their qualifiers and macros would
// disturb them) and in a namespace of their own (the kernel file has its own BayerPattern,
// the host headers their own smoothstep)
namespace clk {
#include "cl_shim.h"
#include CLREF_SOURCE
}
using clk::cl_image;
using clk::float2;
using clk::float3;
using clk::float4;
using clk::sampler_t;
using clk::CLSHIM_U16;
using clk::CLSHIM_U8;
using clk::CLSHIM_F32;
using clk::CLSHIM_F16;
namespace clshim = clk::clshim;

namespace {

template <class T>
cl_image view(const gls::cl_image_2d<T>& im) {
    typedef typename T::dataType D;
    const int kind = std::is_same_v<D, uint16_t> ? CLSHIM_U16
                     : std::is_same_v<D, uint8_t>  ? CLSHIM_U8
                     : std::is_same_v<D, float>    ? CLSHIM_F32
                                                   : CLSHIM_F16;  // the shipped build's __fp16 storage
    return cl_image{im.width, im.height, T::channels, kind, (void*)im.pixels.data()};
}

bool g_mixed = false;
template <class F>
void run(int w, int h, F&& f) {
    clshim::mixed_condition = false;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            clshim::gid[0] = x;
            clshim::gid[1] = y;
            f();
        }
    g_mixed |= clshim::mixed_condition;
}

float3 f3(const gls::Vector<3>& v) { return float3(v[0], v[1], v[2]); }
clk::Matrix3x3 m3(const gls::Matrix<3, 3>& m) {
    clk::Matrix3x3 r;
    for (int i = 0; i < 3; i++) r.m[i] = float3(m[i][0], m[i][1], m[i][2]);
    return r;
}
const sampler_t kLinear = CLK_NORMALIZED_COORDS_TRUE | CLK_ADDRESS_CLAMP_TO_EDGE | CLK_FILTER_LINEAR;

}  // namespace

// demosaic.hpp:30 declares the CFA names (defined in demosaic.cpp, not built here); the host
// code prints them
const char* BayerPatternName[4] = {"GRBG", "GBRG", "RGGB", "BGGR"};

// ---- the host bindings of demosaic_cl.hpp, over the stand-in images ----
void scaleRawData(gls::OpenCLContext*, const gls::cl_image_2d<gls::luma_pixel_16>& rawImage,
                  gls::cl_image_2d<gls::luma_pixel_float>* scaledRawImage, BayerPattern bayerPattern,
                  gls::Vector<4> scaleMul, float blackLevel) {
    cl_image a = view(rawImage), b = view(*scaledRawImage);
    run(scaledRawImage->width / 2, scaledRawImage->height / 2, [&] {
        clk::scaleRawData(&a, &b, bayerPattern, float4(scaleMul[0], scaleMul[1], scaleMul[2], scaleMul[3]), blackLevel);
    });
}

void interpolateGreen(gls::OpenCLContext*, const gls::cl_image_2d<gls::luma_pixel_float>& rawImage,
                      gls::cl_image_2d<gls::luma_pixel_float>* greenImage, BayerPattern bayerPattern, float lumaVariance) {
    cl_image a = view(rawImage), b = view(*greenImage);
    run(greenImage->width, greenImage->height, [&] { clk::interpolateGreen(&a, &b, bayerPattern, lumaVariance); });
}

void interpolateRedBlue(gls::OpenCLContext*, const gls::cl_image_2d<gls::luma_pixel_float>& rawImage,
                        const gls::cl_image_2d<gls::luma_pixel_float>& greenImage,
                        gls::cl_image_2d<gls::rgba_pixel_float>* rgbImage, BayerPattern bayerPattern,
                        float chromaVariance, bool rotate_180) {
    cl_image a = view(rawImage), g = view(greenImage), b = view(*rgbImage);
    run(rgbImage->width, rgbImage->height,
        [&] { clk::interpolateRedBlue(&a, &g, &b, bayerPattern, chromaVariance, rotate_180); });
}

void rawNoiseStatistics(gls::OpenCLContext*, const gls::cl_image_2d<gls::luma_pixel_float>& rawImage,
                        BayerPattern bayerPattern, gls::cl_image_2d<gls::rgba_pixel_float>* meanImage,
                        gls::cl_image_2d<gls::rgba_pixel_float>* varImage) {
    cl_image a = view(rawImage), m = view(*meanImage), v = view(*varImage);
    run(meanImage->width, meanImage->height, [&] { clk::rawNoiseStatistics(&a, bayerPattern, &m, &v); });
}

template <>
void applyKernel<gls::rgba_pixel_float, gls::rgba_pixel_float>(gls::OpenCLContext*, const std::string& name,
                                                                const gls::cl_image_2d<gls::rgba_pixel_float>& in,
                                                                gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    if (name != "noiseStatistics") std::abort();
    run(out->width, out->height, [&] { clk::noiseStatistics(&a, &b); });
}

template <>
void resampleImage<gls::rgba_pixel_float>(gls::OpenCLContext*, const std::string& name,
                                          const gls::cl_image_2d<gls::rgba_pixel_float>& in,
                                          gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    if (name != "downsampleImage") std::abort();
    run(out->width, out->height, [&] { clk::downsampleImage(&a, &b, kLinear); });
}

template <>
void reassembleImage<gls::rgba_pixel_float>(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& d0,
                                            const gls::cl_image_2d<gls::rgba_pixel_float>& i1,
                                            const gls::cl_image_2d<gls::rgba_pixel_float>& d1, float sharpening,
                                            gls::Vector<2> nlf, gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(d0), b = view(i1), c = view(d1), o = view(*out);
    run(out->width, out->height,
        [&] { clk::reassembleImage(&a, &b, &c, sharpening, float2(nlf[0], nlf[1]), &o, kLinear); });
}

void transformImage(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& linearImage,
                    gls::cl_image_2d<gls::rgba_pixel_float>* rgbImage, const gls::Matrix<3, 3>& transform) {
    cl_image a = view(linearImage), b = view(*rgbImage);
    const clk::Matrix3x3 t = m3(transform);
    run(rgbImage->width, rgbImage->height, [&] { clk::transformImage(&a, &b, t); });
}

void convertTosRGB(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& linearImage,
                   const gls::cl_image_2d<gls::luma_pixel_float>& ltmMaskImage, gls::cl_image_2d<gls::rgba_pixel>* rgbImage,
                   const DemosaicParameters& dp) {
    cl_image a = view(linearImage), k = view(ltmMaskImage), b = view(*rgbImage);
    const clk::Matrix3x3 t = m3(dp.rgb_cam);
    const auto& r = dp.rgbConversionParameters;
    clk::RGBConversionParameters p;
    p.contrast = r.contrast;
    p.saturation = r.saturation;
    p.toneCurveSlope = r.toneCurveSlope;
    p.exposureBias = r.exposureBias;
    p.blacks = r.blacks;
    p.localToneMapping = r.localToneMapping;
    run(rgbImage->width, rgbImage->height, [&] { clk::convertTosRGB(&a, &k, &b, t, p); });
}

void despeckleImage(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in, const gls::Vector<3>& var_a,
                    const gls::Vector<3>& var_b, gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    run(out->width, out->height, [&] { clk::despeckleLumaMedianChromaImage(&a, f3(var_a), f3(var_b), &b); });
}

void denoiseImage(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in, const gls::Vector<3>& var_a,
                  const gls::Vector<3>& var_b, float chromaBoost, float gradientBoost,
                  gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    run(out->width, out->height,
        [&] { clk::denoiseImage(&a, f3(var_a), f3(var_b), chromaBoost, gradientBoost, &b); });
}

void denoiseImageGuided(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in,
                        const gls::Vector<3>& var_a, const gls::Vector<3>& var_b,
                        gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    run(out->width, out->height, [&] { clk::denoiseImageGuided(&a, f3(var_a), f3(var_b), &b); });
}

void localToneMappingMask(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in,
                          const gls::cl_image_2d<gls::rgba_pixel_float>& guide, const LTMParameters& l,
                          const gls::Matrix<3, 3>& transform, gls::cl_image_2d<gls::luma_pixel_float>* out) {
    cl_image a = view(in), g = view(guide), b = view(*out);
    clk::LTMParameters p;
    p.guidedFilterEps = l.guidedFilterEps;
    p.shadows = l.shadows;
    p.highlights = l.highlights;
    p.detail = l.detail;
    const clk::Matrix3x3 t = m3(transform);
    run(out->width, out->height, [&] { clk::localToneMappingMaskImage(&a, &g, p, t, &b, kLinear); });
}

void bayerToRawRGBA(gls::OpenCLContext*, const gls::cl_image_2d<gls::luma_pixel_float>& raw,
                    gls::cl_image_2d<gls::rgba_pixel_float>* rgba, BayerPattern bayerPattern) {
    cl_image a = view(raw), b = view(*rgba);
    run(rgba->width, rgba->height, [&] { clk::bayerToRawRGBA(&a, &b, bayerPattern); });
}

void rawRGBAToBayer(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& rgba,
                    gls::cl_image_2d<gls::luma_pixel_float>* raw, BayerPattern bayerPattern) {
    cl_image a = view(rgba), b = view(*raw);
    run(rgba.width, rgba.height, [&] { clk::rawRGBAToBayer(&a, &b, bayerPattern); });
}

void denoiseRawRGBAImage(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in,
                         const gls::Vector<4> rv, gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    run(out->width, out->height, [&] { clk::denoiseRawRGBAImage(&a, float4(rv[0], rv[1], rv[2], rv[3]), &b); });
}

void despeckleRawRGBAImage(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in,
                           gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    run(out->width, out->height, [&] { clk::despeckleRawRGBAImage(&a, &b); });
}

void blendHighlightsImage(gls::OpenCLContext*, const gls::cl_image_2d<gls::rgba_pixel_float>& in, float clip,
                          gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    cl_image a = view(in), b = view(*out);
    run(out->width, out->height, [&] { clk::blendHighlightsImage(&a, clip, &b); });
}

extern "C" {

// The reference's RawConverter::demosaicImage on a raw frame; returns -1 when a kernel met a
// vector condition whose components disagree (see cl_shim.h).  params: black, white,
// exposure_multiplier, noise_level, scale_mul[4], rgb_cam[9], raw_nlf[4], pyramid_nlf[30],
// denoise[25] (luma, chroma, chromaBoost, gradientBoost, sharpening per level), rgb[5],
// ltm[4]; out: RGBA8; raw_nlf_out[4], pyramid_nlf_out[30]: the updated noise model.
int ref_raw_converter(const uint16_t* raw, int w, int h, int bayer, const float* params, int local_tone_mapping, int rotate_180,
                      uint8_t* out, float* raw_nlf_out, float* pyramid_nlf_out) {
    g_mixed = false;
    const float* p = params;
    DemosaicParameters dp;
    dp.bayerPattern = (BayerPattern)bayer;
    dp.black_level = p[0];
    dp.white_level = p[1];
    dp.exposure_multiplier = p[2];
    dp.noiseLevel = p[3];
    p += 4;
    for (int i = 0; i < 4; i++) dp.scale_mul[i] = *p++;
    for (int i = 0; i < 9; i++) dp.rgb_cam[i / 3][i % 3] = *p++;
    for (int i = 0; i < 4; i++) dp.noiseModel.rawNlf[i] = *p++;
    for (int i = 0; i < 30; i++) dp.noiseModel.pyramidNlf[i / 6][i % 6] = *p++;
    for (int l = 0; l < 5; l++) {
        auto& d = dp.denoiseParameters[l];
        d.luma = *p++;
        d.chroma = *p++;
        d.chromaBoost = *p++;
        d.gradientBoost = *p++;
        d.sharpening = *p++;
    }
    auto& r = dp.rgbConversionParameters;
    r.contrast = *p++;
    r.saturation = *p++;
    r.toneCurveSlope = *p++;
    r.exposureBias = *p++;
    r.blacks = *p++;
    r.localToneMapping = local_tone_mapping;
    auto& l = dp.ltmParameters;
    l.guidedFilterEps = *p++;
    l.shadows = *p++;
    l.highlights = *p++;
    l.detail = *p++;

    gls::OpenCLContext ctx;
    RawConverter rc(&ctx);
    gls::image<gls::luma_pixel_16> rawImage(w, h, std::span<gls::luma_pixel_16>((gls::luma_pixel_16*)raw, (size_t)w * h));
    const auto* rgba = rc.demosaicImage(rawImage, &dp, nullptr, rotate_180 != 0);
    std::memcpy(out, rgba->pixels.data(), (size_t)w * h * 4);
    for (int i = 0; i < 4; i++) raw_nlf_out[i] = dp.noiseModel.rawNlf[i];
    for (int i = 0; i < 30; i++) pyramid_nlf_out[i] = dp.noiseModel.pyramidNlf[i / 6][i % 6];
    return g_mixed ? -1 : 0;
}

}  // extern "C"
