// ref_regress.cpp -- runs the reference's own noise-model regressions,
// computeRawNoiseStatistics and computeNoiseStatistics (pyramidal_denoise.cpp:161-362,
// compiled from the reference's source against host_stub/), on given statistics images.
// The OpenCL kernel launches those functions start with (rawNoiseStatistics, applyKernel
// "noiseStatistics") are replaced by copies of the statistics passed in, so only the host
// code runs.  TEST INFRASTRUCTURE ONLY: a checker of the oracle's regression.
#include <cstring>

#include "pyramidal_denoise.hpp"

namespace {
const float* g_mean = nullptr;
const float* g_var = nullptr;
const float* g_stats = nullptr;

template <typename T>
void fill(gls::cl_image_2d<T>* im, const float* src) {
    for (size_t i = 0; i < im->pixels.size(); i++)
        for (int c = 0; c < T::channels; c++) im->pixels[i][c] = src[i * T::channels + c];
}
}  // namespace

void rawNoiseStatistics(gls::OpenCLContext*, const gls::cl_image_2d<gls::luma_pixel_float>&, BayerPattern,
                        gls::cl_image_2d<gls::rgba_pixel_float>* meanImage,
                        gls::cl_image_2d<gls::rgba_pixel_float>* varImage) {
    fill(meanImage, g_mean);
    fill(varImage, g_var);
}

template <>
void applyKernel<gls::rgba_pixel_float, gls::rgba_pixel_float>(gls::OpenCLContext*, const std::string&,
                                                                const gls::cl_image_2d<gls::rgba_pixel_float>&,
                                                                gls::cl_image_2d<gls::rgba_pixel_float>* out) {
    fill(out, g_stats);
}

extern "C" {

// mean, var: (h / 2) x (w / 2) x 4 quad statistics; out: A0..A3, B0..B3
int ref_regress_raw(const float* mean, const float* var, int w, int h, float out[8]) {
    g_mean = mean;
    g_var = var;
    gls::OpenCLContext ctx;
    gls::cl_image_2d<gls::luma_pixel_float> raw(ctx.clContext(), w, h);
    const auto r = computeRawNoiseStatistics(&ctx, raw, rggb);
    for (int i = 0; i < 8; i++) out[i] = r[i];
    return 0;
}

// stats: h x w x 4 (mean Y, var Y, var Cb, var Cr); out: A0..A2, B0..B2
int ref_regress_level(const float* stats, int w, int h, float out[6]) {
    g_stats = stats;
    gls::OpenCLContext ctx;
    gls::cl_image_2d<gls::rgba_pixel_float> image(ctx.clContext(), w, h);
    const auto r = computeNoiseStatistics(&ctx, image);
    for (int i = 0; i < 6; i++) out[i] = r[i];
    return 0;
}

}  // extern "C"
