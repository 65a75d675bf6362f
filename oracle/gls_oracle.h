// gls_oracle.h -- C interface of the CPU oracle of CLImage's RAW->RGB pipeline.
//
// TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the reference
// pipeline (CLImage/app/src/main/cpp/OpenCL/demosaic.cl, raw_converter.cpp,
// pyramidal_denoise.cpp) used by tests/, __graft_entry__.smoke() and the CPU baseline leg
// of bench.py as the checker.  The product (climage_gb300, include/gls_cuda.h) never links,
// loads or calls it.
//
// Parity pins: the host colour math is checked against the reference's own
// demosaic_utils.cpp/gls_linalg.hpp compiled from the reference sources (oracle/_ref, see
// oracle/Makefile) and the integer unpack against hand-packed words derived from
// src/gls_image_tiff.cpp:53-87; the OpenCL kernels themselves cannot run on this machine
// (no OpenCL platform), so kernel parity rests on this restatement, with the OpenCL
// built-ins fixed by climage_gb300/csrc/gls_clmath.h.
#ifndef GLS_ORACLE_H
#define GLS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Precision policy: how intermediate images are stored and how arithmetic is done.
enum {
    ORACLE_F32 = 0,  // fp32 image storage, fp32 arithmetic (x86 macOS build of the reference)
    ORACLE_F16 = 1,  // fp16 image storage, fp32 arithmetic (the reference as shipped on ARM)
    ORACLE_F64 = 2,  // fp64 everywhere, no fp16 rounding: the error oracle
    ORACLE_F16_STATS = 3,  // ORACLE_F16 with the noise-statistics images in fp16 too, as the
                           // shipped build stores them (rgba_pixel_float, pyramidal_denoise.cpp:162,260-261)
};

typedef struct {
    float luma, chroma, chromaBoost, gradientBoost, sharpening;
} oracle_denoise_params;

typedef struct {
    float contrast, saturation, toneCurveSlope, exposureBias, blacks;
    int localToneMapping;
} oracle_rgb_params;

typedef struct {
    float guidedFilterEps, shadows, highlights, detail;
} oracle_ltm_params;

#define ORACLE_MAX_LEVELS 8

typedef struct {
    int bayer_pattern;  // 0 grbg, 1 gbrg, 2 rggb, 3 bggr
    float black_level;  // in raw DN
    float white_level;
    float exposure_multiplier;
    float scale_mul[4];
    float rgb_cam[9];
    float noise_level;
    int pyramid_levels;     // 4..8
    int denoise_algorithm;  // 0 bilateral, 1 guided fast, 2 guided precise
    int rotate_180;         // interpolateRedBlue writes the frame turned by 180 degrees
    float raw_nlf[4];                            // out
    float pyramid_nlf[ORACLE_MAX_LEVELS][6];     // in: [0] used by the despeckle; out: fitted
    oracle_denoise_params denoise[ORACLE_MAX_LEVELS];
    oracle_rgb_params rgb;
    oracle_ltm_params ltm;
} oracle_params;

// Optional intermediate images (float, RGBA unless noted), filled when non-null.
typedef struct {
    float* scaled_raw;   // w*h, after scaleRawData (and the high-noise branch)
    float* green;        // w*h
    float* linear_rgb;   // w*h*4, after interpolateRedBlue
    float* ycbcr;        // w*h*4, after blendHighlights + transformImage
    float* level0;       // w*h*4, after the luma despeckle / chroma median
    float* denoised0;    // w*h*4, pyramid output (YCbCr, before the inverse transform)
    float* ltm_mask;     // w*h
    float* camera_rgb;   // w*h*4, after the inverse transform
} oracle_taps;

int oracle_threads(void);
void oracle_set_threads(int n);

// Full pipeline.  out_rgba8 (w*h*4) and/or out_rgbaf (w*h*4) may be null.
int oracle_demosaic(const uint16_t* raw, int w, int h, int stride, oracle_params* p, int prec,
                    uint8_t* out_rgba8, float* out_rgbaf, oracle_taps* taps);

// Half-resolution fast path (raw_converter.cpp:188-224): out is (w/2)*(h/2)*4.
int oracle_fast_demosaic(const uint16_t* raw, int w, int h, int stride, const oracle_params* p, int prec,
                         uint8_t* out_rgba8, float* out_rgbaf);

// ---- single stages on float images (values as stored, channel-interleaved) ----
int oracle_scale_raw(const uint16_t* raw, int w, int h, int stride, int bayer, const float scale_mul[4],
                     float black_level_norm, int prec, float* out);
int oracle_raw_noise_statistics(const float* scaled, int w, int h, int bayer, float* mean, float* var);
int oracle_compute_raw_nlf(const float* scaled, int w, int h, int bayer, float out_nlf[8]);
int oracle_interpolate_green(const float* scaled, int w, int h, int bayer, float luma_variance, int prec,
                             float* green);
int oracle_interpolate_red_blue(const float* scaled, const float* green, int w, int h, int bayer,
                                float chroma_variance, int prec, int rotate_180, float* rgba);
int oracle_blend_highlights(const float* in, int w, int h, float clip, int prec, float* out);
int oracle_transform(const float* in, int w, int h, const float m[9], int prec, float* out);
int oracle_despeckle(const float* in, int w, int h, const float var_a[3], const float var_b[3], int prec,
                     float* out);
int oracle_downsample(const float* in, int w, int h, int ow, int oh, int prec, float* out);
int oracle_noise_statistics(const float* in, int w, int h, float* out);
int oracle_compute_nlf(const float* in, int w, int h, float out_nlf[6]);
int oracle_denoise_bilateral(const float* in, int w, int h, const float var_a[3], const float var_b[3],
                             float chroma_boost, float gradient_boost, int prec, float* out);
int oracle_denoise_guided(const float* in, int w, int h, const float var_a[3], const float var_b[3], int prec,
                          float* out);
int oracle_guided_filter(const float* in, int w, int h, int filter_size, const float eps[3], int prec,
                         float* out);
int oracle_reassemble(const float* den0, int w, int h, const float* img1, const float* den1, int w1, int h1,
                      float sharpening, const float nlf[2], int prec, float* out);
int oracle_ltm_mask(const float* in, int w, int h, const float* guide, int gw, int gh,
                    const oracle_ltm_params* ltm, const float m[9], int prec, float* out);
int oracle_convert_to_srgb(const float* in, const float* ltm_mask, int w, int h, const float m[9],
                           const oracle_rgb_params* rgb, uint8_t* out_rgba8, float* out_rgbaf);
int oracle_bayer_to_rgba(const float* scaled, int w, int h, int bayer, int prec, float* out);
int oracle_rgba_to_bayer(const float* rgba, int w, int h, int bayer, int prec, float* out);
int oracle_despeckle_rgba(const float* in, int w, int h, int prec, float* out);
int oracle_denoise_rgba(const float* in, int w, int h, const float raw_variance[4], int prec, float* out);
int oracle_fast_debayer(const float* scaled, int w, int h, int bayer, int prec, float* out);

// Regression on caller-supplied statistics (known-answer tests): m is n x mc, v is n x nc.
int oracle_regress(const float* m, const float* v, long n, int mc, int nc, float* out_ab);

// Host colour math (demosaic_utils.cpp:25-52, 809-822; gls_linalg.hpp:440-556)
void oracle_cam_xyz_coeff(const float cam_xyz[9], float pre_mul[3], float rgb_cam[9]);
void oracle_cam_ycbcr(const float rgb_cam[9], float out[9]);
void oracle_inverse3x3(const float m[9], float out[9]);
void oracle_matmul3x3(const float a[9], const float b[9], float out[9]);

// Packed sensor words -> uint16 samples (src/gls_image_tiff.cpp:53-87); 10-bit is this
// project's extension (4 samples in 5 bytes, big-endian bit order).
long oracle_unpack_bits(const uint8_t* packed, long n_bytes, int bits, uint16_t* out, long max_out);

/* colorCheckerRawStats (demosaic_utils.cpp:411-533): per patch of the 6x4 chart at gmb =
 * {x, y, width, height}, mean[24][4] and var[24][4] of the CFA channels {r, g, b, g2}. */
int oracle_color_checker_raw_stats(const uint16_t* raw, int w, int h, int stride, float black, float white,
                                   int bayer, const int gmb[4], int rotate_180, float mean[96], float var[96]);
/* estimateRawParameters (demosaic_utils.cpp:686-785): cam_xyz, pre_mul (green 1) and the raw
 * NLF slopes; -2 when the fitted matrix gives a camera white <= 1e-5 (the reference throws). */
int oracle_estimate_raw_parameters(const uint16_t* raw, int w, int h, int stride, float black, float white, int bayer,
                                   const int gmb[4], int rotate_180, float cam_xyz[9], float pre_mul[3],
                                   float raw_nlf[4]);

/* DecodeLosslessJPEG (src/gls_dng_lossless_jpeg.cpp:3253-3275): one stream -> its samples
 * (rows x cols x components); info = {width, height, components, precision, predictor,
 * point transform, restart interval, frame components}.  Returns the sample count, -1 for a
 * stream the reference rejects, -2 when max_out is too small. */
long oracle_lj92_decode(const uint8_t* data, long size, uint16_t* out, long max_out, int info[8]);
/* Test encoder: any predictor 1-7, restart every restart_rows rows (0: none). */
long oracle_lj92_encode(const uint16_t* src, int rows, int cols, int comps, int precision, int predictor,
                        int restart_rows, uint8_t* out, long cap);

/* autoWhiteBalance (demosaic_utils.cpp:976-1026): raw uint16 -> wb gains {r, g, b}
 * (green = 1) and the highlight fraction. */
int oracle_auto_white_balance(const uint16_t* raw, int w, int h, int stride, const float rgb_ycbcr[9],
                              const float scale_mul[4], float white, float black, int bayer, float wb[3],
                              float* highlights);

// OpenCL built-ins, exported for tests/test_clmath.py
float oracle_atan2pi(float y, float x);
float oracle_tanh(float x);
float oracle_exp2(float x);
float oracle_log2(float x);
float oracle_pow(float x, float y);
uint16_t oracle_f32_to_f16(float x);
float oracle_f16_to_f32(uint16_t h);

#ifdef __cplusplus
}
#endif

#endif
