/*
 * gls_cuda.h -- C ABI of the GB300-native (sm_103a) RAW->RGB pipeline.
 *
 * Drop-in boundary for CLImage's RAW pipeline: every stage that the reference binds as a
 * C++ free function over gls::cl_image_2d<T> (CLImage/app/src/main/cpp/demosaic_cl.hpp,
 * pyramidal_denoise.hpp, guided_filter.hpp, raw_converter.hpp) has one entry point here,
 * taking plain device pointers and sizes.  The header-only C++ layer in
 * include/gls_cuda.hpp restores the reference's signatures (gls::image<T>,
 * gls::cuda_image_2d<T>, RawConverter) on top of it.
 *
 * Conventions
 *  - Every call returns a gls_status; nothing throws across this boundary.
 *  - Stage calls are asynchronous on the context's stream (gls_ctx_set_stream); calls that
 *    return host values (noise models, the host-buffer pipeline) synchronise that stream.
 *  - Images are described by gls_image_desc: a device pointer, width, height, row pitch
 *    in bytes and a pixel format.  Pitches must be multiples of the pixel size.
 *  - One gls_ctx per host thread; a context is not thread-safe.
 */
#ifndef GLS_CUDA_H
#define GLS_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLS_API __attribute__((visibility("default")))

typedef enum {
    GLS_OK = 0,
    GLS_ERR_INVALID_ARGUMENT = 1,
    GLS_ERR_INVALID_SIZE = 2,
    GLS_ERR_UNSUPPORTED = 3,
    GLS_ERR_CUDA = 4,
    GLS_ERR_OUT_OF_MEMORY = 5,
    GLS_ERR_TIMEOUT = 6,
    GLS_ERR_FORMAT = 7,
    GLS_ERR_BAD_STREAM = 8, /* a compressed stream the reference decoder rejects */
} gls_status;

/* Pixel formats (gls_cl_image.hpp:232-292 maps the same pixel types to OpenCL formats). */
typedef enum {
    GLS_R16_UNORM = 0,   /* luma_pixel_16: raw sensor data */
    GLS_R_F32 = 1,       /* luma_pixel_float, fp32 storage */
    GLS_R_F16 = 2,       /* luma_pixel_float, fp16 storage (the reference as built for ARM) */
    GLS_RGBA_F32 = 3,    /* rgba_pixel_float, fp32 storage */
    GLS_RGBA_F16 = 4,    /* rgba_pixel_float, fp16 storage */
    GLS_RGBA8_UNORM = 5, /* rgba_pixel: the pipeline's product */
    GLS_RGB8_UNORM = 6,  /* rgb_pixel: RawConverter::convertToRGBImage's product */
} gls_pixel_format;

typedef struct {
    void* ptr;
    int width;
    int height;
    int stride_bytes;
    int format; /* gls_pixel_format */
} gls_image_desc;

typedef enum { GLS_GRBG = 0, GLS_GBRG = 1, GLS_RGGB = 2, GLS_BGGR = 3 } gls_bayer_pattern;

/* DenoiseParameters, RGBConversionParameters, LTMParameters (demosaic.hpp:32-56); the
 * two structs passed to kernels keep the layout of demosaic.cl:1026-1031, 1423-1430. */
typedef struct {
    float luma, chroma, chromaBoost, gradientBoost, sharpening;
} gls_denoise_params;

typedef struct {
    float contrast, saturation, toneCurveSlope, exposureBias, blacks;
    int localToneMapping;
} gls_rgb_conversion_params;

typedef struct {
    float guidedFilterEps, shadows, highlights, detail;
} gls_ltm_params;

#define GLS_MAX_LEVELS 8

typedef enum { GLS_DENOISE_BILATERAL = 0, GLS_DENOISE_GUIDED_FAST = 1, GLS_DENOISE_GUIDED_PRECISE = 2 } gls_denoise_algorithm;
/* Storage of the intermediate images: fp32; fp16 (USE_FP16_FLOATS, gls_image.hpp:32, 189-205)
 * with the noise models fitted on fp32 statistics; or fp16 with the noise statistics in fp16
 * as well, exactly as the reference ships (its meanImage/varImage and noise-statistics images
 * are rgba_pixel_float too, pyramidal_denoise.cpp:162, 260-261). */
typedef enum { GLS_STORAGE_F32 = 0, GLS_STORAGE_F16 = 1, GLS_STORAGE_F16_STATS = 2 } gls_storage;

/* DemosaicParameters (demosaic.hpp:61-81), generalised from 5 to pyramid_levels levels.
 * raw_nlf and pyramid_nlf are in/out exactly as NoiseModel is in the reference:
 * pyramid_nlf[0] on input parameterises the despeckle (raw_converter.cpp:144-145), and the
 * pipeline overwrites both with the fitted noise model. */
typedef struct {
    int bayer_pattern;
    float black_level;
    float white_level;
    float exposure_multiplier;
    float scale_mul[4];
    float rgb_cam[9];
    float raw_nlf[4];
    float pyramid_nlf[GLS_MAX_LEVELS][6];
    gls_denoise_params denoise[GLS_MAX_LEVELS];
    float noise_level;
    gls_rgb_conversion_params rgb_conversion;
    gls_ltm_params ltm;
    int pyramid_levels;    /* 4..8 (the reference fixes 5) */
    int denoise_algorithm; /* gls_denoise_algorithm (PyramidalDenoise::DenoiseAlgorithm) */
    int storage;           /* gls_storage of the intermediate images */
    int rotate_180;        /* turn the image by 180 degrees at interpolateRedBlue, as the reference
                              does (pixel (x, y) to (w - x, h - y); row 0 and column 0, which the
                              reference leaves unwritten, are zero); runs the single-stage schedule */
} gls_demosaic_params;

typedef struct gls_ctx gls_ctx;
typedef struct gls_raw_converter gls_raw_converter;

/* ---- context ---- */
GLS_API gls_status gls_ctx_create(int device, gls_ctx** out);
/* Destroy the converters and batches made on a context before the context itself. */
GLS_API gls_status gls_ctx_destroy(gls_ctx* ctx);
GLS_API gls_status gls_ctx_set_stream(gls_ctx* ctx, void* cuda_stream);
GLS_API gls_status gls_ctx_synchronize(gls_ctx* ctx);
GLS_API const char* gls_status_string(gls_status s);
GLS_API const char* gls_ctx_last_error(gls_ctx* ctx);
/* Number of kernels this context has launched so far (all entry points). */
GLS_API uint64_t gls_ctx_kernel_launches(gls_ctx* ctx);
GLS_API const char* gls_version(void);

/* ---- single stages (demosaic_cl.hpp:23-129) ---- */
/* scaleRawData (demosaic_cl.cpp:26-44): raw R16_UNORM -> scaled R_F32/R_F16 */
GLS_API gls_status gls_scale_raw_data(gls_ctx* ctx, const gls_image_desc* raw, const gls_image_desc* scaled,
                                      int bayer_pattern, const float scale_mul[4], float black_level);
/* rawNoiseStatistics (demosaic_cl.cpp:104-126): scaled -> mean, var (RGBA_F32, w/2 x h/2) */
GLS_API gls_status gls_raw_noise_statistics(gls_ctx* ctx, const gls_image_desc* scaled, int bayer_pattern,
                                            const gls_image_desc* mean, const gls_image_desc* var);
/* computeRawNoiseStatistics (pyramidal_denoise.hpp:56-58): returns {A0..A3, B0..B3} */
GLS_API gls_status gls_compute_raw_noise_statistics(gls_ctx* ctx, const gls_image_desc* scaled, int bayer_pattern,
                                                    float out_nlf[8]);
/* interpolateGreen (demosaic_cl.cpp:46-64) */
GLS_API gls_status gls_interpolate_green(gls_ctx* ctx, const gls_image_desc* scaled, const gls_image_desc* green,
                                         int bayer_pattern, float luma_variance);
/* interpolateRedBlue (demosaic_cl.cpp:66-86); rotate_180 turns the output by 180 degrees
 * (demosaic.cl:310-313), row 0 and column 0 zero */
GLS_API gls_status gls_interpolate_red_blue(gls_ctx* ctx, const gls_image_desc* scaled, const gls_image_desc* green,
                                            const gls_image_desc* rgb, int bayer_pattern, float chroma_variance,
                                            int rotate_180);
/* fasteDebayer (demosaic_cl.cpp:88-102): scaled -> RGBA at half resolution */
GLS_API gls_status gls_fast_debayer(gls_ctx* ctx, const gls_image_desc* scaled, const gls_image_desc* rgb,
                                    int bayer_pattern);
/* blendHighlightsImage (demosaic_cl.cpp:506-522); in may equal out */
GLS_API gls_status gls_blend_highlights(gls_ctx* ctx, const gls_image_desc* in, float clip, const gls_image_desc* out);
/* transformImage (demosaic_cl.cpp:210-235); row-major 3x3; in may equal out */
GLS_API gls_status gls_transform_image(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out,
                                       const float transform[9]);
/* despeckleImage (demosaic_cl.cpp:270-291, kernel despeckleLumaMedianChromaImage) */
GLS_API gls_status gls_despeckle_image(gls_ctx* ctx, const gls_image_desc* in, const float var_a[3],
                                       const float var_b[3], const gls_image_desc* out);
/* resampleImage("downsampleImage") (demosaic_cl.cpp:157-180) */
GLS_API gls_status gls_downsample_image(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out);
/* applyKernel("noiseStatistics") (pyramidal_denoise.cpp:162-164): RGBA -> RGBA_F32 */
GLS_API gls_status gls_noise_statistics(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out);
/* computeNoiseStatistics (pyramidal_denoise.hpp:53-54): returns {A0..A2, B0..B2} */
GLS_API gls_status gls_compute_noise_statistics(gls_ctx* ctx, const gls_image_desc* in, float out_nlf[6]);
/* denoiseImage (demosaic_cl.cpp:296-319) */
GLS_API gls_status gls_denoise_image(gls_ctx* ctx, const gls_image_desc* in, const float var_a[3],
                                     const float var_b[3], float chroma_boost, float gradient_boost,
                                     const gls_image_desc* out);
/* denoiseImageGuided (demosaic_cl.cpp:321-337) */
GLS_API gls_status gls_denoise_image_guided(gls_ctx* ctx, const gls_image_desc* in, const float var_a[3],
                                            const float var_b[3], const gls_image_desc* out);
/* GuidedFilter::filter (guided_filter.cpp:195-225) */
GLS_API gls_status gls_guided_filter(gls_ctx* ctx, const gls_image_desc* in, int filter_size, const float eps[3],
                                     const gls_image_desc* out);
/* GuidedFilter::filter that allocates nothing.  It has no counterpart in the reference: it
 * serves callers that must not allocate device memory while they run (a frame loop that
 * shares the GPU with other streams, where cudaMalloc/cudaFree would synchronise or fail
 * under memory pressure; a process whose device footprint is fixed after start-up).
 * Arguments, checks and results are those of gls_guided_filter, bit for bit.  Its scratch
 * is one static device array of GLS_GUIDED_FILTER_NOALLOC_SCRATCH_BYTES (16 MiB), not the
 * context's cudaMalloc'd scratch, so the image may hold at most
 * GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS pixels; a larger one is rejected with
 * GLS_ERR_INVALID_SIZE and a message giving both sizes, and nothing is launched.
 * Set-up: the first call on a device, with the context's device current (required on every
 * call), looks up the array's address there with cudaGetSymbolAddress, which loads the array
 * onto that device; make that first call before any stream capture.  Later calls only launch
 * kernels on the context's stream.  The address is remembered together with the CUDA
 * context it belongs to: after a device reset (cudaDeviceReset) the next call, again before
 * any capture, repeats the set-up in the new context.  Under lazy module loading (CUDA's
 * default) a device holds the 16 MiB from that first call on; with
 * CUDA_MODULE_LOADING=EAGER every context reserves it when it is created.  All calls on a device share the one array: calls whose
 * work overlaps on the GPU (other streams, other contexts or threads) race on it and corrupt
 * each other's results, so serialise them.  Nothing in the array has to start at zero (each
 * call writes every buffer in full before reading it), so no call clears it. */
#define GLS_GUIDED_FILTER_NOALLOC_SCRATCH_BYTES (16u << 20)
#define GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS 116490
GLS_API gls_status gls_guided_filter_noalloc(gls_ctx* ctx, const gls_image_desc* in, int filter_size,
                                             const float eps[3], const gls_image_desc* out);
/* reassembleImage (demosaic_cl.cpp:182-208); den0 may equal out */
GLS_API gls_status gls_reassemble_image(gls_ctx* ctx, const gls_image_desc* den0, const gls_image_desc* img1,
                                        const gls_image_desc* den1, float sharpening, const float nlf[2],
                                        const gls_image_desc* out);
/* localToneMappingMask (demosaic_cl.cpp:339-370) */
GLS_API gls_status gls_local_tone_mapping_mask(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* guide,
                                               const gls_ltm_params* ltm, const float transform[9],
                                               const gls_image_desc* out);
/* convertTosRGB (demosaic_cl.cpp:237-268): out RGBA8_UNORM (the product) or RGBA_F32 */
GLS_API gls_status gls_convert_to_srgb(gls_ctx* ctx, const gls_image_desc* linear, const gls_image_desc* ltm_mask,
                                       const gls_image_desc* out, const float rgb_cam[9],
                                       const gls_rgb_conversion_params* params);
/* bayerToRawRGBA / rawRGBAToBayer (demosaic_cl.cpp:372-406) */
GLS_API gls_status gls_bayer_to_raw_rgba(gls_ctx* ctx, const gls_image_desc* raw, const gls_image_desc* rgba,
                                         int bayer_pattern);
GLS_API gls_status gls_raw_rgba_to_bayer(gls_ctx* ctx, const gls_image_desc* rgba, const gls_image_desc* raw,
                                         int bayer_pattern);
/* despeckleRawRGBAImage / denoiseRawRGBAImage (demosaic_cl.cpp:408-444) */
GLS_API gls_status gls_despeckle_raw_rgba(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out);
GLS_API gls_status gls_denoise_raw_rgba(gls_ctx* ctx, const gls_image_desc* in, const float raw_variance[4],
                                        const gls_image_desc* out);
/* unpack12BitsInto16Bits / unpack14BitsInto16Bits (src/gls_image_tiff.cpp:53-87), plus
 * 10-bit: MSB-first packed samples (device bytes) -> uint16 (device), n_samples outputs. */
GLS_API gls_status gls_unpack_raw_bits(gls_ctx* ctx, const void* packed, size_t n_bytes, int bits, uint16_t* out,
                                       size_t n_samples);

/* Device self-test of the exact arithmetic shortcuts the kernels use (no reference
 * counterpart): over n pseudo-random inputs derived from seed, counts the results that
 * differ from the literal operation -- [0] shared-divisor division vs IEEE division,
 * [1] the clamped smoothstep vs its literal form, [2] the squared-length edge test vs
 * sqrt-then-compare, [3] hardware float->half rounding vs the portable conversion. */
GLS_API gls_status gls_selftest(gls_ctx* ctx, uint64_t n, uint64_t seed, uint64_t mismatches[4]);
/* Exhaustive check of the three-instruction reciprocal the shared-divisor division uses:
 * every float divisor of magnitude in [2^-60, 2^31), both signs, against __frcp_rn;
 * *mismatches = the number that differ (0 expected). */
GLS_API gls_status gls_selftest_reciprocal(gls_ctx* ctx, uint64_t* mismatches);

/* autoWhiteBalance (demosaic_utils.cpp:976-1026): the white-balance gains of a raw
 * R16_UNORM frame (device) -- rgb_ycbcr is cam_ycbcr(rgb_cam), scale_mul the four channel
 * multipliers (normalised to green inside), white and black the raw levels.  Writes the
 * gains {r, g, b} (g = 1) to wb_out and, when not null, the fraction of 2x2 quads with a
 * channel in (0.5, 1] to *highlights; both host memory (the call synchronizes the context's
 * stream).  Bit-identical to the reference's fp32 computation, which runs on 4x4 tiles and
 * keeps its sums in quad order. */
GLS_API gls_status gls_auto_white_balance(gls_ctx* ctx, const gls_image_desc* raw, const float rgb_ycbcr[9],
                                          const float scale_mul[4], float white_level, float black_level,
                                          int bayer_pattern, float wb_out[3], float* highlights);

/* colorCheckerRawStats (demosaic_utils.cpp:411-533): the mean and variance of the CFA channels
 * {r, g, b, g2} over the inner half of each patch of a 6x4 ColorChecker chart at gmb_rect =
 * {x, y, width, height} of a raw R16_UNORM frame (device); mean[24 * 4], var[24 * 4] host
 * outputs, patch order reversed when rotate_180; the call synchronizes the stream. */
GLS_API gls_status gls_color_checker_raw_stats(gls_ctx* ctx, const gls_image_desc* raw, float black_level,
                                               float white_level, int bayer_pattern, const int gmb_rect[4],
                                               int rotate_180, float mean[96], float var[96]);
/* estimateRawParameters (demosaic_utils.cpp:686-785): from the chart's patches, the camera
 * matrix cam_xyz (normalised, row-major 3x3), the white point pre_mul (green 1) and the raw
 * noise slopes {r, g, b, g2} of the six neutral patches; host outputs, bit-identical to the
 * reference's fp32/fp64 arithmetic. */
GLS_API gls_status gls_estimate_raw_parameters(gls_ctx* ctx, const gls_image_desc* raw, float black_level,
                                               float white_level, int bayer_pattern, const int gmb_rect[4],
                                               int rotate_180, float cam_xyz[9], float pre_mul[3], float raw_nlf[4]);

/* The fit half of estimateRawParameters from colorCheckerRawStats' output (mean and var as
 * that call returns them, patch-major, 4 CFA channels each): matrixFromColorChecker
 * (demosaic_utils.cpp:83-129) and the raw noise regression over the six neutral patches
 * (linear_regression, 604-621, as estimateRawParameters applies them at 764-784).  Host only.  GLS_ERR_INVALID_ARGUMENT when the fitted matrix has a
 * white at or below 1e-5, as gls_estimate_raw_parameters. */
GLS_API gls_status gls_fit_color_checker(const float mean[96], const float var[96], float cam_xyz[9],
                                         float pre_mul[3], float raw_nlf[4]);

/* DecodeLosslessJPEG (src/gls_dng_lossless_jpeg.cpp:3253-3275) over the tiles or the strip of
 * a DNG image, as the DNG reader calls it (src/gls_image_tiff.cpp:369-440): data is host
 * memory holding the n_streams lossless-JPEG streams (stream i at offsets[i], sizes[i] bytes:
 * TileOffsets/TileByteCounts, or one StripOffsets/StripByteCounts entry); each stream decodes
 * to tile_width x tile_height samples (for a strip: the image size), placed at tile
 * (i mod tiles_across, i div tiles_across), tiles_across = ceil(out->width / tile_width), and
 * clipped at the image border.  out is the R16_UNORM device image.  The span of data that
 * holds the streams is copied to the device once; the call synchronizes the context's
 * stream.  GLS_ERR_BAD_STREAM for a stream the reference decoder rejects. */
GLS_API gls_status gls_dng_decode_lossless_jpeg(gls_ctx* ctx, const uint8_t* data, size_t data_size, int n_streams,
                                                const uint64_t* offsets, const uint64_t* sizes, int tile_width,
                                                int tile_height, const gls_image_desc* out);

/* The header of one lossless-JPEG stream as the decoder reads it (ReadFileHeader, GetDht,
 * GetDri, GetSof, GetSos: src/gls_dng_lossless_jpeg.cpp:590-1000).  Host only, no context or
 * device needed.  GLS_ERR_BAD_STREAM where gls_dng_decode_lossless_jpeg rejects the header. */
typedef struct {
    int width;            /* samples per component per row (the frame's X) */
    int height;           /* rows (the frame's Y) */
    int components;       /* components of the scan (interleaved per MCU) */
    int precision;        /* bits per sample */
    int predictor;        /* 1-7 (0: none) */
    int point_transform;  /* Pt */
    int restart_interval; /* MCUs per restart interval, 0: none */
    int tables_alike;     /* 1 when every table of the scan splits bits into codewords alike */
} gls_ljpeg_info;
GLS_API gls_status gls_lossless_jpeg_info(const uint8_t* data, size_t size, gls_ljpeg_info* info);

/* ---- host colour math (demosaic_utils.cpp:25-52, 809-822; gls_linalg.hpp:545-556) ---- */
GLS_API gls_status gls_cam_xyz_coeff(const float cam_xyz[9], float pre_mul[3], float rgb_cam[9]);
GLS_API gls_status gls_cam_ycbcr(const float rgb_cam[9], float out[9]);
GLS_API gls_status gls_inverse3x3(const float m[9], float out[9]);

/* ---- the pipeline: RawConverter (raw_converter.hpp:22-62) ---- */
GLS_API gls_status gls_raw_converter_create(gls_ctx* ctx, gls_raw_converter** out);
GLS_API gls_status gls_raw_converter_destroy(gls_raw_converter* conv);
/* RawConverter::demosaicImage (raw_converter.cpp:73-186) on a device raw frame; out is
 * RGBA8_UNORM (the reference product) or RGBA_F32.  params is updated with the fitted
 * noise model (raw_nlf, pyramid_nlf) unless defer_noise_model is set, in which case the
 * call does not synchronise and gls_raw_converter_noise_model() returns it later. */
GLS_API gls_status gls_raw_converter_demosaic(gls_raw_converter* conv, const gls_image_desc* raw,
                                              gls_demosaic_params* params, const gls_image_desc* out,
                                              int defer_noise_model);
GLS_API gls_status gls_raw_converter_noise_model(gls_raw_converter* conv, gls_demosaic_params* params);
/* Device-side status of the converter's statistics kernels (no counterpart in the reference):
 * synchronises the converter's stream and returns GLS_ERR_TIMEOUT, once, when a bounded wait
 * of those kernels ran out since the last call (a tile copy or a coarser tile's mark that
 * did not arrive in time; the frame's noise model is then not valid), else GLS_OK. */
GLS_API gls_status gls_raw_converter_status(gls_raw_converter* conv);
/* Diagnostic of those waits: runs both, limited to `polls` polls (1 .. 2^22), on a mark that
 * nothing sets and an mbarrier that nothing arrives at (nothing in flight), so the next
 * gls_raw_converter_status returns GLS_ERR_TIMEOUT.  Needs one converted frame first. */
GLS_API gls_status gls_raw_converter_wait_probe(gls_raw_converter* conv, unsigned polls);
/* demosaicImage + convertToRGBImage on host buffers (demosaic.cpp:34-51): host uint16
 * raw in, host RGBA8 (out_channels 4) or RGB8 (3) out; copies go through pinned staging. */
GLS_API gls_status gls_raw_converter_demosaic_host(gls_raw_converter* conv, const uint16_t* raw, int width, int height,
                                                   int raw_stride_px, gls_demosaic_params* params, uint8_t* out,
                                                   int out_channels);
/* As gls_raw_converter_demosaic_host with a packed raw frame: the width x height samples as
 * one MSB-first stream of `bits`-bit samples (10/12/14/16), the layout of an uncompressed
 * DNG strip that unpack12BitsInto16Bits / unpack14BitsInto16Bits (src/gls_image_tiff.cpp:
 * 53-87) read; the packed bytes cross to the device and are unpacked there. */
GLS_API gls_status gls_raw_converter_demosaic_packed_host(gls_raw_converter* conv, const uint8_t* packed,
                                                          size_t n_bytes, int bits, int width, int height,
                                                          gls_demosaic_params* params, uint8_t* out,
                                                          int out_channels);
/* RawConverter::fastDemosaicImage (raw_converter.cpp:188-224): half-resolution preview */
GLS_API gls_status gls_raw_converter_fast_demosaic(gls_raw_converter* conv, const gls_image_desc* raw,
                                                   const gls_demosaic_params* params, const gls_image_desc* out);
/* Optional intermediate images of the last demosaic call (device RGBA_F32 unless noted),
 * for parity checks: stage 0 scaled raw (R_F32), 1 green (R_F32), 2 level 0 after the
 * despeckle, 3 denoised level 0 (YCbCr), 4 LTM mask (R_F32). */
GLS_API gls_status gls_raw_converter_set_tap(gls_raw_converter* conv, int stage, const gls_image_desc* dst);
/* Kernel schedule: 0 (default) runs the fused tile kernels; 1 runs one kernel per
 * reference stage (the same arithmetic, every intermediate image materialised).  Both
 * give identical results; GuidedPrecise denoising always uses the single-stage schedule. */
GLS_API gls_status gls_raw_converter_set_mode(gls_raw_converter* conv, int mode);
/* Per-stage timing (the reference's PRINT_EXECUTION_TIME, raw_converter.cpp:22, 97-99,
 * 176-183, with CUDA events instead of queue.finish()).  enable != 0 records an event
 * after every stage of later demosaic calls; the report is a JSON object
 * {"stage": [total_ms, calls], ...} accumulated since profiling was enabled. */
GLS_API gls_status gls_raw_converter_profile(gls_raw_converter* conv, int enable);
GLS_API gls_status gls_raw_converter_profile_report(gls_raw_converter* conv, char* buf, size_t buf_len);

/* ---- the learned stage in the pipeline (see gls_cnn below; no counterpart in the reference) ----
 * With a network set (the converter keeps its own copy), demosaicImage runs it after
 * interpolateRedBlue: its residual (sigma times its RGB output) is added to the linear RGB before blendHighlights and
 * transformImage, and 2 sigmoid(strength logit) multiplies the level-0 denoise noise model
 * per pixel.  An all-zero network reproduces the plain pipeline exactly.  Fused schedule
 * only (not with GuidedPrecise).  cnn = NULL returns to the plain pipeline. */
typedef struct gls_cnn gls_cnn;
GLS_API gls_status gls_raw_converter_set_cnn(gls_raw_converter* conv, gls_cnn* cnn);
/* The network's input for a raw frame (the pipeline up to interpolateRedBlue): dense
 * RGBA_F32 out = (R, G, B, sigma), sigma = sqrt(A1 + B1 * G) of the fitted raw noise model. */
GLS_API gls_status gls_raw_converter_cnn_input(gls_raw_converter* conv, const gls_image_desc* raw,
                                               const gls_demosaic_params* params, const gls_image_desc* out);

/* ---- bursts: demosaicImage over many frames at once ----
 * No counterpart in the reference, where a burst is a loop of demosaicImage calls.  The
 * frames (any sizes, CFA phases, bit depths and parameters) are spread over `lanes`
 * converters, each on its own stream, largest frame first to the least-loaded lane; one
 * frame's stages stay in order while different frames overlap.  gls_raw_batch_demosaic
 * forks the lanes from the context's stream and joins them back with events, so it returns
 * at once, later work on that stream sees every output, and the whole call can be captured
 * in a CUDA graph from that stream once gls_raw_batch_reserve has sized the lanes (nothing
 * is allocated for frames that fit; the single-stage schedule of GuidedPrecise may still
 * allocate on first use).  Noise models are not returned (as with defer_noise_model).  On an
 * error, outputs of the call are undefined. */
typedef struct gls_raw_batch gls_raw_batch;
GLS_API gls_status gls_raw_batch_create(gls_ctx* ctx, int lanes, gls_raw_batch** out);
GLS_API gls_status gls_raw_batch_destroy(gls_raw_batch* batch);
/* Sizes every lane for frames up to width x height, `levels` pyramid levels and `storage`. */
GLS_API gls_status gls_raw_batch_reserve(gls_raw_batch* batch, int width, int height, int levels, int storage);
/* n device frames: raws[i] R16_UNORM, outs[i] RGBA8_UNORM or RGBA_F32 of the same size. */
GLS_API gls_status gls_raw_batch_demosaic(gls_raw_batch* batch, int n, const gls_image_desc* raws,
                                          const gls_demosaic_params* params, const gls_image_desc* outs);
/* n host frames (as gls_raw_converter_demosaic_host); returns when every output is written.
 * Copies run on the lanes' streams, so with pinned host buffers they overlap other frames. */
GLS_API gls_status gls_raw_batch_demosaic_host(gls_raw_batch* batch, int n, const uint16_t* const* raws,
                                               const int* widths, const int* heights, const int* raw_strides_px,
                                               const gls_demosaic_params* params, uint8_t* const* outs,
                                               int out_channels);
/* n packed host frames (as gls_raw_converter_demosaic_packed_host) over the batch's lanes. */
GLS_API gls_status gls_raw_batch_demosaic_packed_host(gls_raw_batch* batch, int n, const uint8_t* const* packed,
                                                      const size_t* n_bytes, const int* bits, const int* widths,
                                                      const int* heights, const gls_demosaic_params* params,
                                                      uint8_t* const* outs, int out_channels);
/* ---- the learned stage: a 5-layer 3x3 BF16 CNN ----
 * No counterpart in the reference.  4 -> 32 -> 32 -> 32 -> 32 -> 4 channels, ReLU between
 * layers, zero-padded borders.  Input per pixel: demosaiced linear R, G, B and the noise
 * sigma; output per pixel: a denoise-strength logit and an RGB residual in units of sigma.  Parameters are a
 * flat FP32 array, per layer W[cout][3][3][cin] then b[cout] (gls_cnn_param_count() in all).
 * All tensors are device NHWC fp32: in [n][h][w][4], out [n][h][w][4], gt [n][h][w][3]. */
GLS_API gls_status gls_cnn_create(gls_ctx* ctx, gls_cnn** out);
GLS_API gls_status gls_cnn_destroy(gls_cnn* cnn);
GLS_API int gls_cnn_param_count(void);
GLS_API gls_status gls_cnn_set_params(gls_cnn* cnn, const float* params, int n);
GLS_API gls_status gls_cnn_get_params(gls_cnn* cnn, float* params, int n);
/* the gradients of the last training step (of the mean losses below) */
GLS_API gls_status gls_cnn_get_grads(gls_cnn* cnn, float* grads, int n);
GLS_API gls_status gls_cnn_forward(gls_cnn* cnn, const float* in, int width, int height, int n, float* out);
/* Tensor-core path of the hidden layers' forward pass (inference and training): 1 (default)
 * 5th-generation tcgen05.mma with tensor-memory accumulators, 0 warp-level mma.sync; the
 * backward pass always uses mma.sync.  A converter given this network copies the choice. */
GLS_API gls_status gls_cnn_set_backend(gls_cnn* cnn, int backend);
GLS_API int gls_cnn_get_backend(gls_cnn* cnn);
/* Synchronises; GLS_ERR_TIMEOUT when a tcgen05 block gave up waiting for its MMAs (reported
 * once: the flag is cleared, and the next status is GLS_OK unless another wait ran out). */
GLS_API gls_status gls_cnn_status(gls_cnn* cnn);
/* Diagnostic of the bounded waits (no counterpart in the reference): runs the tensor-core
 * kernels' mbarrier wait, limited to `polls` polls (1 .. 2^24), on a barrier that nothing
 * arrives at and to which no MMA was committed, so the wait runs out with nothing in flight
 * and the next gls_cnn_status returns GLS_ERR_TIMEOUT. */
GLS_API gls_status gls_cnn_wait_probe(gls_cnn* cnn, unsigned polls);
/* One Adam step (lr > 0; lr = 0 only computes the gradients) on a batch against the clean
 * RGB gt; loss[0] = mean squared error of (input RGB + residual), loss[1] = strength loss. */
GLS_API gls_status gls_cnn_train_step(gls_cnn* cnn, const float* in, const float* gt, int width, int height, int n,
                                      float lr, float loss[2]);

/* every lane runs the learned stage with (its own copy of) this network; NULL: plain */
GLS_API gls_status gls_raw_batch_set_cnn(gls_raw_batch* batch, gls_cnn* cnn);
/* The lane of each frame, as the batch assigns them (frames by decreasing pixel count, each
 * to the lane with the fewest pixels so far; ties to the lower frame index and lane). */
GLS_API gls_status gls_raw_batch_plan(int n, const int* widths, const int* heights, int lanes, int* lane_of);

/* ---- launch-shape tuner (no counterpart in the reference; its work-group sizes come from
 * src/gls_cl.cpp:227-261, computeWorkGroupSizes) ----
 * The demosaic (kernel 0: tiles 44x28, 32x24, 64x32, or split in a green kernel and a
 * red/blue + despeckle kernel through a green image) and the final stage (kernel 1: tiles
 * 32x16, 64x16) are compiled for several tile shapes that compute the same values.  On the
 * first frame of a size (and storage/input form) the converter times every shape on that
 * frame (best of three) and keeps the fastest for the process if it beats shape 0 by 3 %
 * (shape 0 otherwise); frames converted while their stream is
 * captured into a graph, and every frame when the environment sets GLS_TUNE=0, use shape 0
 * until a size has been tuned. */
/* pins kernel's shape for every size (-1: tuned choice again) */
GLS_API gls_status gls_tune_force(int kernel, int shape);
/* forgets every tuned choice and forced shape */
GLS_API gls_status gls_tune_reset(void);
/* number of tuned (kernel, size, flags) entries, and entry `index` with the best time of each
 * shape in ms (zero for shapes the kernel does not have) */
GLS_API int gls_tune_count(void);
GLS_API gls_status gls_tune_entry(int index, int* kernel, int* width, int* height, int* flags, int* shape,
                                  float ms[4]);

#ifdef __cplusplus
}
#endif

#endif /* GLS_CUDA_H */
