// gls_fused.h -- argument blocks and launchers of the fused pipeline kernels (k_fused.cu).
#ifndef GLS_FUSED_H
#define GLS_FUSED_H

#include "gls_internal.h"
#include "gls_pixel_ops.cuh"

namespace gls {

struct RawPass1Args {
    const uint16_t* raw;
    int w, h, pitch;
    int bayer;
    float sm[4];  // scale factor per (y & 1) * 2 + (x & 1)
    float black;
    NlfThresholds th;
    NlfScratch nlf;  // regression scratch (set by the launcher)
    float* nlf_out;  // fitted {A0..3, B0..3}
    int sums_exact;  // set by the launcher: every 5x5 sum and its square lie where x / 25 has its exact shortcut
    int stats_half;  // the statistics rounded to binary16 before the fit (GLS_STORAGE_F16_STATS)
    int tma;         // the raw image's tensor map is valid (set by the launcher)
};

struct DemosaicArgs {
    const void* in;  // uint16 raw (scaled on the fly) or the scaled raw image
    int w, h, in_pitch;
    int bayer;
    float sm[4];
    float black;
    const float* rawB_dev;  // fitted raw noise model B[0..3] (or null: lv_host / cv_host)
    float lv_host, cv_host;
    Mat3 cam_ycbcr;
    float va0, vb0;  // luma despeckle noise model (pyramidNlf[0])
    half4* level0;
    int l0_pitch;
    float* tap_scaled;
    float* tap_green;
    int tap_pitch;
    // learned stage: with cnn_in set, the kernel stops after interpolateRedBlue and writes
    // the network input [h][w][4] = (R, G, B, sigma), sigma = sqrt(A1 + B1 * G) from the
    // fitted raw noise model (rawA_dev = A[0..3])
    float* cnn_in;
    const float* rawA_dev;
    // the split form (two kernels): the green image between them, in the storage precision
    void* green;
    int green_pitch;
};

// After the learned stage: linear RGB + the network's residual, blendHighlights,
// cam -> YCbCr, despeckle -> level 0, and the level-0 noise-model multiplier
// 2 sigmoid(logit) per pixel.
struct PostCnnArgs {
    const float* cnn_in;  // [h][w][4]
    const float* head;    // [h][w][4]: strength logit, residual RGB in units of sigma
    int w, h;
    Mat3 cam_ycbcr;
    float va0, vb0;
    half4* level0;
    int l0_pitch;
    float* strength;      // [h][w]
};

struct LevelPass1Args {
    const void* in;
    int w, h, pitch;
    void* out;  // downsampled level (null for the coarsest level)
    int ow, oh, opitch;
    NlfThresholds th;
    NlfScratch nlf;  // regression scratch (set by the launcher)
    float* nlf_out;  // fitted {A0..2, B0..2}
    int stats_half;  // the statistics rounded to binary16 before the fit (GLS_STORAGE_F16_STATS)
    int tma;         // the input's tensor map is valid (set by the launcher)
};

// Levels 1 .. L-1 of the pyramid's statistics in one launch (pyramid_stats_kernel): level p
// of the launch is image level p + 1.
struct PyrLevel {
    const void* in;  // the level's image
    int w, h, pitch;
    void* out;  // the next level (null for the coarsest)
    int ow, oh, opitch;
    int tiles_x, first, count;  // its 32x32 tiles: work items [first, first + count)
    NlfScratch nlf;              // its regression scratch (one per level: the fits run together)
    float* nlf_out;              // fitted {A0..2, B0..2}
    unsigned* done;              // per tile: the launch's mark once its downsampled block is written
};
// Device-side state of the launch, zero when first allocated; the last block to leave resets
// the queue and advances the mark, so a captured graph can replay the launch.
struct PyrCtl {
    unsigned queue;  // next work item
    unsigned exits;  // blocks that have left the work loop
    unsigned mark;   // this launch's tiles are marked mark + 1
    unsigned pad;
    unsigned flushed[GLS_MAX_LEVELS];  // per level: tiles whose sums have reached the totals
};
struct PyramidArgs {
    PyrLevel lv[GLS_MAX_LEVELS - 1];
    int nlev, items;
    NlfThresholds th;
    int stats_half;
    PyrCtl* ctl;
    int tma;  // the first level's tensor map is valid
};

struct DenoiseArgs {
    const void* in;
    int w, h, pitch;
    void* out;
    int opitch;
    const void* coarse_img;
    const void* coarse_den;
    int cw, ch, cpitch;
    const float* nlf_dev;
    float mul[6];
    float chroma_boost, gradient_boost, sharpening;
};

struct FinalArgs {
    const half4* level0;
    int w, h, l0_pitch;
    const void* pyr0;
    const void* den1;
    int cw, ch, cpitch;
    const void* guide;
    int gw, gh, gpitch;
    const float* nlf_dev;
    float mul[6];
    float chroma_boost, gradient_boost, sharpening;
    LtmParams ltm;
    Mat3 icy;
    Mat3 rgb_cam;
    RgbParams rgb;
    void* out;
    int opitch;
    float* tap_den;
    float* tap_mask;
    int tap_pitch;
    const float* strength;  // learned stage: level-0 noise-model multiplier per pixel (or null)
    int tile_y0;            // first tile row of the launch (set by the launcher: bands of rows)
};

// Called after each band of output rows [y_begin, y_end) has been launched (the caller
// enqueues work on the band, e.g. its copy to the host, behind it on the same stream).
struct FinalBandFn {
    gls_status (*fn)(void* user, int y_begin, int y_end);
    void* user;
};

gls_status fused_raw_fit(gls_ctx* ctx, const RawPass1Args& a, bool half, NlfScratch s, float* out_dev);
gls_status fused_demosaic(gls_ctx* ctx, const DemosaicArgs& a, bool raw_u16, bool half);
gls_status fused_post_cnn(gls_ctx* ctx, const PostCnnArgs& a, bool half);
gls_status fused_level_fit(gls_ctx* ctx, const LevelPass1Args& a, bool in_half, bool half, NlfScratch s,
                           float* out_dev);
gls_status fused_pyramid_stats(gls_ctx* ctx, const PyramidArgs& a, bool half);
// both bounded waits of the statistics kernels, made to run out (polls each): s's error word
gls_status fused_wait_probe(gls_ctx* ctx, NlfScratch s, unsigned polls);
gls_status fused_denoise(gls_ctx* ctx, const DenoiseArgs& a, bool in_half, bool half, int algo, bool reasm);
// The final stage over the whole frame, or in `bands` bands of tile rows with band->fn
// called after each (bands > 1 needs band).
gls_status fused_final(gls_ctx* ctx, const FinalArgs& a, bool half, int algo, bool ltm, bool out_f32, int bands = 1,
                       const FinalBandFn* band = nullptr);

}  // namespace gls

#endif  // GLS_FUSED_H
