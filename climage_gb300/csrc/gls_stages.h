// gls_stages.h -- launchers of the single-stage kernels (k_stages.cu) and of the fused
// pipeline kernels (k_fused.cu), in terms of plain image references.
#ifndef GLS_STAGES_H
#define GLS_STAGES_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "gls_internal.h"

namespace gls {

// A device image: pointer, size, pitch in pixels, fp16 or fp32 storage.
struct ImgRef {
    void* ptr;
    int w, h, pitch;
    bool half;
};

// Noise model source of a denoise kernel: the fitted device slot {A0..A2, B0..B2} (when
// dev is set) or host values, each multiplied by mul[k] as the reference calibrates
// (pyramidal_denoise.cpp:97-101, 119).
struct NlfArg {
    const float* dev;
    float host[6];
    float mul[6];
};

struct LtmParams;
struct RgbParams;

void launch_scale_raw(gls_ctx* ctx, const uint16_t* raw, int w, int h, int rpitch, const ImgRef& out, int bayer,
                      const float sm[4], float black);
void launch_raw_stats(gls_ctx* ctx, const ImgRef& scaled, int bayer, float4* mean, int mpitch, float4* var, int vpitch);
void launch_green(gls_ctx* ctx, const ImgRef& scaled, const ImgRef& green, int bayer, float lv, const float* lv_dev);
// rotate_180: the output turned by 180 degrees as the reference writes it (row 0 and column 0 zero)
void launch_red_blue(gls_ctx* ctx, const ImgRef& scaled, const ImgRef& green, const ImgRef& rgb, int bayer, float cv,
                     const float* rawB_dev, int rotate_180 = 0);
void launch_highlights(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, float clip);
void launch_transform(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const float m[9]);
void launch_despeckle(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, float va0, float vb0);
void launch_downsample(gls_ctx* ctx, const ImgRef& in, const ImgRef& out);
void launch_noise_stats(gls_ctx* ctx, const ImgRef& in, float4* out, int opitch);
void launch_bilateral(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const NlfArg& nlf, float cb, float gb);
void launch_guided_fast(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const NlfArg& nlf);
void launch_reassemble(gls_ctx* ctx, const ImgRef& d0, const ImgRef& i1, const ImgRef& d1, const ImgRef& out,
                       float sharpening, const NlfArg& nlf);
void launch_ltm(gls_ctx* ctx, const ImgRef& in, const ImgRef& guide, const ImgRef& out, const LtmParams& lp,
                const float m[9]);
void launch_srgb(gls_ctx* ctx, const ImgRef& in, const ImgRef* mask, void* out, bool out_float, int opitch,
                 const float m[9], const RgbParams& rp);
void launch_bayer_to_rgba(gls_ctx* ctx, const ImgRef& raw, const ImgRef& rgba, int bayer);
void launch_rgba_to_bayer(gls_ctx* ctx, const ImgRef& rgba, const ImgRef& raw, int bayer);
void launch_despeckle_rgba(gls_ctx* ctx, const ImgRef& in, const ImgRef& out);
void launch_denoise_rgba(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, const float rv[4], const float* rawB_dev);
void launch_fast_debayer(gls_ctx* ctx, const ImgRef& raw, const ImgRef& rgb, int bayer);
size_t guided_filter_scratch_bytes(int w, int h);
// eps: the noise model's B part (b[0..2] of the NlfArg) regularises the covariance
void launch_guided_filter(gls_ctx* ctx, const ImgRef& in, const ImgRef& out, int fs, const NlfArg& eps, void* scratch);
void launch_unpack(gls_ctx* ctx, const void* packed, size_t n_bytes, int bits, uint16_t* out, size_t n);

}  // namespace gls

#endif  // GLS_STAGES_H
