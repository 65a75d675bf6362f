// k_nlf.cu -- the noise-model regressions of computeNoiseStatistics and
// computeRawNoiseStatistics (CLImage/app/src/main/cpp/pyramidal_denoise.cpp:161-362),
// kept entirely on the device so the pipeline never waits for a host round trip.
//
// The reference fits var = A + B * mean in FP64 over the pixels whose statistics fall in
// [0.001, 0.5] x [0, 0.001] (pass 1), measures the RMS residual (pass 2), and refits on the
// pixels whose squared residual is <= that RMS (pass 3).  Here:
//   pass 1  every thread accumulates the sums of its pixels in float-float (exact
//           products, compensated adds) and converts them to 128-bit fixed point; blocks
//           reduce those exactly (integer adds) to per-block rows;
//   solve 1 the last block to finish pass 1 adds the rows (exact again), rounds each total
//           once to a double, and fits A, B in FP64.  It bounds every pass-1 residual by the extremes of the selected statistics; when
//           even the largest possible squared residual is below a lower bound of the RMS
//           (computed from the sums), pass 3 provably keeps every pass-1 pixel and the
//           pass-1 fit is the answer -- the common case, one pass over the data;
//   pass 2/3 otherwise run as the reference does, per pixel in FP64 (the refit sums of
//           pass 3 travel in fixed point like those of pass 1), each solved by its last block.
#include "gls_nlf.cuh"

namespace gls {

NlfThresholds nlf_thresholds() {
    NlfThresholds t;
    t.m_lo = 0.001f;
    while ((double)t.m_lo < 0.001) t.m_lo = nextafterf(t.m_lo, 1.0f);
    while ((double)nextafterf(t.m_lo, 0.0f) >= 0.001) t.m_lo = nextafterf(t.m_lo, 0.0f);
    t.m_hi = 0.5f;
    t.v_lo = 0.0f;
    t.v_hi = 0.001f;
    while ((double)t.v_hi > 0.001) t.v_hi = nextafterf(t.v_hi, 0.0f);
    while ((double)nextafterf(t.v_hi, 1.0f) <= 0.001) t.v_hi = nextafterf(t.v_hi, 1.0f);
    return t;
}

gls_status nlf_fit_raw_scaled(gls_ctx* ctx, const void* scaled, bool half, int w, int h, int pitch, int bayer,
                              NlfScratch s, float* out_dev, bool half_stats) {
    if (half) {
        RawScaledSrc<__half> src{{(const __half*)scaled, w, h, pitch}, bayer, half_stats};
        return run_fit<4, 4>(ctx, src, w / 2, h / 2, s, out_dev);
    }
    RawScaledSrc<float> src{{(const float*)scaled, w, h, pitch}, bayer, half_stats};
    return run_fit<4, 4>(ctx, src, w / 2, h / 2, s, out_dev);
}

gls_status nlf_fit_raw_u16(gls_ctx* ctx, const uint16_t* raw, int w, int h, int pitch, int bayer,
                           const float scale_mul[4], float black, bool half_storage, NlfScratch s, float* out_dev,
                           bool half_stats) {
    RawU16Src src;
    src.half_stats = half_stats;
    src.acc.raw = GRaw16{raw, w, h, pitch};
    for (int c = 0; c < 4; c++) src.acc.sm[bayer_dy(bayer, c) * 2 + bayer_dx(bayer, c)] = scale_mul[c];
    src.acc.black = black;
    src.acc.half = half_storage;
    src.bayer = bayer;
    return run_fit<4, 4>(ctx, src, w / 2, h / 2, s, out_dev);
}

gls_status nlf_fit_level(gls_ctx* ctx, const void* img, bool half, int w, int h, int pitch, NlfScratch s,
                         float* out_dev, bool half_stats) {
    if (half) {
        LevelSrc<__half> src{{(const half4*)img, w, h, pitch}, half_stats};
        return run_fit<1, 3>(ctx, src, w, h, s, out_dev);
    }
    LevelSrc<float> src{{(const float4*)img, w, h, pitch}, half_stats};
    return run_fit<1, 3>(ctx, src, w, h, s, out_dev);
}

}  // namespace gls
