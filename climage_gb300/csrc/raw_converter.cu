// raw_converter.cu -- RawConverter (CLImage/app/src/main/cpp/raw_converter.cpp:73-237) and
// PyramidalDenoise<levels> (pyramidal_denoise.cpp:104-149) on the GPU.
//
// The stage order, the parameter plumbing and the image each stage reads follow the
// reference exactly; the differences are in how the work is scheduled:
//   * the noise-model regressions run on the device (k_nlf.cu), so one frame is a single
//     stream of kernel launches with no host round trip;
//   * working images are allocated for the largest frame and deepest pyramid seen so far
//     and smaller frames run in views of them (the reference sizes them once, by the first
//     frame, and cannot take a larger one);
//   * gls_raw_batch spreads the frames of a burst over converters on their own streams.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "gls_internal.h"
#include "gls_pipeline.h"
#include "gls_pixel_ops.cuh"
#include "gls_fused.h"
#include "gls_stages.h"

using namespace gls;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// half -> float copies for the parity taps
__global__ void tap_copy_kernel(const void* src, bool half, int channels, int w, int h, int spitch, float* dst,
                                int dpitch) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= w || y >= h) return;
    for (int c = 0; c < channels; c++) {
        const size_t si = ((size_t)y * spitch + x) * channels + c;
        const float v = half ? __half2float(((const __half*)src)[si]) : ((const float*)src)[si];
        dst[((size_t)y * dpitch + x) * channels + c] = v;
    }
}

// rows [y0, y1) of an RGBA8 frame packed to RGB8
__global__ void rgba8_to_rgb8_kernel(const uchar4* in, int w, int y0, int y1, uint8_t* out) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = y0 + blockIdx.y * 8 + threadIdx.y;
    if (x >= w || y >= y1) return;
    const uchar4 p = in[(size_t)y * w + x];
    uint8_t* o = out + ((size_t)y * w + x) * 3;
    o[0] = p.x;
    o[1] = p.y;
    o[2] = p.z;
}

}  // namespace

struct gls_raw_converter {
    gls_ctx* ctx = nullptr;
    int w = 0, h = 0, L = 0;
    bool half = false;
    std::vector<DevBuf> owned;
    ImgRef scaled{}, green{}, linA{}, linB{}, mask{}, hnA{}, hnB{}, split_green{};
    ImgRef pyr[GLS_MAX_LEVELS]{}, den[GLS_MAX_LEVELS]{};
    float* nlf_dev = nullptr;  // slot 0: raw {A0..A3, B0..B3}; slot 1+i: level i {A0..A2, B0..B2, -, -}
    void* nlf_scratch = nullptr;
    void* pyr_state = nullptr;  // PyrCtl, then the per-tile marks of levels 1..cap_L-1
    // a lane of a multi-lane burst (gls_raw_batch): levels 1.. take one launch each
    bool overlapped = false;
    void* gf_scratch = nullptr;
    size_t gf_scratch_bytes = 0;
    float* nlf_host = nullptr;  // pinned
    // host-buffer entry point
    uint16_t* raw_dev = nullptr;
    size_t raw_dev_bytes = 0;
    uint8_t* out_dev = nullptr;
    size_t out_dev_bytes = 0;
    uint8_t* packed_dev = nullptr;  // packed 10/12/14-bit raw bytes of the packed host entry point
    size_t packed_dev_bytes = 0;
    // parity taps
    gls_image_desc taps[5]{};
    bool tap_set[5]{};
    // learned stage: this converter's own copy of the network (on its stream), its input,
    // its output and the level-0 noise-model multiplier, all dense [h][w]
    gls_cnn* cnn = nullptr;
    float* cnn_in = nullptr;
    float* cnn_head = nullptr;
    float* strength = nullptr;
    bool learned_alloc = false;

    ~gls_raw_converter() { release(); }

    void release() {
        for (auto& b : owned)
            if (b.p) cudaFree(b.p);
        owned.clear();
        w = h = L = 0;
        cap_w = cap_h = cap_L = 0;
    }

    gls_status alloc(void** p, size_t bytes) {
        GLS_CHECK(check_cuda(ctx, cudaMalloc(p, bytes), "cudaMalloc(working image)"));
        owned.push_back(DevBuf{*p, bytes});
        return GLS_OK;
    }

    gls_status img(ImgRef& r, int iw, int ih, int channels) {
        const size_t es = half ? 2 : 4;
        void* p = nullptr;
        GLS_CHECK(alloc(&p, (size_t)iw * ih * channels * es));
        r = ImgRef{p, iw, ih, iw, half};
        return GLS_OK;
    }

    // level 0 of the pyramid in binary16 (the fused path: the despeckle output is binary16)
    ImgRef level0{};
    // host-buffer conversions: where the final stage's row bands are copied (out null: none)
    struct HostBand {
        uint8_t* out = nullptr;
        int channels = 4, w = 0, h = 0;
        int bands = 0;  // bands whose copies were enqueued
    } host_band;
    static constexpr int kHostBands = 8;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t band_ev[kHostBands + 1] = {};  // after each band's launch; [kHostBands]: the last copy
    bool staged_alloc = false, high_noise_alloc = false;

    // Working images are allocated for a capacity (the largest frame, deepest pyramid seen so
    // far) with the capacity's pitch; a frame that fits is processed in views of them, so a
    // converter that alternates frame sizes neither reallocates nor synchronises.
    int cap_w = 0, cap_h = 0, cap_L = 0;

    void set_views() {
        auto view = [](ImgRef& r, int iw, int ih) {
            if (r.ptr) {
                r.w = iw;
                r.h = ih;
            }
        };
        view(level0, w, h);
        for (int i = 0; i < cap_L - 1; i++) view(pyr[i], w >> (i + 1), h >> (i + 1));
        for (int i = 0; i < cap_L; i++) view(den[i], w >> i, h >> i);
        view(green, w, h);
        view(linA, w, h);
        view(linB, w, h);
        view(mask, w, h);
        view(scaled, w, h);
        view(hnA, w / 2, h / 2);
        view(hnB, w / 2, h / 2);
    }

    gls_status ensure(int width, int height, int levels, bool half_storage) {
        const bool fits = cap_w >= width && cap_h >= height && cap_L >= levels && half_storage == half;
        if (!fits) {
            const bool keep = half_storage == half && cap_w > 0;
            const int nw = keep ? std::max(cap_w, width) : width, nh = keep ? std::max(cap_h, height) : height;
            const int nL = keep ? std::max(cap_L, levels) : levels;
            cudaStreamSynchronize(ctx->stream);
            release();
            for (int i = 0; i < GLS_MAX_LEVELS; i++) pyr[i] = den[i] = ImgRef{};
            green = linA = linB = mask = scaled = hnA = hnB = split_green = ImgRef{};
            staged_alloc = high_noise_alloc = learned_alloc = false;
            half = half_storage;
            {
                void* p = nullptr;
                GLS_CHECK(alloc(&p, (size_t)nw * nh * 8));
                level0 = ImgRef{p, nw, nh, nw, true};
            }
            for (int i = 0; i < nL - 1; i++) GLS_CHECK(img(pyr[i], nw >> (i + 1), nh >> (i + 1), 4));
            for (int i = 1; i < nL; i++) GLS_CHECK(img(den[i], nw >> i, nh >> i, 4));
            void* p = nullptr;
            GLS_CHECK(alloc(&p, (1 + GLS_MAX_LEVELS) * 8 * sizeof(float)));
            nlf_dev = (float*)p;
            // one regression scratch for the raw fit, level 0 and the single-stage schedule, and
            // one per pyramid level for the fused levels 1.. (their fits run in one launch)
            GLS_CHECK(alloc(&nlf_scratch, kNlfScratchBytes * (1 + GLS_MAX_LEVELS)));
            // the regression state starts at zero; every pass leaves it at zero
            GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(nlf_scratch, 0, kNlfScratchBytes * (1 + GLS_MAX_LEVELS), ctx->stream),
                                 "clear regression state"));
            // the pyramid launch's control block and per-tile marks, zero to start with
            size_t marks = 0;
            for (int i = 1; i < nL; i++) marks += (size_t)(((nw >> i) + 31) / 32) * (((nh >> i) + 31) / 32);
            GLS_CHECK(alloc(&pyr_state, sizeof(PyrCtl) + marks * sizeof(unsigned)));
            GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(pyr_state, 0, sizeof(PyrCtl) + marks * sizeof(unsigned), ctx->stream),
                                 "clear pyramid state"));
            gf_scratch = nullptr;
            gf_scratch_bytes = 0;
            cap_w = nw;
            cap_h = nh;
            cap_L = nL;
        }
        w = width;
        h = height;
        L = levels;
        set_views();
        return GLS_OK;
    }

    // the green image between the split demosaic's two kernels (a tile shape of the tuner),
    // allocated on first use at the capacity
    gls_status ensure_split_green() {
        if (split_green.ptr) {
            split_green.w = w;
            split_green.h = h;
            return GLS_OK;
        }
        GLS_CHECK(img(split_green, cap_w, cap_h, 1));
        split_green.w = w;
        split_green.h = h;
        return GLS_OK;
    }

    // working images of the single-stage pipeline, allocated on first use
    gls_status ensure_staged() {
        if (staged_alloc) return GLS_OK;
        GLS_CHECK(img(green, cap_w, cap_h, 1));
        GLS_CHECK(img(linA, cap_w, cap_h, 4));
        GLS_CHECK(img(linB, cap_w, cap_h, 4));
        GLS_CHECK(img(mask, cap_w, cap_h, 1));
        GLS_CHECK(img(den[0], cap_w, cap_h, 4));
        staged_alloc = true;
        GLS_CHECK(ensure_high_noise());
        set_views();
        return GLS_OK;
    }

    gls_status ensure_high_noise() {
        if (high_noise_alloc) return GLS_OK;
        GLS_CHECK(img(scaled, cap_w, cap_h, 1));
        GLS_CHECK(img(hnA, cap_w / 2, cap_h / 2, 4));
        GLS_CHECK(img(hnB, cap_w / 2, cap_h / 2, 4));
        high_noise_alloc = true;
        set_views();
        return GLS_OK;
    }

    gls_status ensure_learned() {
        if (learned_alloc) return GLS_OK;
        const size_t n = (size_t)cap_w * cap_h;
        GLS_CHECK(alloc((void**)&cnn_in, n * 16));
        GLS_CHECK(alloc((void**)&cnn_head, n * 16));
        GLS_CHECK(alloc((void**)&strength, n * 4));
        learned_alloc = true;
        return GLS_OK;
    }

    void tap(int stage, const ImgRef& src, int channels) {
        if (stage < 0 || stage >= 5 || !tap_set[stage]) return;
        const gls_image_desc& d = taps[stage];
        if (d.width != src.w || d.height != src.h) return;
        tap_copy_kernel<<<dim3((src.w + 31) / 32, (src.h + 7) / 8), dim3(32, 8), 0, ctx->stream>>>(
            src.ptr, src.half, channels, src.w, src.h, src.pitch, (float*)d.ptr, d.stride_bytes / (4 * channels));
        ctx->launches++;
    }

    gls_status denoise_level(int algo, bool coarsest, const ImgRef& in, const ImgRef& out, int level,
                             const gls_denoise_params& dp) {
        NlfArg a;
        a.dev = nlf_dev + 8 * (1 + level);
        const float lm = dp.luma * dp.luma, cm = dp.chroma * dp.chroma;
        const float mul[6] = {lm, cm, cm, lm, cm, cm};
        for (int k = 0; k < 6; k++) {
            a.host[k] = 0;
            a.mul[k] = mul[k];
        }
        if (algo == GLS_DENOISE_BILATERAL || (algo == GLS_DENOISE_GUIDED_FAST && coarsest)) {
            launch_bilateral(ctx, in, out, a, dp.chromaBoost, dp.gradientBoost);
        } else if (algo == GLS_DENOISE_GUIDED_FAST) {
            launch_guided_fast(ctx, in, out, a);
        } else {
            const size_t need = guided_filter_scratch_bytes(w, h);
            if (gf_scratch_bytes < need) {
                GLS_CHECK(alloc(&gf_scratch, need));
                gf_scratch_bytes = need;
            }
            launch_guided_filter(ctx, in, out, 5, a, gf_scratch);
        }
        return GLS_OK;
    }

    // ---- per-stage timing ----
    bool profiling = false;
    cudaEvent_t ev_pool[64];
    int ev_used = 0;
    const char* ev_name[64];
    std::vector<std::pair<std::string, std::pair<double, long>>> prof;

    void mark(const char* name) {
        if (!profiling || ev_used >= 64) return;
        cudaEventRecord(ev_pool[ev_used], ctx->stream);
        ev_name[ev_used++] = name;
    }

    void collect() {
        if (!profiling || ev_used < 2) {
            ev_used = 0;
            return;
        }
        cudaEventSynchronize(ev_pool[ev_used - 1]);
        for (int i = 1; i < ev_used; i++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev_pool[i - 1], ev_pool[i]);
            bool found = false;
            for (auto& e : prof)
                if (e.first == ev_name[i]) {
                    e.second.first += ms;
                    e.second.second += 1;
                    found = true;
                }
            if (!found) prof.push_back({ev_name[i], {ms, 1L}});
        }
        ev_used = 0;
    }

    int mode = 0;  // 0 fused kernels, 1 one kernel per reference stage

    gls_status run(const uint16_t* raw, int rpitch, gls_demosaic_params* p, void* out, bool out_float, int opitch) {
        // rotate_180 turns the image at interpolateRedBlue; the later stages read the turned
        // image, so a rotated frame takes the single-stage schedule
        if (mode == 0 && p->denoise_algorithm != GLS_DENOISE_GUIDED_PRECISE && !p->rotate_180)
            return run_fused(raw, rpitch, p, out, out_float, opitch);
        if (cnn)
            return set_error(ctx, GLS_ERR_UNSUPPORTED,
                             "the learned stage runs in the fused schedule only (not with GuidedPrecise or rotate_180)");
        return run_staged(raw, rpitch, p, out, out_float, opitch);
    }

    float* tap_ptr(int stage) { return tap_set[stage] ? (float*)taps[stage].ptr : nullptr; }

    // cnn_input_only: stop after interpolateRedBlue, writing the learned stage's input there
    gls_status run_fused(const uint16_t* raw, int rpitch, gls_demosaic_params* p, void* out, bool out_float,
                         int opitch, float* cnn_input_only = nullptr) {
        const int Lv = L;
        const int bayer = p->bayer_pattern;
        const bool high_noise = p->noise_level > 0.6f;
        ev_used = 0;
        mark("start");
        float sm[4];
        for (int c = 0; c < 4; c++) sm[bayer_dy(bayer, c) * 2 + bayer_dx(bayer, c)] = p->scale_mul[c];
        const float black = p->black_level / 0xffff;

        // raw noise model, fitted on the fly from the uint16 frame
        RawPass1Args ra{};
        ra.raw = raw;
        ra.w = w;
        ra.h = h;
        ra.pitch = rpitch;
        ra.bayer = bayer;
        memcpy(ra.sm, sm, sizeof(sm));
        ra.black = black;
        ra.stats_half = p->storage == GLS_STORAGE_F16_STATS;
        GLS_CHECK(fused_raw_fit(ctx, ra, half, nlf_scratch_at(nlf_scratch), nlf_dev));
        mark("rawNoiseStatistics+fit");
        const float* rawB = nlf_dev + 4;

        DemosaicArgs da{};
        da.w = w;
        da.h = h;
        da.bayer = bayer;
        memcpy(da.sm, sm, sizeof(sm));
        da.black = black;
        da.rawB_dev = rawB;
        float cam_to_ycbcr[9];
        host_cam_ycbcr(p->rgb_cam, cam_to_ycbcr);
        memcpy(da.cam_ycbcr.m, cam_to_ycbcr, sizeof(cam_to_ycbcr));
        da.va0 = p->pyramid_nlf[0][0];
        da.vb0 = p->pyramid_nlf[0][3];
        da.level0 = (half4*)level0.ptr;
        da.l0_pitch = level0.pitch;
        da.tap_scaled = tap_ptr(0);
        da.tap_green = tap_ptr(1);
        da.tap_pitch = w;
        da.rawA_dev = nlf_dev;
        GLS_CHECK(ensure_split_green());
        da.green = split_green.ptr;
        da.green_pitch = split_green.pitch;
        const bool learned = cnn != nullptr && !cnn_input_only;
        if (learned) GLS_CHECK(ensure_learned());
        da.cnn_in = cnn_input_only ? cnn_input_only : (learned ? cnn_in : nullptr);
        if (high_noise) {
            // raw-domain despeckle and bilateral on the quarter-resolution CFA planes
            GLS_CHECK(ensure_high_noise());
            launch_scale_raw(ctx, raw, w, h, rpitch, scaled, bayer, p->scale_mul, black);
            launch_bayer_to_rgba(ctx, scaled, hnA, bayer);
            launch_despeckle_rgba(ctx, hnA, hnB);
            launch_denoise_rgba(ctx, hnB, hnA, p->raw_nlf, rawB);
            launch_rgba_to_bayer(ctx, hnA, scaled, bayer);
            mark("rawDenoise");
            da.in = scaled.ptr;
            da.in_pitch = scaled.pitch;
            GLS_CHECK(fused_demosaic(ctx, da, false, half));
        } else {
            da.in = raw;
            da.in_pitch = rpitch;
            GLS_CHECK(fused_demosaic(ctx, da, true, half));
        }
        mark("demosaic");
        if (cnn_input_only) {
            collect();
            return check_launch(ctx, "learned stage input");
        }
        if (learned) {
            GLS_CHECK(gls_cnn_forward(cnn, cnn_in, w, h, 1, cnn_head));
            mark("learned stage");
            PostCnnArgs pa{};
            pa.cnn_in = cnn_in;
            pa.head = cnn_head;
            pa.w = w;
            pa.h = h;
            pa.cam_ycbcr = da.cam_ycbcr;
            pa.va0 = da.va0;
            pa.vb0 = da.vb0;
            pa.level0 = (half4*)level0.ptr;
            pa.l0_pitch = level0.pitch;
            pa.strength = strength;
            GLS_CHECK(fused_post_cnn(ctx, pa, half));
            mark("residual+highlights+despeckle");
        }
        tap(2, level0, 4);

        // pyramid: level 0's noise model and level 1 (one launch), then the noise models of
        // levels 1 .. Lv-1 and their downsampled levels (one launch)
        {
            LevelPass1Args la{};
            la.in = level0.ptr;
            la.w = level0.w;
            la.h = level0.h;
            la.pitch = level0.pitch;
            la.out = pyr[0].ptr;
            la.ow = pyr[0].w;
            la.oh = pyr[0].h;
            la.opitch = pyr[0].pitch;
            la.stats_half = p->storage == GLS_STORAGE_F16_STATS;
            GLS_CHECK(fused_level_fit(ctx, la, true, half, nlf_scratch_at(nlf_scratch), nlf_dev + 8));
            mark("noiseStatistics+downsample L0");
        }
        if (overlapped) {
            // a lane of a burst: the other lanes' kernels fill the small levels' idle SMs, so
            // the levels keep one launch each (measured faster there than the one-launch form,
            // whose blocks hold every SM for the whole pyramid)
            for (int i = 1; i < Lv; i++) {
                const ImgRef& src = pyr[i - 1];
                LevelPass1Args la{};
                la.in = src.ptr;
                la.w = src.w;
                la.h = src.h;
                la.pitch = src.pitch;
                if (i < Lv - 1) {
                    la.out = pyr[i].ptr;
                    la.ow = pyr[i].w;
                    la.oh = pyr[i].h;
                    la.opitch = pyr[i].pitch;
                }
                la.stats_half = p->storage == GLS_STORAGE_F16_STATS;
                GLS_CHECK(fused_level_fit(ctx, la, half, half, nlf_scratch_at(nlf_scratch), nlf_dev + 8 * (1 + i)));
            }
            mark("noiseStatistics+downsample L1+");
        } else {
            PyramidArgs pa{};
            pa.nlev = Lv - 1;
            pa.stats_half = p->storage == GLS_STORAGE_F16_STATS;
            pa.ctl = (PyrCtl*)pyr_state;
            unsigned* marks = (unsigned*)((char*)pyr_state + sizeof(PyrCtl));
            int first = 0;
            for (int q = 0; q < pa.nlev; q++) {
                PyrLevel& lv = pa.lv[q];
                const ImgRef& src = pyr[q];
                lv.in = src.ptr;
                lv.w = src.w;
                lv.h = src.h;
                lv.pitch = src.pitch;
                if (q + 1 < pa.nlev) {
                    lv.out = pyr[q + 1].ptr;
                    lv.ow = pyr[q + 1].w;
                    lv.oh = pyr[q + 1].h;
                    lv.opitch = pyr[q + 1].pitch;
                }
                lv.tiles_x = (src.w + 31) / 32;
                lv.first = first;
                lv.count = lv.tiles_x * ((src.h + 31) / 32);
                first += lv.count;
                lv.nlf = nlf_scratch_at((char*)nlf_scratch + kNlfScratchBytes * (1 + q));
                lv.nlf_out = nlf_dev + 8 * (2 + q);
                lv.done = marks;
                marks += (size_t)(((cap_w >> (q + 1)) + 31) / 32) * (((cap_h >> (q + 1)) + 31) / 32);
            }
            pa.items = first;
            GLS_CHECK(fused_pyramid_stats(ctx, pa, half));
            mark("noiseStatistics+downsample L1+");
        }

        // denoise coarse to fine
        const int algo = p->denoise_algorithm;
        for (int i = Lv - 1; i >= 1; i--) {
            const gls_denoise_params& dp = p->denoise[i];
            DenoiseArgs a{};
            const ImgRef& in = pyr[i - 1];
            a.in = in.ptr;
            a.w = in.w;
            a.h = in.h;
            a.pitch = in.pitch;
            a.out = den[i].ptr;
            a.opitch = den[i].pitch;
            const bool reasm = i < Lv - 1;
            if (reasm) {
                a.coarse_img = pyr[i].ptr;
                a.coarse_den = den[i + 1].ptr;
                a.cw = pyr[i].w;
                a.ch = pyr[i].h;
                a.cpitch = pyr[i].pitch;
            }
            a.nlf_dev = nlf_dev + 8 * (1 + i);
            const float lm = dp.luma * dp.luma, cm = dp.chroma * dp.chroma;
            const float mul[6] = {lm, cm, cm, lm, cm, cm};
            memcpy(a.mul, mul, sizeof(mul));
            a.chroma_boost = dp.chromaBoost;
            a.gradient_boost = dp.gradientBoost;
            a.sharpening = dp.sharpening;
            const int level_algo = (algo == GLS_DENOISE_GUIDED_FAST && i < Lv - 1) ? 1 : 0;
            GLS_CHECK(fused_denoise(ctx, a, in.half, half, level_algo, reasm));
            mark("denoise+reassemble L1+");
        }

        // level 0 + local tone mapping + output
        FinalArgs f{};
        f.level0 = (const half4*)level0.ptr;
        f.w = w;
        f.h = h;
        f.l0_pitch = level0.pitch;
        f.pyr0 = pyr[0].ptr;
        f.den1 = den[1].ptr;
        f.cw = pyr[0].w;
        f.ch = pyr[0].h;
        f.cpitch = pyr[0].pitch;
        f.guide = den[3].ptr;
        f.gw = den[3].w;
        f.gh = den[3].h;
        f.gpitch = den[3].pitch;
        f.nlf_dev = nlf_dev + 8;
        {
            const gls_denoise_params& dp = p->denoise[0];
            const float lm = dp.luma * dp.luma, cm = dp.chroma * dp.chroma;
            const float mul[6] = {lm, cm, cm, lm, cm, cm};
            memcpy(f.mul, mul, sizeof(mul));
            f.chroma_boost = dp.chromaBoost;
            f.gradient_boost = dp.gradientBoost;
            f.sharpening = dp.sharpening;
        }
        f.ltm = LtmParams{p->ltm.guidedFilterEps, p->ltm.shadows, p->ltm.highlights, p->ltm.detail};
        float inv[9];
        if (!host_inverse3x3(cam_to_ycbcr, inv)) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "singular cam_ycbcr");
        for (int k = 0; k < 9; k++) f.icy.m[k] = inv[k] * p->exposure_multiplier;
        memcpy(f.rgb_cam.m, p->rgb_cam, sizeof(f.rgb_cam.m));
        const gls_rgb_conversion_params& rc = p->rgb_conversion;
        f.rgb = rgb_params_init(rc.contrast, rc.saturation, rc.toneCurveSlope, rc.exposureBias, rc.blacks, rc.localToneMapping);
        f.out = out;
        f.opitch = opitch;
        f.tap_den = tap_ptr(3);
        f.tap_mask = tap_ptr(4);
        f.tap_pitch = w;
        f.strength = learned ? strength : nullptr;
        const int algo0 = (algo == GLS_DENOISE_GUIDED_FAST) ? 1 : 0;
        if (host_band.out && !out_float && out == out_dev) {
            const FinalBandFn band{&gls_raw_converter::copy_rows_cb, this};
            GLS_CHECK(fused_final(ctx, f, half, algo0, rc.localToneMapping != 0, false, kHostBands, &band));
        } else {
            GLS_CHECK(fused_final(ctx, f, half, algo0, rc.localToneMapping != 0, out_float));
        }
        mark("denoise L0+LTM+sRGB");
        collect();
        return GLS_OK;
    }

    gls_status run_staged(const uint16_t* raw, int rpitch, gls_demosaic_params* p, void* out, bool out_float,
                          int opitch) {
        GLS_CHECK(ensure_staged());
        const int Lv = L;
        const int bayer = p->bayer_pattern;
        const bool high_noise = p->noise_level > 0.6f;
        ev_used = 0;
        mark("start");

        // --- image demosaicing (raw_converter.cpp:101-131) ---
        launch_scale_raw(ctx, raw, w, h, rpitch, scaled, bayer, p->scale_mul, p->black_level / 0xffff);
        mark("scaleRawData");
        GLS_CHECK(nlf_fit_raw_scaled(ctx, scaled.ptr, half, w, h, scaled.pitch, bayer, nlf_scratch_at(nlf_scratch),
                                     nlf_dev, p->storage == GLS_STORAGE_F16_STATS));
        mark("rawNoiseStatistics+fit");
        const float* rawB = nlf_dev + 4;
        if (high_noise) {
            launch_bayer_to_rgba(ctx, scaled, hnA, bayer);
            launch_despeckle_rgba(ctx, hnA, hnB);
            launch_denoise_rgba(ctx, hnB, hnA, p->raw_nlf, rawB);
            launch_rgba_to_bayer(ctx, hnA, scaled, bayer);
            mark("rawDenoise");
        }
        tap(0, scaled, 1);
        launch_green(ctx, scaled, green, bayer, 0.0f, rawB + 1);
        mark("interpolateGreen");
        tap(1, green, 1);
        launch_red_blue(ctx, scaled, green, linA, bayer, 0.0f, rawB, p->rotate_180 != 0);
        mark("interpolateRedBlue");
        launch_highlights(ctx, linA, linA, 1.0f);
        mark("blendHighlights");

        // --- image denoising (raw_converter.cpp:133-160) ---
        float cam_to_ycbcr[9];
        host_cam_ycbcr(p->rgb_cam, cam_to_ycbcr);
        launch_transform(ctx, linA, linA, cam_to_ycbcr);
        mark("transformImage");
        launch_despeckle(ctx, linA, linB, p->pyramid_nlf[0][0], p->pyramid_nlf[0][3]);
        mark("despeckleImage");
        tap(2, linB, 4);

        // PyramidalDenoise::denoise
        for (int i = 0; i < Lv; i++) {
            const ImgRef& src = i == 0 ? linB : pyr[i - 1];
            if (i < Lv - 1) launch_downsample(ctx, src, pyr[i]);
            mark("downsampleImage");
            GLS_CHECK(nlf_fit_level(ctx, src.ptr, half, src.w, src.h, src.pitch, nlf_scratch_at(nlf_scratch),
                                    nlf_dev + 8 * (1 + i), p->storage == GLS_STORAGE_F16_STATS));
            mark(i == 0 ? "noiseStatistics+fit L0" : "noiseStatistics+fit L1+");
        }
        const int algo = p->denoise_algorithm;
        GLS_CHECK(denoise_level(algo, true, pyr[Lv - 2], den[Lv - 1], Lv - 1, p->denoise[Lv - 1]));
        mark("denoise L1+");
        for (int i = Lv - 2; i >= 0; i--) {
            const ImgRef& input = i > 0 ? pyr[i - 1] : linB;
            GLS_CHECK(denoise_level(algo, false, input, den[i], i, p->denoise[i]));
            mark(i == 0 ? "denoise L0" : "denoise L1+");
            NlfArg a;
            a.dev = nlf_dev + 8 * (1 + i);
            const float lm = p->denoise[i].luma * p->denoise[i].luma;
            const float cm = p->denoise[i].chroma * p->denoise[i].chroma;
            const float mul[6] = {lm, cm, cm, lm, cm, cm};
            for (int k = 0; k < 6; k++) {
                a.host[k] = 0;
                a.mul[k] = mul[k];
            }
            launch_reassemble(ctx, den[i], pyr[i], den[i + 1], den[i], p->denoise[i].sharpening, a);
            mark(i == 0 ? "reassemble L0" : "reassemble L1+");
        }
        const ImgRef& denoised = den[0];
        tap(3, denoised, 4);

        // --- local tone mapping and output (raw_converter.cpp:162-174) ---
        float inv[9], icy_e[9];
        if (!host_inverse3x3(cam_to_ycbcr, inv)) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "singular cam_ycbcr");
        for (int k = 0; k < 9; k++) icy_e[k] = inv[k] * p->exposure_multiplier;
        const bool ltm = p->rgb_conversion.localToneMapping != 0;
        if (ltm) {
            LtmParams lp{p->ltm.guidedFilterEps, p->ltm.shadows, p->ltm.highlights, p->ltm.detail};
            launch_ltm(ctx, denoised, den[3], mask, lp, icy_e);
            mark("localToneMappingMask");
            tap(4, mask, 1);
        }
        launch_transform(ctx, denoised, denoised, icy_e);
        mark("transformImage");
        const gls_rgb_conversion_params& rc = p->rgb_conversion;
        const RgbParams rp = rgb_params_init(rc.contrast, rc.saturation, rc.toneCurveSlope, rc.exposureBias, rc.blacks, rc.localToneMapping);
        launch_srgb(ctx, denoised, ltm ? &mask : nullptr, out, out_float, opitch, p->rgb_cam, rp);
        mark("convertTosRGB");
        collect();
        return check_launch(ctx, "RawConverter::demosaicImage");
    }

    // device staging of the host-buffer entry points: raw frame, RGBA8 output and its RGB8 copy
    gls_status ensure_staging(int fw, int fh) {
        const size_t rb = (size_t)fw * fh * 2, ob = (size_t)fw * fh * 4 + (size_t)fw * fh * 3;
        if (raw_dev_bytes < rb) {
            if (raw_dev) cudaFree(raw_dev);
            raw_dev = nullptr;
            raw_dev_bytes = 0;
            GLS_CHECK(check_cuda(ctx, cudaMalloc(&raw_dev, rb), "cudaMalloc(raw)"));
            raw_dev_bytes = rb;
        }
        if (out_dev_bytes < ob) {
            if (out_dev) cudaFree(out_dev);
            out_dev = nullptr;
            out_dev_bytes = 0;
            GLS_CHECK(check_cuda(ctx, cudaMalloc(&out_dev, ob), "cudaMalloc(output)"));
            out_dev_bytes = ob;
        }
        return GLS_OK;
    }

    // host raw in, host RGBA8/RGB8 out, all on this converter's stream (no synchronisation)
    // after / copied: a burst's uploads go one at a time (each waits for the previous frame's
    // copy), so the first frame's kernels start after one copy rather than after all of them
    gls_status upload_order(cudaEvent_t after) {
        if (!after) return GLS_OK;
        return check_cuda(ctx, cudaStreamWaitEvent(ctx->stream, after, 0), "cudaStreamWaitEvent(upload)");
    }
    gls_status upload_done(cudaEvent_t copied) {
        if (!copied) return GLS_OK;
        return check_cuda(ctx, cudaEventRecord(copied, ctx->stream), "cudaEventRecord(upload)");
    }

    gls_status run_host(const uint16_t* raw, int fw, int fh, int stride, gls_demosaic_params* p, uint8_t* out,
                        int out_channels, cudaEvent_t after = nullptr, cudaEvent_t copied = nullptr) {
        GLS_CHECK(ensure_staging(fw, fh));
        GLS_CHECK(upload_order(after));
        GLS_CHECK(check_cuda(ctx, cudaMemcpy2DAsync(raw_dev, (size_t)fw * 2, raw, (size_t)stride * 2, (size_t)fw * 2,
                                                    fh, cudaMemcpyHostToDevice, ctx->stream), "copy raw frame"));
        GLS_CHECK(upload_done(copied));
        return finish_host(fw, fh, p, out, out_channels);
    }

    // packed host raw in (the frame's samples as one MSB-first bit stream, as a DNG strip of
    // 10/12/14-bit samples stores them): the packed bytes cross to the device and are
    // unpacked there into the staging frame (unpack12BitsInto16Bits and
    // unpack14BitsInto16Bits, src/gls_image_tiff.cpp:53-87)
    gls_status run_packed_host(const uint8_t* packed, size_t n_bytes, int bits, int fw, int fh,
                               gls_demosaic_params* p, uint8_t* out, int out_channels, cudaEvent_t after = nullptr,
                               cudaEvent_t copied = nullptr) {
        GLS_CHECK(ensure_staging(fw, fh));
        if (packed_dev_bytes < n_bytes) {
            if (packed_dev) cudaFree(packed_dev);
            packed_dev = nullptr;
            packed_dev_bytes = 0;
            GLS_CHECK(check_cuda(ctx, cudaMalloc(&packed_dev, n_bytes), "cudaMalloc(packed raw)"));
            packed_dev_bytes = n_bytes;
        }
        GLS_CHECK(upload_order(after));
        GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(packed_dev, packed, n_bytes, cudaMemcpyHostToDevice, ctx->stream),
                             "copy packed raw frame"));
        GLS_CHECK(upload_done(copied));
        launch_unpack(ctx, packed_dev, n_bytes, bits, raw_dev, (size_t)fw * fh);
        return finish_host(fw, fh, p, out, out_channels);
    }

    // The host product of the final stage's rows [y0, y1): packed to RGB8 when asked and copied
    // back on the converter's copy stream, which waits only for the rows' own launch, so the
    // copy runs while the next band's kernel does.
    gls_status ensure_copy_stream() {
        if (copy_stream) return GLS_OK;
        GLS_CHECK(check_cuda(ctx, cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate(copy)"));
        for (int k = 0; k <= kHostBands; k++)
            GLS_CHECK(check_cuda(ctx, cudaEventCreateWithFlags(&band_ev[k], cudaEventDisableTiming), "cudaEventCreate(band)"));
        return GLS_OK;
    }
    gls_status copy_rows(int y0, int y1, cudaStream_t st) {
        const int fw = host_band.w, ch = host_band.channels;
        const uint8_t* src = out_dev + (size_t)y0 * fw * 4;
        if (ch == 3) {
            uint8_t* rgb = out_dev + (size_t)fw * host_band.h * 4;
            rgba8_to_rgb8_kernel<<<dim3((fw + 31) / 32, (y1 - y0 + 7) / 8), dim3(32, 8), 0, st>>>(
                (const uchar4*)out_dev, fw, y0, y1, rgb);
            ctx->launches++;
            src = rgb + (size_t)y0 * fw * 3;
        }
        return check_cuda(ctx, cudaMemcpyAsync(host_band.out + (size_t)y0 * fw * ch, src, (size_t)(y1 - y0) * fw * ch,
                                               cudaMemcpyDeviceToHost, st), "copy output rows");
    }
    static gls_status copy_rows_cb(void* self, int y0, int y1) {
        gls_raw_converter* c = static_cast<gls_raw_converter*>(self);
        const int k = c->host_band.bands++;
        if (k >= kHostBands) return set_error(c->ctx, GLS_ERR_INVALID_ARGUMENT, "more output bands than events");
        GLS_CHECK(check_cuda(c->ctx, cudaEventRecord(c->band_ev[k], c->ctx->stream), "cudaEventRecord(band)"));
        GLS_CHECK(check_cuda(c->ctx, cudaStreamWaitEvent(c->copy_stream, c->band_ev[k], 0), "cudaStreamWaitEvent(band)"));
        return c->copy_rows(y0, y1, c->copy_stream);
    }

    // the staged raw frame through the pipeline, RGBA8 (or RGB8) back to the host: the fused
    // schedule runs its final stage in row bands whose copies overlap the following bands'
    // kernels (the converter's stream then waits for the last copy); the other schedules copy
    // the whole frame at the end
    gls_status finish_host(int fw, int fh, gls_demosaic_params* p, uint8_t* out, int out_channels) {
        GLS_CHECK(ensure(fw, fh, p->pyramid_levels, p->storage != GLS_STORAGE_F32));
        GLS_CHECK(ensure_copy_stream());
        host_band = HostBand{out, out_channels, fw, fh, 0};
        const gls_status s = run(raw_dev, fw, p, out_dev, false, fw);
        const int bands = host_band.bands;
        if (bands > 0) {
            GLS_CHECK(check_cuda(ctx, cudaEventRecord(band_ev[kHostBands], copy_stream), "cudaEventRecord(copied)"));
            GLS_CHECK(check_cuda(ctx, cudaStreamWaitEvent(ctx->stream, band_ev[kHostBands], 0), "cudaStreamWaitEvent(copied)"));
        }
        GLS_CHECK(s);
        if (bands > 0) {
            host_band = HostBand{};
            return GLS_OK;
        }
        const gls_status c = copy_rows(0, fh, ctx->stream);
        host_band = HostBand{};
        return c;
    }

    gls_status fetch_noise_model(gls_demosaic_params* p) {
        const size_t n = (1 + GLS_MAX_LEVELS) * 8;
        GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(nlf_host, nlf_dev, n * sizeof(float), cudaMemcpyDeviceToHost,
                                                  ctx->stream), "copy noise model"));
        GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize"));
        for (int c = 0; c < 4; c++) p->raw_nlf[c] = nlf_host[4 + c];
        for (int i = 0; i < L; i++)
            for (int k = 0; k < 6; k++) p->pyramid_nlf[i][k] = nlf_host[8 * (1 + i) + k];
        return GLS_OK;
    }
};

static gls_status validate_params(gls_ctx* ctx, const gls_demosaic_params* p, int w, int h) {
    if (!p) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "params is null");
    if (p->bayer_pattern < 0 || p->bayer_pattern > 3)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "unknown bayer pattern %d", p->bayer_pattern);
    if (p->pyramid_levels < 4 || p->pyramid_levels > GLS_MAX_LEVELS)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "pyramid_levels must be in [4, %d]", GLS_MAX_LEVELS);
    if (p->storage != GLS_STORAGE_F32 && p->storage != GLS_STORAGE_F16 && p->storage != GLS_STORAGE_F16_STATS)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "unknown storage %d", p->storage);
    if (p->denoise_algorithm < 0 || p->denoise_algorithm > 2)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "unknown denoise algorithm %d", p->denoise_algorithm);
    if (w <= 0 || h <= 0 || (w & 1) || (h & 1))
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "raw frames must have positive, even width and height");
    if ((w >> (p->pyramid_levels - 1)) < 1 || (h >> (p->pyramid_levels - 1)) < 1)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "frame too small for %d pyramid levels", p->pyramid_levels);
    return GLS_OK;
}

extern "C" {

gls_status gls_raw_converter_create(gls_ctx* ctx, gls_raw_converter** out) {
    if (!ctx || !out) return GLS_ERR_INVALID_ARGUMENT;
    gls_raw_converter* c = new gls_raw_converter();
    c->ctx = ctx;
    if (cudaMallocHost(&c->nlf_host, (1 + GLS_MAX_LEVELS) * 8 * sizeof(float)) != cudaSuccess) {
        delete c;
        return set_error(ctx, GLS_ERR_OUT_OF_MEMORY, "cudaMallocHost");
    }
    *out = c;
    return GLS_OK;
}

gls_status gls_raw_converter_destroy(gls_raw_converter* c) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(c->ctx->stream);
    if (c->nlf_host) cudaFreeHost(c->nlf_host);
    if (c->raw_dev) cudaFree(c->raw_dev);
    if (c->out_dev) cudaFree(c->out_dev);
    if (c->packed_dev) cudaFree(c->packed_dev);
    if (c->cnn) gls_cnn_destroy(c->cnn);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    for (cudaEvent_t e : c->band_ev)
        if (e) cudaEventDestroy(e);
    delete c;
    return GLS_OK;
}

gls_status gls_raw_converter_set_cnn(gls_raw_converter* c, gls_cnn* src) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    if (c->cnn) {
        cudaStreamSynchronize(c->ctx->stream);
        gls_cnn_destroy(c->cnn);
        c->cnn = nullptr;
    }
    if (!src) return GLS_OK;
    const int n = gls_cnn_param_count();
    std::vector<float> prm(n);
    gls_status s = gls_cnn_get_params(src, prm.data(), n);
    if (s != GLS_OK) return set_error(c->ctx, s, "learned stage: reading the network's parameters");
    GLS_CHECK(gls_cnn_create(c->ctx, &c->cnn));
    s = gls_cnn_set_params(c->cnn, prm.data(), n);
    if (s == GLS_OK) s = gls_cnn_set_backend(c->cnn, gls_cnn_get_backend(src));
    if (s != GLS_OK) {
        gls_cnn_destroy(c->cnn);
        c->cnn = nullptr;
    }
    return s;
}

gls_status gls_raw_converter_cnn_input(gls_raw_converter* c, const gls_image_desc* raw,
                                       const gls_demosaic_params* params, const gls_image_desc* out) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = c->ctx;
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R16_UNORM));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32));
    if (out->width != raw->width || out->height != raw->height || out->stride_bytes != out->width * 16)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "learned stage input: dense RGBA_F32 of the raw frame's size");
    GLS_CHECK(validate_params(ctx, params, raw->width, raw->height));
    GLS_CHECK(c->ensure(raw->width, raw->height, params->pyramid_levels, params->storage != GLS_STORAGE_F32));
    gls_demosaic_params p = *params;
    return c->run_fused((const uint16_t*)raw->ptr, pitch_elems(raw), &p, nullptr, false, 0, (float*)out->ptr);
}

gls_status gls_raw_converter_set_mode(gls_raw_converter* c, int mode) {
    if (!c || (mode != 0 && mode != 1)) return GLS_ERR_INVALID_ARGUMENT;
    c->mode = mode;
    return GLS_OK;
}

gls_status gls_raw_converter_profile(gls_raw_converter* c, int enable) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    if (enable && !c->profiling) {
        for (int i = 0; i < 64; i++)
            GLS_CHECK(check_cuda(c->ctx, cudaEventCreate(&c->ev_pool[i]), "cudaEventCreate"));
        c->prof.clear();
        c->profiling = true;
    } else if (!enable && c->profiling) {
        cudaStreamSynchronize(c->ctx->stream);
        for (int i = 0; i < 64; i++) cudaEventDestroy(c->ev_pool[i]);
        c->profiling = false;
    }
    return GLS_OK;
}

gls_status gls_raw_converter_profile_report(gls_raw_converter* c, char* buf, size_t len) {
    if (!c || !buf || len == 0) return GLS_ERR_INVALID_ARGUMENT;
    std::string s = "{";
    for (size_t i = 0; i < c->prof.size(); i++) {
        char item[160];
        snprintf(item, sizeof(item), "%s\"%s\": [%.6f, %ld]", i ? ", " : "", c->prof[i].first.c_str(),
                 c->prof[i].second.first, c->prof[i].second.second);
        s += item;
    }
    s += "}";
    if (s.size() + 1 > len) return GLS_ERR_INVALID_SIZE;
    memcpy(buf, s.c_str(), s.size() + 1);
    return GLS_OK;
}

gls_status gls_raw_converter_set_tap(gls_raw_converter* c, int stage, const gls_image_desc* dst) {
    if (!c || stage < 0 || stage >= 5) return GLS_ERR_INVALID_ARGUMENT;
    if (!dst) {
        c->tap_set[stage] = false;
        return GLS_OK;
    }
    const int want = (stage == 0 || stage == 1 || stage == 4) ? GLS_R_F32 : GLS_RGBA_F32;
    GLS_CHECK(check_desc(c->ctx, dst, "tap", want));
    c->taps[stage] = *dst;
    c->tap_set[stage] = true;
    return GLS_OK;
}

gls_status gls_raw_converter_demosaic(gls_raw_converter* c, const gls_image_desc* raw, gls_demosaic_params* p,
                                      const gls_image_desc* out, int defer) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = c->ctx;
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R16_UNORM));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA8_UNORM, GLS_RGBA_F32));
    if (out->width != raw->width || out->height != raw->height)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "output size differs from the raw frame");
    GLS_CHECK(validate_params(ctx, p, raw->width, raw->height));
    GLS_CHECK(c->ensure(raw->width, raw->height, p->pyramid_levels, p->storage != GLS_STORAGE_F32));
    GLS_CHECK(c->run((const uint16_t*)raw->ptr, pitch_elems(raw), p, out->ptr, out->format == GLS_RGBA_F32,
                     pitch_elems(out)));
    if (!defer) GLS_CHECK(c->fetch_noise_model(p));
    return GLS_OK;
}

gls_status gls_raw_converter_noise_model(gls_raw_converter* c, gls_demosaic_params* p) {
    if (!c || !p) return GLS_ERR_INVALID_ARGUMENT;
    if (c->L == 0) return set_error(c->ctx, GLS_ERR_INVALID_ARGUMENT, "no frame processed yet");
    return c->fetch_noise_model(p);
}

gls_status gls_raw_converter_status(gls_raw_converter* c) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    if (!c->nlf_scratch) return GLS_OK;
    gls_ctx* ctx = c->ctx;
    GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize"));
    unsigned any = 0;
    for (int r = 0; r <= GLS_MAX_LEVELS; r++) {
        unsigned* e = (unsigned*)((char*)c->nlf_scratch + kNlfScratchBytes * r + kNlfErrOff);
        unsigned v = 0;
        GLS_CHECK(check_cuda(ctx, cudaMemcpy(&v, e, sizeof(v), cudaMemcpyDeviceToHost), "read error word"));
        if (v) {
            any |= v;
            GLS_CHECK(check_cuda(ctx, cudaMemset(e, 0, sizeof(v)), "clear error word"));
        }
    }
    if (any)
        return set_error(ctx, GLS_ERR_TIMEOUT, "a bounded wait of a statistics kernel ran out (%s)",
                         (any & 1u) ? ((any & 2u) ? "tile copy and tile mark" : "tile copy") : "tile mark");
    return GLS_OK;
}

gls_status gls_raw_converter_wait_probe(gls_raw_converter* c, unsigned polls) {
    if (!c || polls == 0 || polls > (1u << 22)) return GLS_ERR_INVALID_ARGUMENT;
    if (!c->nlf_scratch) return set_error(c->ctx, GLS_ERR_INVALID_ARGUMENT, "no frame processed yet");
    return fused_wait_probe(c->ctx, nlf_scratch_at(c->nlf_scratch), polls);
}

gls_status gls_raw_converter_demosaic_host(gls_raw_converter* c, const uint16_t* raw, int w, int h, int stride,
                                           gls_demosaic_params* p, uint8_t* out, int out_channels) {
    if (!c || !raw || !out) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = c->ctx;
    if (out_channels != 3 && out_channels != 4)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "out_channels must be 3 or 4");
    if (stride < w) return set_error(ctx, GLS_ERR_INVALID_SIZE, "raw stride smaller than width");
    GLS_CHECK(validate_params(ctx, p, w, h));
    GLS_CHECK(c->run_host(raw, w, h, stride, p, out, out_channels));
    return c->fetch_noise_model(p);
}

static gls_status check_packed(gls_ctx* ctx, const void* packed, size_t n_bytes, int bits, int w, int h) {
    if (!packed) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "packed raw is null");
    if (bits != 10 && bits != 12 && bits != 14 && bits != 16)
        return set_error(ctx, GLS_ERR_UNSUPPORTED, "unsupported bit depth %d", bits);
    if ((unsigned long long)w * h > (unsigned long long)(n_bytes * 8 / (size_t)bits))
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "packed raw holds %zu samples, the frame needs %lld",
                         n_bytes * 8 / (size_t)bits, (long long)w * h);
    return GLS_OK;
}

gls_status gls_raw_converter_demosaic_packed_host(gls_raw_converter* c, const uint8_t* packed, size_t n_bytes,
                                                  int bits, int w, int h, gls_demosaic_params* p, uint8_t* out,
                                                  int out_channels) {
    if (!c || !out) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = c->ctx;
    if (out_channels != 3 && out_channels != 4)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "out_channels must be 3 or 4");
    GLS_CHECK(validate_params(ctx, p, w, h));
    GLS_CHECK(check_packed(ctx, packed, n_bytes, bits, w, h));
    GLS_CHECK(c->run_packed_host(packed, n_bytes, bits, w, h, p, out, out_channels));
    return c->fetch_noise_model(p);
}

gls_status gls_raw_converter_fast_demosaic(gls_raw_converter* c, const gls_image_desc* raw,
                                           const gls_demosaic_params* p, const gls_image_desc* out) {
    if (!c) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = c->ctx;
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R16_UNORM));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA8_UNORM, GLS_RGBA_F32));
    if (!p) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "params is null");
    if ((raw->width & 1) || (raw->height & 1)) return set_error(ctx, GLS_ERR_INVALID_SIZE, "odd raw frame size");
    if (out->width != raw->width / 2 || out->height != raw->height / 2)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "fastDemosaicImage output must be half size");
    if (p->bayer_pattern < 0 || p->bayer_pattern > 3) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "bayer pattern");
    const bool half = p->storage != GLS_STORAGE_F32;
    GLS_CHECK(c->ensure(raw->width, raw->height, c->L ? c->L : 4, half));
    GLS_CHECK(c->ensure_staged());
    const int w = raw->width, h = raw->height;
    launch_scale_raw(ctx, (const uint16_t*)raw->ptr, w, h, pitch_elems(raw), c->scaled, p->bayer_pattern, p->scale_mul,
                     p->black_level / 0xffff);
    ImgRef half_rgb{c->linA.ptr, w / 2, h / 2, w / 2, half};
    launch_fast_debayer(ctx, c->scaled, half_rgb, p->bayer_pattern);
    launch_highlights(ctx, half_rgb, half_rgb, 1.0f);
    const gls_rgb_conversion_params& rc = p->rgb_conversion;
    const RgbParams rp = rgb_params_init(rc.contrast, rc.saturation, rc.toneCurveSlope, rc.exposureBias, rc.blacks, 0);
    launch_srgb(ctx, half_rgb, nullptr, out->ptr, out->format == GLS_RGBA_F32, pitch_elems(out), p->rgb_cam, rp);
    return check_launch(ctx, "RawConverter::fastDemosaicImage");
}

}  // extern "C"

// =========================================================================================
// gls_raw_batch: a burst of frames spread over converters ("lanes") on their own streams.
// The work of one frame stays a serial chain (raw fit -> demosaic -> level fits -> denoise
// -> final); frames are independent, so lanes overlap one frame's latency-bound parts (the
// small pyramid levels, the regression solves) with another's full-frame kernels.
// =========================================================================================
struct gls_raw_batch {
    gls_ctx* ctx = nullptr;  // the caller's context: its stream forks and joins the lanes
    std::vector<gls_ctx*> lane_ctx;
    std::vector<cudaStream_t> lane_stream;
    std::vector<gls_raw_converter*> lane;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    std::vector<cudaEvent_t> copied;  // per lane: its latest host-to-device copy
    std::vector<int> lane_of;
};

namespace {

// Longest processing time first: frames by pixel count, largest first, each to the lane with
// the fewest pixels so far (ties: the lower frame index, the lower lane).
void plan_lanes(int n, const int* widths, const int* heights, int lanes, int* lane_of) {
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    auto px = [&](int i) { return (long long)widths[i] * heights[i]; };
    for (int i = 1; i < n; i++) {  // stable insertion sort by decreasing pixel count
        const int v = order[i];
        int j = i - 1;
        while (j >= 0 && px(order[j]) < px(v)) {
            order[j + 1] = order[j];
            j--;
        }
        order[j + 1] = v;
    }
    std::vector<long long> load(lanes, 0);
    for (int k = 0; k < n; k++) {
        const int i = order[k];
        int best = 0;
        for (int l = 1; l < lanes; l++)
            if (load[l] < load[best]) best = l;
        lane_of[i] = best;
        load[best] += px(i);
    }
}

gls_status batch_error(gls_raw_batch* b, int l, gls_status s) {
    if (s != GLS_OK && l >= 0) set_error(b->ctx, s, "lane %d: %s", l, b->lane_ctx[l]->last_error.c_str());
    return s;
}

// fork: every lane waits for the work already on the caller's stream
gls_status batch_fork(gls_raw_batch* b) {
    GLS_CHECK(check_cuda(b->ctx, cudaEventRecord(b->fork, b->ctx->stream), "cudaEventRecord(fork)"));
    for (size_t l = 0; l < b->lane.size(); l++)
        GLS_CHECK(check_cuda(b->ctx, cudaStreamWaitEvent(b->lane_stream[l], b->fork, 0), "cudaStreamWaitEvent(fork)"));
    return GLS_OK;
}

// join: the caller's stream waits for every lane; the lanes' launches count on the context
gls_status batch_join(gls_raw_batch* b, const std::vector<uint64_t>& launches0) {
    for (size_t l = 0; l < b->lane.size(); l++) {
        GLS_CHECK(check_cuda(b->ctx, cudaEventRecord(b->join[l], b->lane_stream[l]), "cudaEventRecord(join)"));
        GLS_CHECK(check_cuda(b->ctx, cudaStreamWaitEvent(b->ctx->stream, b->join[l], 0), "cudaStreamWaitEvent(join)"));
        b->ctx->launches += b->lane_ctx[l]->launches - launches0[l];
    }
    return GLS_OK;
}

std::vector<uint64_t> lane_launches(gls_raw_batch* b) {
    std::vector<uint64_t> v;
    for (auto* c : b->lane_ctx) v.push_back(c->launches);
    return v;
}

}  // namespace

extern "C" {

gls_status gls_raw_batch_set_cnn(gls_raw_batch* b, gls_cnn* cnn) {
    if (!b) return GLS_ERR_INVALID_ARGUMENT;
    for (size_t l = 0; l < b->lane.size(); l++) {
        const gls_status s = gls_raw_converter_set_cnn(b->lane[l], cnn);
        if (s != GLS_OK) return batch_error(b, (int)l, s);
    }
    return GLS_OK;
}

gls_status gls_raw_batch_plan(int n, const int* widths, const int* heights, int lanes, int* lane_of) {
    if (n < 0 || lanes < 1 || (n > 0 && (!widths || !heights || !lane_of))) return GLS_ERR_INVALID_ARGUMENT;
    plan_lanes(n, widths, heights, lanes, lane_of);
    return GLS_OK;
}

gls_status gls_raw_batch_destroy(gls_raw_batch* b) {
    if (!b) return GLS_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(b->ctx->stream);
    for (size_t l = 0; l < b->lane.size(); l++) {
        if (b->lane[l]) gls_raw_converter_destroy(b->lane[l]);
        if (b->lane_ctx[l]) gls_ctx_destroy(b->lane_ctx[l]);
        if (b->lane_stream[l]) cudaStreamDestroy(b->lane_stream[l]);
        if (b->join[l]) cudaEventDestroy(b->join[l]);
        if (b->copied[l]) cudaEventDestroy(b->copied[l]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    delete b;
    return GLS_OK;
}

gls_status gls_raw_batch_create(gls_ctx* ctx, int lanes, gls_raw_batch** out) {
    if (!ctx || !out) return GLS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (lanes < 1 || lanes > 16) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "lanes must be in [1, 16]");
    gls_raw_batch* b = new gls_raw_batch();
    b->ctx = ctx;
    b->lane_ctx.assign(lanes, nullptr);
    b->lane_stream.assign(lanes, nullptr);
    b->lane.assign(lanes, nullptr);
    b->join.assign(lanes, nullptr);
    b->copied.assign(lanes, nullptr);
    gls_status s = check_cuda(ctx, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate");
    for (int l = 0; l < lanes && s == GLS_OK; l++) {
        s = gls_ctx_create(ctx->device, &b->lane_ctx[l]);
        if (s != GLS_OK) {
            set_error(ctx, s, "lane %d: context", l);
            break;
        }
        s = check_cuda(ctx, cudaStreamCreateWithFlags(&b->lane_stream[l], cudaStreamNonBlocking), "cudaStreamCreate");
        if (s != GLS_OK) break;
        b->lane_ctx[l]->stream = b->lane_stream[l];
        s = check_cuda(ctx, cudaEventCreateWithFlags(&b->join[l], cudaEventDisableTiming), "cudaEventCreate");
        if (s != GLS_OK) break;
        s = check_cuda(ctx, cudaEventCreateWithFlags(&b->copied[l], cudaEventDisableTiming), "cudaEventCreate");
        if (s != GLS_OK) break;
        s = gls_raw_converter_create(b->lane_ctx[l], &b->lane[l]);
        if (s != GLS_OK) batch_error(b, l, s);
        else b->lane[l]->overlapped = lanes > 1;
    }
    if (s != GLS_OK) {
        gls_raw_batch_destroy(b);
        return s;
    }
    *out = b;
    return GLS_OK;
}

gls_status gls_raw_batch_reserve(gls_raw_batch* b, int width, int height, int levels, int storage) {
    if (!b) return GLS_ERR_INVALID_ARGUMENT;
    if (width <= 0 || height <= 0 || (width & 1) || (height & 1) || levels < 4 || levels > GLS_MAX_LEVELS ||
        (storage != GLS_STORAGE_F32 && storage != GLS_STORAGE_F16 && storage != GLS_STORAGE_F16_STATS))
        return set_error(b->ctx, GLS_ERR_INVALID_ARGUMENT, "reserve: bad frame size, levels or storage");
    for (size_t l = 0; l < b->lane.size(); l++) {
        gls_raw_converter* c = b->lane[l];
        gls_status s = c->ensure(width, height, levels, storage != GLS_STORAGE_F32);
        if (s == GLS_OK) s = c->ensure_high_noise();
        if (s == GLS_OK) s = c->ensure_staging(width, height);
        if (s != GLS_OK) return batch_error(b, (int)l, s);
    }
    for (size_t l = 0; l < b->lane.size(); l++)
        GLS_CHECK(check_cuda(b->ctx, cudaStreamSynchronize(b->lane_stream[l]), "synchronize lanes"));
    return GLS_OK;
}

gls_status gls_raw_batch_demosaic(gls_raw_batch* b, int n, const gls_image_desc* raws,
                                  const gls_demosaic_params* params, const gls_image_desc* outs) {
    if (!b) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = b->ctx;
    if (n < 0 || (n > 0 && (!raws || !params || !outs))) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "batch arrays");
    std::vector<int> ws(n), hs(n);
    for (int i = 0; i < n; i++) {
        GLS_CHECK(check_desc(ctx, &raws[i], "raw", GLS_R16_UNORM));
        GLS_CHECK(check_desc(ctx, &outs[i], "out", GLS_RGBA8_UNORM, GLS_RGBA_F32));
        if (outs[i].width != raws[i].width || outs[i].height != raws[i].height)
            return set_error(ctx, GLS_ERR_INVALID_SIZE, "frame %d: output size differs from the raw frame", i);
        GLS_CHECK(validate_params(ctx, &params[i], raws[i].width, raws[i].height));
        ws[i] = raws[i].width;
        hs[i] = raws[i].height;
    }
    b->lane_of.assign(n, 0);
    const int lanes = (int)b->lane.size();
    plan_lanes(n, ws.data(), hs.data(), lanes, b->lane_of.data());
    const std::vector<uint64_t> l0 = lane_launches(b);
    GLS_CHECK(batch_fork(b));
    // frames in index order, so the lanes' work is enqueued interleaved
    for (int i = 0; i < n; i++) {
        const int l = b->lane_of[i];
        gls_raw_converter* c = b->lane[l];
        gls_demosaic_params p = params[i];
        gls_status s = c->ensure(ws[i], hs[i], p.pyramid_levels, p.storage != GLS_STORAGE_F32);
        if (s == GLS_OK)
            s = c->run((const uint16_t*)raws[i].ptr, pitch_elems(&raws[i]), &p, outs[i].ptr,
                       outs[i].format == GLS_RGBA_F32, pitch_elems(&outs[i]));
        if (s != GLS_OK) return batch_error(b, l, s);
    }
    return batch_join(b, l0);
}

gls_status gls_raw_batch_demosaic_host(gls_raw_batch* b, int n, const uint16_t* const* raws, const int* widths,
                                       const int* heights, const int* raw_strides, const gls_demosaic_params* params,
                                       uint8_t* const* outs, int out_channels) {
    if (!b) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = b->ctx;
    if (n < 0 || (n > 0 && (!raws || !widths || !heights || !raw_strides || !params || !outs)))
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "batch arrays");
    if (out_channels != 3 && out_channels != 4)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "out_channels must be 3 or 4");
    for (int i = 0; i < n; i++) {
        if (!raws[i] || !outs[i]) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "frame %d: null buffer", i);
        if (raw_strides[i] < widths[i]) return set_error(ctx, GLS_ERR_INVALID_SIZE, "frame %d: stride < width", i);
        GLS_CHECK(validate_params(ctx, &params[i], widths[i], heights[i]));
    }
    b->lane_of.assign(n, 0);
    const int lanes = (int)b->lane.size();
    plan_lanes(n, widths, heights, lanes, b->lane_of.data());
    const std::vector<uint64_t> l0 = lane_launches(b);
    GLS_CHECK(batch_fork(b));
    for (int i = 0; i < n; i++) {
        const int l = b->lane_of[i];
        gls_demosaic_params p = params[i];
        const gls_status s = b->lane[l]->run_host(raws[i], widths[i], heights[i], raw_strides[i], &p, outs[i],
                                                  out_channels, i > 0 ? b->copied[b->lane_of[i - 1]] : nullptr,
                                                  b->copied[l]);
        if (s != GLS_OK) return batch_error(b, l, s);
    }
    GLS_CHECK(batch_join(b, l0));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
}

gls_status gls_raw_batch_demosaic_packed_host(gls_raw_batch* b, int n, const uint8_t* const* packed,
                                              const size_t* n_bytes, const int* bits, const int* widths,
                                              const int* heights, const gls_demosaic_params* params,
                                              uint8_t* const* outs, int out_channels) {
    if (!b) return GLS_ERR_INVALID_ARGUMENT;
    gls_ctx* ctx = b->ctx;
    if (n < 0 || (n > 0 && (!packed || !n_bytes || !bits || !widths || !heights || !params || !outs)))
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "batch arrays");
    if (out_channels != 3 && out_channels != 4)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "out_channels must be 3 or 4");
    for (int i = 0; i < n; i++) {
        if (!outs[i]) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "frame %d: null buffer", i);
        GLS_CHECK(validate_params(ctx, &params[i], widths[i], heights[i]));
        GLS_CHECK(check_packed(ctx, packed[i], n_bytes[i], bits[i], widths[i], heights[i]));
    }
    b->lane_of.assign(n, 0);
    const int lanes = (int)b->lane.size();
    plan_lanes(n, widths, heights, lanes, b->lane_of.data());
    const std::vector<uint64_t> l0 = lane_launches(b);
    GLS_CHECK(batch_fork(b));
    for (int i = 0; i < n; i++) {
        const int l = b->lane_of[i];
        gls_demosaic_params p = params[i];
        const gls_status s = b->lane[l]->run_packed_host(packed[i], n_bytes[i], bits[i], widths[i], heights[i], &p,
                                                         outs[i], out_channels,
                                                         i > 0 ? b->copied[b->lane_of[i - 1]] : nullptr, b->copied[l]);
        if (s != GLS_OK) return batch_error(b, l, s);
    }
    GLS_CHECK(batch_join(b, l0));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
}

}  // extern "C"
