// gls_api.cu -- the C ABI of libgls_cuda (include/gls_cuda.h): context, single-stage
// entry points, host colour math and the RawConverter pipeline.
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gls_internal.h"
#include "gls_pipeline.h"
#include "gls_pixel_ops.cuh"
#include "gls_stages.h"

namespace gls {

gls_status set_error(gls_ctx* ctx, gls_status s, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return s;
}

gls_status check_cuda(gls_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return GLS_OK;
    cudaGetLastError();
    return set_error(ctx, e == cudaErrorMemoryAllocation ? GLS_ERR_OUT_OF_MEMORY : GLS_ERR_CUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

gls_status check_launch(gls_ctx* ctx, const char* what) { return check_cuda(ctx, cudaGetLastError(), what); }

gls_status ensure_scratch(gls_ctx* ctx, size_t bytes) {
    if (ctx->scratch_bytes >= bytes) return GLS_OK;
    if (ctx->scratch) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    GLS_CHECK(check_cuda(ctx, cudaMalloc(&ctx->scratch, bytes), "cudaMalloc(scratch)"));
    ctx->scratch_bytes = bytes;
    return GLS_OK;
}

gls_status check_desc(gls_ctx* ctx, const gls_image_desc* d, const char* name, int fmt0, int fmt1) {
    if (!d) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "%s: null descriptor", name);
    if (!d->ptr) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "%s: null pointer", name);
    if (d->width <= 0 || d->height <= 0) return set_error(ctx, GLS_ERR_INVALID_SIZE, "%s: empty image", name);
    const int pb = fmt_bytes(d->format);
    if (pb == 0) return set_error(ctx, GLS_ERR_FORMAT, "%s: unknown pixel format %d", name, d->format);
    if (fmt0 >= 0 && d->format != fmt0 && d->format != fmt1)
        return set_error(ctx, GLS_ERR_FORMAT, "%s: unexpected pixel format %d", name, d->format);
    if (d->stride_bytes < d->width * pb || d->stride_bytes % pb != 0)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "%s: bad stride %d", name, d->stride_bytes);
    if ((uintptr_t)d->ptr % (pb >= 16 ? 16 : pb) != 0)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "%s: misaligned pointer", name);
    return GLS_OK;
}

ImgRef ref_of(const gls_image_desc* d) {
    return ImgRef{d->ptr, d->width, d->height, pitch_elems(d), fmt_is_half(d->format)};
}

// ---- host colour math, restated from demosaic_utils.cpp:25-52, 809-822 and
// gls_linalg.hpp:347-556 in the same float operation order ----
namespace hm {
typedef float M3[3][3];

void mat_mul(const M3 a, const M3 b, M3 out) {
    M3 r;
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            float s = 0;
            for (int k = 0; k < 3; k++) s += a[j][k] * b[k][i];
            r[j][i] = s;
        }
    memcpy(out, r, sizeof(M3));
}

float det2(float a, float b, float c, float d) {
    float r = 0;
    r += 1.0f * a * d;
    r += -1.0f * b * c;
    return r;
}

void minor2(const M3 m, int p, int q, float out[4]) {
    int n = 0;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            if (r != p && c != q) out[n++] = m[r][c];
}

bool inverse(const M3 m, M3 out) {
    float sign = 1, det = 0;
    for (int f = 0; f < 3; f++) {
        float c[4];
        minor2(m, 0, f, c);
        det += sign * m[0][f] * det2(c[0], c[1], c[2], c[3]);
        sign = -sign;
    }
    if (det == 0) return false;
    M3 adj;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const float s = ((i + j) % 2 == 0) ? 1.0f : -1.0f;
            float c[4];
            minor2(m, i, j, c);
            const float d = det2(c[0], c[1], c[2], c[3]);
            adj[j][i] = d != 0 ? s * d : 0;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[i][j] = adj[i][j] / det;
    return true;
}

const M3 kXyzRgb = {{0.4124564f, 0.3575761f, 0.1804375f},
                    {0.2126729f, 0.7151522f, 0.0721750f},
                    {0.0193339f, 0.1191920f, 0.9503041f}};

void cam_ycbcr(const M3 rgb_cam, M3 out) {
    float y[3];
    for (int i = 0; i < 3; i++) {
        float s = 0;
        for (int k = 0; k < 3; k++) s += kXyzRgb[1][k] * rgb_cam[k][i];
        y[i] = s;
    }
    const float KR = y[0], KG = y[1], KB = y[2];
    const M3 r = {{KR, KG, KB},
                  {-0.5f * KR / (1.0f - KB), -0.5f * KG / (1 - KB), 0.5f},
                  {0.5f, -0.5f * KG / (1 - KR), -0.5f * KB / (1 - KR)}};
    memcpy(out, r, sizeof(M3));
}
}  // namespace hm

void host_cam_ycbcr(const float rgb_cam[9], float out[9]) {
    hm::M3 a, r;
    memcpy(a, rgb_cam, sizeof(a));
    hm::cam_ycbcr(a, r);
    memcpy(out, r, sizeof(r));
}

bool host_inverse3x3(const float m[9], float out[9]) {
    hm::M3 a, r;
    memcpy(a, m, sizeof(a));
    if (!hm::inverse(a, r)) return false;
    memcpy(out, r, sizeof(r));
    return true;
}

}  // namespace gls

using namespace gls;

// =========================================================================================
// Context
// =========================================================================================
extern "C" {

gls_status gls_ctx_create(int device, gls_ctx** out) {
    if (!out) return GLS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return GLS_ERR_CUDA;
    }
    if (device < 0 || device >= n) return GLS_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return GLS_ERR_CUDA;
    gls_ctx* ctx = new gls_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaMallocHost(&ctx->host_pinned, 4096) != cudaSuccess) {
        delete ctx;
        return GLS_ERR_OUT_OF_MEMORY;
    }
    *out = ctx;
    return GLS_OK;
}

gls_status gls_ctx_destroy(gls_ctx* ctx) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
    delete ctx;
    return GLS_OK;
}

gls_status gls_ctx_set_stream(gls_ctx* ctx, void* stream) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    ctx->stream = (cudaStream_t)stream;
    return GLS_OK;
}

gls_status gls_ctx_synchronize(gls_ctx* ctx) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
}

const char* gls_status_string(gls_status s) {
    switch (s) {
        case GLS_OK: return "ok";
        case GLS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GLS_ERR_INVALID_SIZE: return "invalid size";
        case GLS_ERR_UNSUPPORTED: return "unsupported";
        case GLS_ERR_CUDA: return "CUDA error";
        case GLS_ERR_OUT_OF_MEMORY: return "out of memory";
        case GLS_ERR_TIMEOUT: return "timeout";
        case GLS_ERR_FORMAT: return "unsupported pixel format";
        case GLS_ERR_BAD_STREAM: return "malformed compressed stream";
    }
    return "unknown status";
}

const char* gls_ctx_last_error(gls_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

uint64_t gls_ctx_kernel_launches(gls_ctx* ctx) { return ctx ? ctx->launches.load() : 0; }

const char* gls_version(void) { return "gls-cuda 0.1 (sm_103a)"; }

// =========================================================================================
// Single stages
// =========================================================================================
#define REQ_CTX \
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;

static gls_status same_size(gls_ctx* ctx, const gls_image_desc* a, const gls_image_desc* b, const char* what) {
    if (a->width != b->width || a->height != b->height)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "%s: image sizes differ", what);
    return GLS_OK;
}

static gls_status same_storage(gls_ctx* ctx, const gls_image_desc* a, const gls_image_desc* b, const char* what) {
    if (fmt_is_half(a->format) != fmt_is_half(b->format))
        return set_error(ctx, GLS_ERR_FORMAT, "%s: input and output storage precision differ", what);
    return GLS_OK;
}

static gls_status check_bayer(gls_ctx* ctx, int bayer) {
    if (bayer < 0 || bayer > 3) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "unknown bayer pattern %d", bayer);
    return GLS_OK;
}

static gls_status check_even(gls_ctx* ctx, const gls_image_desc* d, const char* what) {
    if ((d->width & 1) || (d->height & 1))
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "%s: raw frames must have even width and height", what);
    return GLS_OK;
}

gls_status gls_scale_raw_data(gls_ctx* ctx, const gls_image_desc* raw, const gls_image_desc* scaled, int bayer,
                              const float scale_mul[4], float black_level) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R16_UNORM));
    GLS_CHECK(check_desc(ctx, scaled, "scaled", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(same_size(ctx, raw, scaled, "scaleRawData"));
    GLS_CHECK(check_even(ctx, raw, "scaleRawData"));
    GLS_CHECK(check_bayer(ctx, bayer));
    if (!scale_mul) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "scale_mul is null");
    launch_scale_raw(ctx, (const uint16_t*)raw->ptr, raw->width, raw->height, pitch_elems(raw), ref_of(scaled), bayer,
                     scale_mul, black_level);
    return check_launch(ctx, "scaleRawData");
}

gls_status gls_raw_noise_statistics(gls_ctx* ctx, const gls_image_desc* scaled, int bayer, const gls_image_desc* mean,
                                    const gls_image_desc* var) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, scaled, "scaled", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_desc(ctx, mean, "mean", GLS_RGBA_F32));
    GLS_CHECK(check_desc(ctx, var, "var", GLS_RGBA_F32));
    GLS_CHECK(check_even(ctx, scaled, "rawNoiseStatistics"));
    GLS_CHECK(check_bayer(ctx, bayer));
    if (mean->width != scaled->width / 2 || mean->height != scaled->height / 2 || var->width != mean->width ||
        var->height != mean->height)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "rawNoiseStatistics: statistics images must be half size");
    launch_raw_stats(ctx, ref_of(scaled), bayer, (float4*)mean->ptr, pitch_elems(mean), (float4*)var->ptr,
                     pitch_elems(var));
    return check_launch(ctx, "rawNoiseStatistics");
}

static gls_status fetch_nlf(gls_ctx* ctx, const float* dev, float* out, int n) {
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(ctx->host_pinned, dev, n * sizeof(float), cudaMemcpyDeviceToHost,
                                              ctx->stream), "copy noise model"));
    GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize"));
    memcpy(out, ctx->host_pinned, n * sizeof(float));
    return GLS_OK;
}

gls_status gls_compute_raw_noise_statistics(gls_ctx* ctx, const gls_image_desc* scaled, int bayer, float out_nlf[8]) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, scaled, "scaled", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_even(ctx, scaled, "computeRawNoiseStatistics"));
    GLS_CHECK(check_bayer(ctx, bayer));
    if (!out_nlf) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "out_nlf is null");
    GLS_CHECK(ensure_scratch(ctx, kNlfScratchBytes + 256));
    NlfScratch s = nlf_scratch_at(ctx->scratch);
    float* out_dev = (float*)((char*)ctx->scratch + kNlfScratchBytes);
    GLS_CHECK(nlf_fit_raw_scaled(ctx, scaled->ptr, fmt_is_half(scaled->format), scaled->width, scaled->height,
                                 pitch_elems(scaled), bayer, s, out_dev));
    return fetch_nlf(ctx, out_dev, out_nlf, 8);
}

gls_status gls_interpolate_green(gls_ctx* ctx, const gls_image_desc* scaled, const gls_image_desc* green, int bayer,
                                 float luma_variance) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, scaled, "scaled", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_desc(ctx, green, "green", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(same_size(ctx, scaled, green, "interpolateGreen"));
    GLS_CHECK(same_storage(ctx, scaled, green, "interpolateGreen"));
    GLS_CHECK(check_bayer(ctx, bayer));
    launch_green(ctx, ref_of(scaled), ref_of(green), bayer, luma_variance, nullptr);
    return check_launch(ctx, "interpolateGreen");
}

gls_status gls_interpolate_red_blue(gls_ctx* ctx, const gls_image_desc* scaled, const gls_image_desc* green,
                                    const gls_image_desc* rgb, int bayer, float chroma_variance, int rotate_180) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, scaled, "scaled", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_desc(ctx, green, "green", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_desc(ctx, rgb, "rgb", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, scaled, green, "interpolateRedBlue"));
    GLS_CHECK(same_size(ctx, scaled, rgb, "interpolateRedBlue"));
    GLS_CHECK(same_storage(ctx, scaled, green, "interpolateRedBlue"));
    GLS_CHECK(same_storage(ctx, scaled, rgb, "interpolateRedBlue"));
    GLS_CHECK(check_bayer(ctx, bayer));
    launch_red_blue(ctx, ref_of(scaled), ref_of(green), ref_of(rgb), bayer, chroma_variance, nullptr, rotate_180 != 0);
    return check_launch(ctx, "interpolateRedBlue");
}

gls_status gls_fast_debayer(gls_ctx* ctx, const gls_image_desc* scaled, const gls_image_desc* rgb, int bayer) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, scaled, "scaled", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_desc(ctx, rgb, "rgb", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_storage(ctx, scaled, rgb, "fastDebayer"));
    GLS_CHECK(check_even(ctx, scaled, "fastDebayer"));
    GLS_CHECK(check_bayer(ctx, bayer));
    if (rgb->width != scaled->width / 2 || rgb->height != scaled->height / 2)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "fastDebayer: output must be half size");
    launch_fast_debayer(ctx, ref_of(scaled), ref_of(rgb), bayer);
    return check_launch(ctx, "fastDebayer");
}

gls_status gls_blend_highlights(gls_ctx* ctx, const gls_image_desc* in, float clip, const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "blendHighlights"));
    GLS_CHECK(same_storage(ctx, in, out, "blendHighlights"));
    launch_highlights(ctx, ref_of(in), ref_of(out), clip);
    return check_launch(ctx, "blendHighlights");
}

gls_status gls_transform_image(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out,
                               const float transform[9]) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "transformImage"));
    GLS_CHECK(same_storage(ctx, in, out, "transformImage"));
    if (!transform) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "transform is null");
    launch_transform(ctx, ref_of(in), ref_of(out), transform);
    return check_launch(ctx, "transformImage");
}

gls_status gls_despeckle_image(gls_ctx* ctx, const gls_image_desc* in, const float var_a[3], const float var_b[3],
                               const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "despeckleImage"));
    GLS_CHECK(same_storage(ctx, in, out, "despeckleImage"));
    if (!var_a || !var_b) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "var_a/var_b is null");
    if (in->ptr == out->ptr) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "despeckleImage cannot run in place");
    launch_despeckle(ctx, ref_of(in), ref_of(out), var_a[0], var_b[0]);
    return check_launch(ctx, "despeckleImage");
}

gls_status gls_downsample_image(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_storage(ctx, in, out, "downsampleImage"));
    launch_downsample(ctx, ref_of(in), ref_of(out));
    return check_launch(ctx, "downsampleImage");
}

gls_status gls_noise_statistics(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32));
    GLS_CHECK(same_size(ctx, in, out, "noiseStatistics"));
    launch_noise_stats(ctx, ref_of(in), (float4*)out->ptr, pitch_elems(out));
    return check_launch(ctx, "noiseStatistics");
}

gls_status gls_compute_noise_statistics(gls_ctx* ctx, const gls_image_desc* in, float out_nlf[6]) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    if (!out_nlf) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "out_nlf is null");
    GLS_CHECK(ensure_scratch(ctx, kNlfScratchBytes + 256));
    NlfScratch s = nlf_scratch_at(ctx->scratch);
    float* out_dev = (float*)((char*)ctx->scratch + kNlfScratchBytes);
    GLS_CHECK(nlf_fit_level(ctx, in->ptr, fmt_is_half(in->format), in->width, in->height, pitch_elems(in), s, out_dev));
    return fetch_nlf(ctx, out_dev, out_nlf, 6);
}

static NlfArg host_nlf(const float var_a[3], const float var_b[3]) {
    NlfArg a;
    a.dev = nullptr;
    for (int k = 0; k < 3; k++) {
        a.host[k] = var_a[k];
        a.host[3 + k] = var_b[k];
    }
    for (int k = 0; k < 6; k++) a.mul[k] = 1.0f;
    return a;
}

gls_status gls_denoise_image(gls_ctx* ctx, const gls_image_desc* in, const float var_a[3], const float var_b[3],
                             float chroma_boost, float gradient_boost, const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "denoiseImage"));
    GLS_CHECK(same_storage(ctx, in, out, "denoiseImage"));
    if (!var_a || !var_b) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "var_a/var_b is null");
    if (in->ptr == out->ptr) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "denoiseImage cannot run in place");
    launch_bilateral(ctx, ref_of(in), ref_of(out), host_nlf(var_a, var_b), chroma_boost, gradient_boost);
    return check_launch(ctx, "denoiseImage");
}

gls_status gls_denoise_image_guided(gls_ctx* ctx, const gls_image_desc* in, const float var_a[3], const float var_b[3],
                                    const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "denoiseImageGuided"));
    GLS_CHECK(same_storage(ctx, in, out, "denoiseImageGuided"));
    if (!var_a || !var_b) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "var_a/var_b is null");
    if (in->ptr == out->ptr) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "denoiseImageGuided cannot run in place");
    launch_guided_fast(ctx, ref_of(in), ref_of(out), host_nlf(var_a, var_b));
    return check_launch(ctx, "denoiseImageGuided");
}

gls_status gls_guided_filter(gls_ctx* ctx, const gls_image_desc* in, int filter_size, const float eps[3],
                             const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "GuidedFilter::filter"));
    GLS_CHECK(same_storage(ctx, in, out, "GuidedFilter::filter"));
    if (!eps) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "eps is null");
    if (filter_size < 1) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "filter_size must be >= 1");
    GLS_CHECK(ensure_scratch(ctx, guided_filter_scratch_bytes(in->width, in->height)));
    const float zero[3] = {0, 0, 0};
    launch_guided_filter(ctx, ref_of(in), ref_of(out), filter_size, host_nlf(zero, eps), ctx->scratch);
    return check_launch(ctx, "GuidedFilter::filter");
}

gls_status gls_reassemble_image(gls_ctx* ctx, const gls_image_desc* den0, const gls_image_desc* img1,
                                const gls_image_desc* den1, float sharpening, const float nlf[2],
                                const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, den0, "den0", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, img1, "img1", den0->format));
    GLS_CHECK(check_desc(ctx, den1, "den1", den0->format));
    GLS_CHECK(check_desc(ctx, out, "out", den0->format));
    GLS_CHECK(same_size(ctx, den0, out, "reassembleImage"));
    GLS_CHECK(same_size(ctx, img1, den1, "reassembleImage"));
    if (!nlf) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "nlf is null");
    NlfArg a;
    a.dev = nullptr;
    for (int k = 0; k < 6; k++) {
        a.host[k] = 0;
        a.mul[k] = 1;
    }
    a.host[0] = nlf[0];
    a.host[3] = nlf[1];
    launch_reassemble(ctx, ref_of(den0), ref_of(img1), ref_of(den1), ref_of(out), sharpening, a);
    return check_launch(ctx, "reassembleImage");
}

gls_status gls_local_tone_mapping_mask(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* guide,
                                       const gls_ltm_params* ltm, const float transform[9], const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, guide, "guide", in->format));
    GLS_CHECK(check_desc(ctx, out, "out", fmt_is_half(in->format) ? GLS_R_F16 : GLS_R_F32));
    GLS_CHECK(same_size(ctx, in, out, "localToneMappingMask"));
    if (!ltm || !transform) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "ltm/transform is null");
    LtmParams lp{ltm->guidedFilterEps, ltm->shadows, ltm->highlights, ltm->detail};
    launch_ltm(ctx, ref_of(in), ref_of(guide), ref_of(out), lp, transform);
    return check_launch(ctx, "localToneMappingMask");
}

gls_status gls_convert_to_srgb(gls_ctx* ctx, const gls_image_desc* linear, const gls_image_desc* ltm_mask,
                               const gls_image_desc* out, const float rgb_cam[9], const gls_rgb_conversion_params* p) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, linear, "linear", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA8_UNORM, GLS_RGBA_F32));
    GLS_CHECK(same_size(ctx, linear, out, "convertTosRGB"));
    if (!rgb_cam || !p) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "rgb_cam/params is null");
    ImgRef mk;
    if (p->localToneMapping) {
        if (!ltm_mask) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "localToneMapping needs an ltm mask");
        GLS_CHECK(check_desc(ctx, ltm_mask, "ltm_mask", fmt_is_half(linear->format) ? GLS_R_F16 : GLS_R_F32));
        GLS_CHECK(same_size(ctx, linear, ltm_mask, "convertTosRGB"));
        mk = ref_of(ltm_mask);
    }
    const RgbParams rp = rgb_params_init(p->contrast, p->saturation, p->toneCurveSlope, p->exposureBias, p->blacks, p->localToneMapping);
    launch_srgb(ctx, ref_of(linear), p->localToneMapping ? &mk : nullptr, out->ptr, out->format == GLS_RGBA_F32,
                pitch_elems(out), rgb_cam, rp);
    return check_launch(ctx, "convertTosRGB");
}

gls_status gls_bayer_to_raw_rgba(gls_ctx* ctx, const gls_image_desc* raw, const gls_image_desc* rgba, int bayer) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(check_desc(ctx, rgba, "rgba", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_storage(ctx, raw, rgba, "bayerToRawRGBA"));
    GLS_CHECK(check_even(ctx, raw, "bayerToRawRGBA"));
    GLS_CHECK(check_bayer(ctx, bayer));
    if (rgba->width != raw->width / 2 || rgba->height != raw->height / 2)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "bayerToRawRGBA: output must be half size");
    launch_bayer_to_rgba(ctx, ref_of(raw), ref_of(rgba), bayer);
    return check_launch(ctx, "bayerToRawRGBA");
}

gls_status gls_raw_rgba_to_bayer(gls_ctx* ctx, const gls_image_desc* rgba, const gls_image_desc* raw, int bayer) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, rgba, "rgba", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R_F32, GLS_R_F16));
    GLS_CHECK(same_storage(ctx, raw, rgba, "rawRGBAToBayer"));
    GLS_CHECK(check_even(ctx, raw, "rawRGBAToBayer"));
    GLS_CHECK(check_bayer(ctx, bayer));
    if (rgba->width != raw->width / 2 || rgba->height != raw->height / 2)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "rawRGBAToBayer: input must be half size");
    launch_rgba_to_bayer(ctx, ref_of(rgba), ref_of(raw), bayer);
    return check_launch(ctx, "rawRGBAToBayer");
}

gls_status gls_despeckle_raw_rgba(gls_ctx* ctx, const gls_image_desc* in, const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "despeckleRawRGBAImage"));
    GLS_CHECK(same_storage(ctx, in, out, "despeckleRawRGBAImage"));
    if (in->ptr == out->ptr) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "despeckleRawRGBAImage cannot run in place");
    launch_despeckle_rgba(ctx, ref_of(in), ref_of(out));
    return check_launch(ctx, "despeckleRawRGBAImage");
}

gls_status gls_denoise_raw_rgba(gls_ctx* ctx, const gls_image_desc* in, const float raw_variance[4],
                                const gls_image_desc* out) {
    REQ_CTX
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(same_size(ctx, in, out, "denoiseRawRGBAImage"));
    GLS_CHECK(same_storage(ctx, in, out, "denoiseRawRGBAImage"));
    if (!raw_variance) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "raw_variance is null");
    if (in->ptr == out->ptr) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "denoiseRawRGBAImage cannot run in place");
    launch_denoise_rgba(ctx, ref_of(in), ref_of(out), raw_variance, nullptr);
    return check_launch(ctx, "denoiseRawRGBAImage");
}

gls_status gls_unpack_raw_bits(gls_ctx* ctx, const void* packed, size_t n_bytes, int bits, uint16_t* out,
                               size_t n_samples) {
    REQ_CTX
    if (!packed || !out) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "null pointer");
    if (bits != 10 && bits != 12 && bits != 14 && bits != 16)
        return set_error(ctx, GLS_ERR_UNSUPPORTED, "unsupported bit depth %d", bits);
    if (n_samples == 0) return GLS_OK;
    if (n_samples > (n_bytes * 8) / (size_t)bits)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "packed buffer holds only %zu samples", (n_bytes * 8) / bits);
    launch_unpack(ctx, packed, n_bytes, bits, out, n_samples);
    return check_launch(ctx, "unpack raw bits");
}

// ---- host colour math ----
gls_status gls_cam_xyz_coeff(const float cam_xyz[9], float pre_mul[3], float rgb_cam[9]) {
    if (!cam_xyz || !pre_mul || !rgb_cam) return GLS_ERR_INVALID_ARGUMENT;
    hm::M3 cx, rc;
    memcpy(cx, cam_xyz, sizeof(cx));
    hm::mat_mul(cx, hm::kXyzRgb, rc);
    float white[3];
    for (int i = 0; i < 3; i++) {
        float s = 0;
        for (int k = 0; k < 3; k++) s += rc[i][k] * 1.0f;
        white[i] = s;
    }
    for (int i = 0; i < 3; i++)
        if (!(white[i] > 0.00001f)) return GLS_ERR_INVALID_ARGUMENT;  // std::range_error in the reference
    const hm::M3 pm = {{1 / white[0], 0, 0}, {0, 1 / white[1], 0}, {0, 0, 1 / white[2]}};
    for (int i = 0; i < 3; i++) pre_mul[i] = 1 / white[i];
    hm::M3 t, inv;
    hm::mat_mul(pm, rc, t);
    if (!hm::inverse(t, inv)) return GLS_ERR_INVALID_ARGUMENT;
    memcpy(rgb_cam, inv, sizeof(inv));
    return GLS_OK;
}

gls_status gls_cam_ycbcr(const float rgb_cam[9], float out[9]) {
    if (!rgb_cam || !out) return GLS_ERR_INVALID_ARGUMENT;
    host_cam_ycbcr(rgb_cam, out);
    return GLS_OK;
}

gls_status gls_inverse3x3(const float m[9], float out[9]) {
    if (!m || !out) return GLS_ERR_INVALID_ARGUMENT;
    return host_inverse3x3(m, out) ? GLS_OK : GLS_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
