// k_calib.cu -- colour-checker calibration (estimateRawParameters, demosaic_utils.cpp:686-785).
//
// The patch statistics (colorCheckerRawStats, demosaic_utils.cpp:411-533) run on the GPU, one
// block per patch of the 6x4 chart: for each of the four CFA channels, the fp32 sum of the
// clamped normalised values over the patch's quads in raster order, then the fp32 sum of the
// squared deviations from the mean, in the same order -- the reference's own sums, so the
// block's other warps compute a chunk of quads while four lanes of warp 0 add them up, one
// lane per channel.  The chart fit is host arithmetic in the reference's operation order:
// the camera matrix from the patch means and the pseudoinverse of the chart's XYZ
// (matrixFromColorChecker, 83-129; dcraw's pseudoinverse, gls_linalg.hpp:559-590), its white
// point (cam_xyz_coeff, 25-52), and the raw noise slopes of the six neutral patches
// (linear_regression, 604-621: double sums of fp32 products).
#include <algorithm>
#include <cstring>

#include "gls_internal.h"

namespace gls {
namespace {

constexpr int kCalThreads = 128;
constexpr int kCalChunk = 512;  // quads per chunk

// host CFA table (demosaic.hpp:83-88): (x, y) of red, green, blue, green2
__constant__ int c_cal_cfa[4][4][2] = {
    {{1, 0}, {0, 0}, {0, 1}, {1, 1}},
    {{0, 1}, {0, 0}, {1, 0}, {1, 1}},
    {{0, 0}, {1, 0}, {1, 1}, {0, 1}},
    {{1, 1}, {1, 0}, {0, 0}, {0, 1}},
};

struct PatchRect {
    int x, y, w, h;
};

struct CalArgs {
    const uint16_t* raw;
    int stride, bayer;
    float black, white;
    PatchRect patch[24];
};

__device__ __forceinline__ float cal_value(const CalArgs& a, int y, int x, int c) {
    const int(*o)[2] = c_cal_cfa[a.bayer];
    const float v = ((float)a.raw[(size_t)(y + o[c][1]) * a.stride + x + o[c][0]] - a.black) / a.white;
    return fminf(fmaxf(v, 0.0f), 1.0f);
}

// out[c] = sum over the patch's quads (raster order) of the channel value (MODE 0) or of its
// squared deviation from mean[c] (MODE 1)
template <int MODE>
__device__ void cal_sum(const CalArgs& a, const PatchRect& pr, const float* mean, float (*s_v)[kCalChunk],
                        float* out) {
    const int qw = pr.w / 2, n = qw * (pr.h / 2);
    __shared__ float s_out[4];
    float acc = 0.0f;
    for (int base = 0; base < n; base += kCalChunk) {
        for (int i = threadIdx.x; i < kCalChunk && base + i < n; i += kCalThreads) {
            const int q = base + i, y = pr.y + 2 * (q / qw), x = pr.x + 2 * (q % qw);
#pragma unroll
            for (int c = 0; c < 4; c++) {
                float v = cal_value(a, y, x, c);
                if (MODE == 1) {
                    const float d = v - mean[c];
                    v = d * d;
                }
                s_v[c][i] = v;
            }
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            const int cnt = min(kCalChunk, n - base);
            for (int i = 0; i < cnt; i++) acc = acc + s_v[threadIdx.x][i];
        }
        __syncthreads();
    }
    if (threadIdx.x < 4) s_out[threadIdx.x] = acc;
    __syncthreads();
    for (int c = 0; c < 4; c++) out[c] = s_out[c];
    __syncthreads();
}

__global__ void __launch_bounds__(kCalThreads) cal_patch_kernel(CalArgs a, float* stats) {
    __shared__ float s_v[4][kCalChunk];
    const PatchRect pr = a.patch[blockIdx.x];
    const float samples = (float)(pr.w * pr.h / 4);
    float mean[4], var[4];
    cal_sum<0>(a, pr, nullptr, s_v, mean);
    for (int c = 0; c < 4; c++) mean[c] = mean[c] / samples;
    cal_sum<1>(a, pr, mean, s_v, var);
    if (threadIdx.x < 4) {
        stats[blockIdx.x * 8 + threadIdx.x] = mean[threadIdx.x];
        stats[blockIdx.x * 8 + 4 + threadIdx.x] = var[threadIdx.x] / samples;
    }
}

// alignToQuad (demosaic_utils.cpp:54-71)
PatchRect align_to_quad(PatchRect r) {
    if (r.y & 1) {
        r.y += 1;
        r.h -= 1;
    }
    if (r.h & 1) r.h -= 1;
    if (r.x & 1) {
        r.x += 1;
        r.w -= 1;
    }
    if (r.w & 1) r.w -= 1;
    return r;
}

// ColorChecker chart under D65, xyY (matrixFromColorChecker's table)
const float kChartxyY[24][3] = {
    {0.400f, 0.350f, 10.1f}, {0.377f, 0.345f, 35.8f}, {0.247f, 0.251f, 19.3f}, {0.337f, 0.422f, 13.3f},
    {0.265f, 0.240f, 24.3f}, {0.261f, 0.343f, 43.1f}, {0.506f, 0.407f, 30.1f}, {0.211f, 0.175f, 12.0f},
    {0.453f, 0.306f, 19.8f}, {0.285f, 0.202f, 6.6f},  {0.380f, 0.489f, 44.3f}, {0.473f, 0.438f, 43.1f},
    {0.187f, 0.129f, 6.1f},  {0.305f, 0.478f, 23.4f}, {0.539f, 0.313f, 12.0f}, {0.448f, 0.470f, 59.1f},
    {0.364f, 0.233f, 19.8f}, {0.196f, 0.252f, 19.8f}, {0.310f, 0.316f, 90.0f}, {0.310f, 0.316f, 59.1f},
    {0.310f, 0.316f, 36.2f}, {0.310f, 0.316f, 19.8f}, {0.310f, 0.316f, 9.0f},  {0.310f, 0.316f, 3.1f}};

// sRGB -> XYZ (D65), demosaic.hpp's xyz_rgb
const float kXyzRgbCal[3][3] = {
    {0.4124564f, 0.3575761f, 0.1804375f}, {0.2126729f, 0.7151522f, 0.0721750f}, {0.0193339f, 0.1191920f, 0.9503041f}};

void chart_pseudoinverse(const float in[24][3], float out[24][3]) {
    float work[3][6];
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 6; j++) work[i][j] = j == i + 3 ? 1.0f : 0.0f;
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 24; k++) work[i][j] += in[k][i] * in[k][j];
    }
    for (int i = 0; i < 3; i++) {
        float num = work[i][i];
        for (int j = 0; j < 6; j++) work[i][j] /= num;
        for (int k = 0; k < 3; k++) {
            if (k == i) continue;
            num = work[k][i];
            for (int j = 0; j < 6; j++) work[k][j] -= work[i][j] * num;
        }
    }
    for (int i = 0; i < 24; i++)
        for (int j = 0; j < 3; j++) {
            float acc = 0;
            for (int k = 0; k < 3; k++) acc += work[j][k + 3] * in[i][k];
            out[i][j] = acc;
        }
}

bool chart_fit(const float* stats, float cam_xyz[9], float pre_mul[3], float nlf[4]) {
    float xyz[24][3], inv[24][3];
    for (int q = 0; q < 24; q++) {
        const float x = kChartxyY[q][0], y = kChartxyY[q][1], Y = kChartxyY[q][2];
        xyz[q][0] = Y * x / y;
        xyz[q][1] = Y;
        xyz[q][2] = Y * (1 - x - y) / y;
    }
    chart_pseudoinverse(xyz, inv);
    float cx[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            float acc = 0;
            for (int k = 0; k < 24; k++) acc += stats[k * 8 + i] * inv[k][j];
            cx[i][j] = acc;
        }
    // the white point of cam_xyz_coeff: rgb_cam = cam_xyz * xyz_rgb, white = rgb_cam * (1, 1, 1)
    for (int i = 0; i < 3; i++) {
        float rc[3];
        for (int j = 0; j < 3; j++) {
            float acc = 0;
            for (int k = 0; k < 3; k++) acc += cx[i][k] * kXyzRgbCal[k][j];
            rc[j] = acc;
        }
        float white = 0;
        for (int k = 0; k < 3; k++) white += rc[k] * 1.0f;
        if (!((double)white > 0.00001)) return false;
        pre_mul[i] = 1 / white;
    }
    const float norm = cx[1][0] + cx[1][1] + cx[1][2];
    for (int k = 0; k < 9; k++) cam_xyz[k] = cx[k / 3][k % 3] / norm;
    const float p1 = pre_mul[1];
    for (int k = 0; k < 3; k++) pre_mul[k] = pre_mul[k] / p1;
    const int neutral[6] = {23, 22, 21, 20, 19, 18};  // Black, Neutral 3.5, 5, 6.5, 8, White
    for (int c = 0; c < 4; c++) {
        double sx = 0.0, sy = 0.0, sxx = 0.0, sxy = 0.0;
        for (int i = 0; i < 6; i++) sx = sx + stats[neutral[i] * 8 + c];
        for (int i = 0; i < 6; i++) sy = sy + stats[neutral[i] * 8 + 4 + c];
        for (int i = 0; i < 6; i++) {
            const float x = stats[neutral[i] * 8 + c];
            sxx = sxx + (double)(x * x);
        }
        for (int i = 0; i < 6; i++) sxy = sxy + (double)(stats[neutral[i] * 8 + c] * stats[neutral[i] * 8 + 4 + c]);
        nlf[c] = (float)((6.0 * sxy - sx * sy) / (6.0 * sxx - sx * sx));
    }
    return true;
}

gls_status patch_stats(gls_ctx* ctx, const gls_image_desc* raw, float black, float white, int bayer,
                       const int gmb[4], int rotate_180, float stats_out[24 * 8]) {
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R16_UNORM));
    if (!gmb) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "colorCheckerRawStats: chart rectangle is null");
    if (bayer < 0 || bayer > 3) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "bayer pattern %d", bayer);
    if (gmb[0] < 0 || gmb[1] < 0 || gmb[2] < 12 || gmb[3] < 8 || gmb[0] + gmb[2] > raw->width ||
        gmb[1] + gmb[3] > raw->height)
        return set_error(ctx, GLS_ERR_INVALID_SIZE,
                         "colorCheckerRawStats: chart %d,%d %dx%d must lie in the %dx%d frame and be at least 12x8",
                         gmb[0], gmb[1], gmb[2], gmb[3], raw->width, raw->height);
    CalArgs a;
    a.raw = (const uint16_t*)raw->ptr;
    a.stride = pitch_elems(raw);
    a.bayer = bayer;
    a.black = black;
    a.white = white;
    const int pw = gmb[2] / 6, ph = gmb[3] / 4;
    for (int row = 0; row < 4; row++)
        for (int col = 0; col < 6; col++)
            a.patch[row * 6 + col] = align_to_quad({gmb[0] + col * pw + (int)(0.25 * pw),
                                                    gmb[1] + row * ph + (int)(0.25 * ph), (int)(0.5 * pw),
                                                    (int)(0.5 * ph)});
    GLS_CHECK(ensure_scratch(ctx, 24 * 8 * sizeof(float)));
    float* dev = (float*)ctx->scratch;
    cal_patch_kernel<<<24, kCalThreads, 0, ctx->stream>>>(a, dev);
    ctx->launches++;
    GLS_CHECK(check_launch(ctx, "colorCheckerRawStats"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(ctx->host_pinned, dev, 24 * 8 * sizeof(float), cudaMemcpyDeviceToHost,
                                              ctx->stream), "copy patch statistics"));
    GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize"));
    for (int q = 0; q < 24; q++) {  // rotate_180 reverses the patch order
        const int src = rotate_180 ? 23 - q : q;
        memcpy(stats_out + q * 8, ctx->host_pinned + src * 8, 8 * sizeof(float));
    }
    return GLS_OK;
}

}  // namespace
}  // namespace gls

using namespace gls;

extern "C" gls_status gls_color_checker_raw_stats(gls_ctx* ctx, const gls_image_desc* raw, float black_level,
                                                  float white_level, int bayer_pattern, const int gmb_rect[4],
                                                  int rotate_180, float mean[96], float var[96]) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    if (!mean || !var) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "colorCheckerRawStats: null output");
    float st[24 * 8];
    GLS_CHECK(patch_stats(ctx, raw, black_level, white_level, bayer_pattern, gmb_rect, rotate_180, st));
    for (int q = 0; q < 24; q++)
        for (int c = 0; c < 4; c++) {
            mean[q * 4 + c] = st[q * 8 + c];
            var[q * 4 + c] = st[q * 8 + 4 + c];
        }
    return GLS_OK;
}

extern "C" gls_status gls_estimate_raw_parameters(gls_ctx* ctx, const gls_image_desc* raw, float black_level,
                                                  float white_level, int bayer_pattern, const int gmb_rect[4],
                                                  int rotate_180, float cam_xyz[9], float pre_mul[3],
                                                  float raw_nlf[4]) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    if (!cam_xyz || !pre_mul || !raw_nlf)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "estimateRawParameters: null output");
    float st[24 * 8];
    GLS_CHECK(patch_stats(ctx, raw, black_level, white_level, bayer_pattern, gmb_rect, rotate_180, st));
    if (!chart_fit(st, cam_xyz, pre_mul, raw_nlf))
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT,
                         "estimateRawParameters: the fitted camera matrix has a white at or below 1e-5");
    return GLS_OK;
}

extern "C" gls_status gls_fit_color_checker(const float mean[96], const float var[96], float cam_xyz[9],
                                            float pre_mul[3], float raw_nlf[4]) {
    if (!mean || !var || !cam_xyz || !pre_mul || !raw_nlf) return GLS_ERR_INVALID_ARGUMENT;
    float st[24 * 8];
    for (int q = 0; q < 24; q++)
        for (int c = 0; c < 4; c++) {
            st[q * 8 + c] = mean[q * 4 + c];
            st[q * 8 + 4 + c] = var[q * 4 + c];
        }
    return chart_fit(st, cam_xyz, pre_mul, raw_nlf) ? GLS_OK : GLS_ERR_INVALID_ARGUMENT;
}
