// k_awb.cu -- autoWhiteBalance (demosaic_utils.cpp:832-1026) on the GPU, bit-exact.
//
// The reference splits the raw frame into 4x4 tiles of even size and, per tile, walks its
// 2x2 quads in raster order three times, each time keeping fp32 running sums:
//   1. M = mean YCbCr of the quads (camera RGB scaled by scale_mul / 65535 and clipped at
//      1, times the camera->YCbCr matrix), plus the count of quads with a channel in (0.5, 1];
//   2. D = mean |YCbCr - M|;
//   3. for the "near-white" quads (Cb and Cr inside windows set by M and D): per luma bin
//      (128 bins of round(127 Y)), the sum of their (raw - black) / white, the count, and the
//      largest luma.
// The gain of a tile comes from the brightest bins holding 1 % of the near-white quads; the
// frame's gain is the mean of the 16 tiles' gains.
//
// fp32 sums in a fixed order are not associative, so the kernel keeps the reference's order:
// one block per tile; in passes 1 and 2 the block's other warps compute the per-quad terms
// of a chunk in parallel while three lanes of warp 0 add up the previous chunk, one lane per
// component, in quad order (the adds form the critical path: one dependent add per quad and
// pass).  In pass 3 the selected quads of a chunk are sorted by bin, stably (warp match
// ranks plus per-bin offsets), and 128 threads, one per bin, add their own bin's entries in
// quad order.  Counts, the luma
// maximum and the highlight count are exact in any order.  The 16 tile results are combined
// in tile order by the last block to finish (a ticket, no waiting).
#include "gls_internal.h"

namespace gls {
namespace {

constexpr int kAwbThreads = 256;
constexpr int kAwbChunk = 1024;  // quads per chunk
constexpr int kAwbBins = 128;
constexpr int kAwbTiles = 16;

// host CFA table (demosaic.hpp:83-88): (x, y) of red, green, blue, green2
__constant__ int c_awb_cfa[4][4][2] = {
    {{1, 0}, {0, 0}, {0, 1}, {1, 1}},  // grbg
    {{0, 1}, {0, 0}, {1, 0}, {1, 1}},  // gbrg
    {{0, 0}, {1, 0}, {1, 1}, {0, 1}},  // rggb
    {{1, 1}, {1, 0}, {0, 0}, {0, 1}},  // bggr
};

struct AwbArgs {
    const uint16_t* raw;
    int stride;  // pixels per row
    int tw, th;  // tile size (even)
    int bayer;
    float m[9];     // camera RGB -> YCbCr
    float smul[3];  // scale_mul / scale_mul[1]
    float black, white;
    float hl_div;  // (float)(width * height / 4)
};

struct AwbTile {
    float gain[3];
    int highlights;
};

// The four raw values of quad (qx, qy): red, green, blue, green2 (readQuad,
// demosaic_utils.cpp:836-849, before its conversion).
struct RawQuad {
    uint16_t v[4];
};

__device__ __forceinline__ RawQuad awb_load(const AwbArgs& a, const uint16_t* tile, int qx, int qy) {
    const int(*o)[2] = c_awb_cfa[a.bayer];
    const uint16_t* p = tile + (size_t)(2 * qy) * a.stride + 2 * qx;
    RawQuad r;
#pragma unroll
    for (int c = 0; c < 4; c++) r.v[c] = __ldg(p + o[c][1] * a.stride + o[c][0]);
    return r;
}

// readQuad's value: {red, (green + green2) / 2, blue}
__device__ __forceinline__ void awb_quad(const RawQuad& r, float q[3]) {
    q[0] = (float)r.v[0];
    q[1] = ((float)r.v[1] + (float)r.v[3]) / 2.0f;
    q[2] = (float)r.v[2];
}

// The YCbCr of a quad (rows accumulated from 0, as gls::Matrix * gls::Vector does) and
// whether a channel of its clipped RGB lies in (0.5, 1] (demosaic_utils.cpp:861-881).
__device__ __forceinline__ bool awb_ycbcr(const AwbArgs& a, const float q[3], float p[3]) {
    float rgb[3];
    bool hl = false;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        rgb[c] = (a.smul[c] * (q[c] - a.black)) / 65535.0f;
        if (rgb[c] > 1.0f) rgb[c] = 1.0f;
        else if (rgb[c] > 0.5f) hl = true;
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) acc = acc + a.m[3 * j + k] * rgb[k];
        p[j] = acc;
    }
    return hl;
}

// round(127 Y) clamped to the bins; a negative value goes to the top bin, as the
// reference's size_t conversion before its clamp does on x86-64.
__device__ __forceinline__ int awb_bin(float Y) {
    const float r = roundf((float)(kAwbBins - 1) * Y);
    if (r < 0.0f || r > (float)(kAwbBins - 1)) return kAwbBins - 1;
    return (int)r;
}

// acc += v[0] + ... + v[n-1], one add at a time in index order.  v holds kAwbChunk floats;
// the next 16 are loaded while the current 16 are added (reads stay inside the buffer).
__device__ __forceinline__ float serial_sum(float acc, const float* v, int n) {
    int i = 0;
    float4 cur[4];
#pragma unroll
    for (int j = 0; j < 4; j++) cur[j] = reinterpret_cast<const float4*>(v)[j];
    for (; i + 16 <= n; i += 16) {
        const int nx = min(i + 16, kAwbChunk - 16);
        float4 nxt[4];
#pragma unroll
        for (int j = 0; j < 4; j++) nxt[j] = reinterpret_cast<const float4*>(v + nx)[j];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            acc = acc + cur[j].x;
            acc = acc + cur[j].y;
            acc = acc + cur[j].z;
            acc = acc + cur[j].w;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) cur[j] = nxt[j];
    }
    for (; i < n; i++) acc = acc + v[i];
    return acc;
}

constexpr int kProducers = kAwbThreads - 32;
constexpr int kPerProducer = (kAwbChunk + kProducers - 1) / kProducers;
constexpr int kRounds = kAwbChunk / kAwbThreads;  // pass 3: quads per thread and chunk
constexpr int kWarps = kAwbThreads / 32;

union AwbSmem {
    float v[2][3][kAwbChunk];  // passes 1 and 2: double-buffered per-quad terms
    struct {
        int off[kWarps][kAwbBins];  // per (warp, bin): count, then offset
        float4 sorted[kAwbChunk];   // the chunk's near-white entries, by bin then quad
    } p3;
};

// Passes 1 and 2: the quad-order fp32 sums of the three YCbCr components (MODE 0) or of
// their absolute deviations from mean[] (MODE 1).  Warps 1.. compute chunk k while lanes
// 0-2 of warp 0 add up chunk k - 1.  Returns the thread's count of highlight quads
// (MODE 0) and leaves the sums in out[] (all threads).
template <int MODE>
__device__ int awb_sum_pass(const AwbArgs& a, const uint16_t* tile, int qw, int n, const float* mean, AwbSmem& sm,
                            float* out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunks = (n + kAwbChunk - 1) / kAwbChunk;
    int hl = 0;
    float acc = 0.0f;
    for (int k = 0; k <= nchunks; k++) {
        if (warp != 0) {
            if (k < nchunks) {
                RawQuad r[kPerProducer];
#pragma unroll
                for (int j = 0; j < kPerProducer; j++) {  // every load first, then the arithmetic
                    const int i = threadIdx.x - 32 + j * kProducers, q = k * kAwbChunk + i;
                    if (i < kAwbChunk && q < n) r[j] = awb_load(a, tile, q % qw, q / qw);
                }
#pragma unroll
                for (int j = 0; j < kPerProducer; j++) {
                    const int i = threadIdx.x - 32 + j * kProducers, q = k * kAwbChunk + i;
                    if (i < kAwbChunk && q < n) {
                        float qv[3], p[3];
                        awb_quad(r[j], qv);
                        const bool h = awb_ycbcr(a, qv, p);
                        if (MODE == 0) {
                            hl += h;
                        } else {
#pragma unroll
                            for (int c = 0; c < 3; c++) p[c] = fabsf(p[c] - mean[c]);
                        }
#pragma unroll
                        for (int c = 0; c < 3; c++) sm.v[k & 1][c][i] = p[c];
                    }
                }
            }
        } else if (k > 0 && lane < 3) {
            const int base = (k - 1) * kAwbChunk;
            acc = serial_sum(acc, sm.v[(k - 1) & 1][lane], min(kAwbChunk, n - base));
        }
        __syncthreads();
    }
    __shared__ float s_out[3];
    if (warp == 0 && lane < 3) s_out[lane] = acc;
    __syncthreads();
    for (int c = 0; c < 3; c++) out[c] = s_out[c];
    __syncthreads();
    return hl;
}

__device__ __forceinline__ int block_sum_int(int v, int* s_red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    for (int w = 0; w < kWarps; w++) t += s_red[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kAwbThreads) awb_tile_kernel(AwbArgs a, AwbTile* tiles, unsigned* ticket,
                                                               float* out) {
    __shared__ __align__(16) AwbSmem sm;
    __shared__ float s_bin[kAwbBins][3];
    __shared__ int s_bin_n[kAwbBins];
    __shared__ int s_base[kAwbBins], s_count[kAwbBins];
    __shared__ int s_red[kWarps];
    __shared__ float s_fmax[kWarps];
    __shared__ bool s_last;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tx = blockIdx.x & 3, ty = blockIdx.x >> 2;
    const uint16_t* tile = a.raw + (size_t)ty * a.th * a.stride + (size_t)tx * a.tw;
    const int qw = a.tw / 2, qh = a.th / 2, n = qw * qh;

    // pass 1: M (demosaic_utils.cpp:859-882)
    float M[3], D[3];
    const int hl = block_sum_int(awb_sum_pass<0>(a, tile, qw, n, nullptr, sm, M), s_red);
    const float n_quads = (float)a.th * (float)a.tw / 4.0f;
    for (int c = 0; c < 3; c++) M[c] = M[c] / n_quads;
    // pass 2: D (demosaic_utils.cpp:899-906)
    awb_sum_pass<1>(a, tile, qw, n, M, sm, D);
    const float n_yuv = (float)qh * (float)qw;
    for (int c = 0; c < 3; c++) D[c] = D[c] / n_yuv;

    // pass 3: near-white quads by luma bin (demosaic_utils.cpp:908-940).  Per chunk, warp w
    // holds quads base + 128 w + 32 r + lane (r = 0..3), so (warp, r, lane) is quad order;
    // the entries of a bin are placed in that order (warp offsets, then ranks over rounds),
    // a stable sort by bin, and thread b < 128 adds bin b's entries in quad order.
    const float Wr = 1.5f, WCr = 1.5f;
    const float c1 = M[1] + copysignf(D[1], M[1]), c2 = WCr * M[2] + copysignf(D[2], M[2]);
    const float w1 = Wr * D[1], w2 = Wr * D[2];
    const unsigned lanes_below = (1u << lane) - 1u;
    float bin_acc[3] = {0.0f, 0.0f, 0.0f};
    int bin_n = 0, white_n = 0;
    float ymax = 0.0f;
    int* off_flat = &sm.p3.off[0][0];
    RawQuad rq[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
        const int q = warp * (kRounds * 32) + r * 32 + lane;
        if (q < n) rq[r] = awb_load(a, tile, q % qw, q / qw);
    }
    for (int base = 0; base < n; base += kAwbChunk) {
        for (int i = tid; i < kWarps * kAwbBins; i += kAwbThreads) off_flat[i] = 0;
        int bin[kRounds];
        float4 e[kRounds];
#pragma unroll
        for (int r = 0; r < kRounds; r++) {
            bin[r] = -1;
            const int q = base + warp * (kRounds * 32) + r * 32 + lane;
            if (q < n) {
                float qv[3], p[3];
                awb_quad(rq[r], qv);
                awb_ycbcr(a, qv, p);
                if (fabsf(p[1] - c1) < w1 && fabsf(p[2] - c2) < w2) {
                    const float Y = p[0];
                    ymax = Y > ymax ? Y : ymax;
                    bin[r] = awb_bin(Y);
                    e[r] = make_float4((qv[0] - a.black) / a.white, (qv[1] - a.black) / a.white,
                                       (qv[2] - a.black) / a.white, 0.0f);
                    white_n++;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kRounds; r++) {  // the next chunk's quads load during the sort
            const int q = base + kAwbChunk + warp * (kRounds * 32) + r * 32 + lane;
            if (q < n) rq[r] = awb_load(a, tile, q % qw, q / qw);
        }
        __syncthreads();  // counts cleared
        // rank of each entry among the same bin's entries of this warp, rounds in order:
        // the lowest lane of a match group reads and advances the warp's count of the bin
        int rank[kRounds];
#pragma unroll
        for (int r = 0; r < kRounds; r++) {
            const unsigned same = __match_any_sync(0xffffffffu, bin[r]);
            const int leader = __ffs(same) - 1;
            int prior = 0;
            if (bin[r] >= 0 && lane == leader) {
                prior = sm.p3.off[warp][bin[r]];
                sm.p3.off[warp][bin[r]] = prior + __popc(same);
            }
            prior = __shfl_sync(0xffffffffu, prior, leader);
            rank[r] = prior + __popc(same & lanes_below);
            __syncwarp();
        }
        __syncthreads();
        if (tid < kAwbBins) {  // per bin: offsets over warps, then over bins
            int total = 0;
#pragma unroll
            for (int w = 0; w < kWarps; w++) {
                const int c = sm.p3.off[w][tid];
                sm.p3.off[w][tid] = total;
                total += c;
            }
            int incl = total;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) s_red[warp] = incl;
            s_count[tid] = total;
            s_base[tid] = incl - total;
        }
        __syncthreads();
        if (tid < kAwbBins)
            for (int w = 0; w < (tid >> 5); w++) s_base[tid] += s_red[w];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kRounds; r++)
            if (bin[r] >= 0) sm.p3.sorted[s_base[bin[r]] + sm.p3.off[warp][bin[r]] + rank[r]] = e[r];
        __syncthreads();
        if (tid < kAwbBins) {
            const int b0 = s_base[tid], b1 = b0 + s_count[tid];
            for (int i = b0; i < b1; i++) {
                const float4 v = sm.p3.sorted[i];
                bin_acc[0] = bin_acc[0] + v.x;
                bin_acc[1] = bin_acc[1] + v.y;
                bin_acc[2] = bin_acc[2] + v.z;
            }
            bin_n += b1 - b0;
        }
        __syncthreads();
    }
    if (tid < kAwbBins) {
        for (int c = 0; c < 3; c++) s_bin[tid][c] = bin_acc[c];
        s_bin_n[tid] = bin_n;
    }
    white_n = block_sum_int(white_n, s_red);
    for (int o = 16; o > 0; o >>= 1) {
        const float v = __shfl_xor_sync(0xffffffffu, ymax, o);
        ymax = v > ymax ? v : ymax;
    }
    if (lane == 0) s_fmax[warp] = ymax;
    __syncthreads();

    // the tile's gain (demosaic_utils.cpp:942-965)
    if (tid == 0) {
        float YMax = 0.0f;
        for (int w = 0; w < kWarps; w++) YMax = s_fmax[w] > YMax ? s_fmax[w] : YMax;
        AwbTile r;
        const int top = awb_bin(YMax);
        if (top == 0) {
            r = AwbTile{{1.0f, 1.0f, 1.0f}, 0};
        } else {
            int n90 = 0;
            float avg[3] = {0.0f, 0.0f, 0.0f};
            for (int i = top; i >= 0; i--) {
                for (int c = 0; c < 3; c++) avg[c] = avg[c] + s_bin[i][c];
                n90 += s_bin_n[i];
                if ((float)n90 > 0.01f * (float)white_n) break;
            }
            float g[3];
            for (int c = 0; c < 3; c++) g[c] = YMax / (avg[c] / (float)n90);
            for (int c = 0; c < 3; c++) r.gain[c] = g[c] / g[1];
            r.highlights = hl;
        }
        tiles[blockIdx.x] = r;
        __threadfence();
        s_last = atomicAdd(ticket, 1u) == kAwbTiles - 1;
    }
    __syncthreads();

    // the frame's gain: mean of the tiles' gains in tile order (demosaic_utils.cpp:1005-1018)
    if (s_last && tid == 0) {
        __threadfence();
        const volatile AwbTile* vt = tiles;
        float g[3] = {0.0f, 0.0f, 0.0f}, h = 0.0f;
        for (int t = 0; t < kAwbTiles; t++) {
            for (int c = 0; c < 3; c++) g[c] = g[c] + vt[t].gain[c];
            h = h + (float)vt[t].highlights;
        }
        for (int c = 0; c < 3; c++) g[c] = g[c] / 16.0f;
        const float g1 = g[1];
        for (int c = 0; c < 3; c++) out[c] = g[c] / g1;
        out[3] = h / a.hl_div;
        *ticket = 0u;
    }
}

}  // namespace
}  // namespace gls

using namespace gls;

extern "C" gls_status gls_auto_white_balance(gls_ctx* ctx, const gls_image_desc* raw, const float rgb_ycbcr[9],
                                             const float scale_mul[4], float white_level, float black_level,
                                             int bayer_pattern, float wb_out[3], float* highlights) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    GLS_CHECK(check_desc(ctx, raw, "raw", GLS_R16_UNORM));
    if (!rgb_ycbcr || !scale_mul || !wb_out)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "autoWhiteBalance: null matrix, scale_mul or output");
    if (bayer_pattern < 0 || bayer_pattern > 3)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "autoWhiteBalance: bayer pattern %d", bayer_pattern);
    AwbArgs a;
    a.raw = (const uint16_t*)raw->ptr;
    a.stride = pitch_elems(raw);
    a.tw = 2 * ((raw->width / 4) / 2);
    a.th = 2 * ((raw->height / 4) / 2);
    a.bayer = bayer_pattern;
    for (int i = 0; i < 9; i++) a.m[i] = rgb_ycbcr[i];
    const float s1 = scale_mul[1];
    for (int c = 0; c < 3; c++) a.smul[c] = scale_mul[c] / s1;
    a.black = black_level;
    a.white = white_level;
    a.hl_div = (float)((long long)raw->width * raw->height / 4);

    constexpr size_t kTilesBytes = 256, kTicketOff = 256, kOutOff = 512;
    GLS_CHECK(ensure_scratch(ctx, 1024));
    char* s = (char*)ctx->scratch;
    static_assert(sizeof(AwbTile) * kAwbTiles <= kTilesBytes, "tile results");
    GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(s + kTicketOff, 0, sizeof(unsigned), ctx->stream), "clear ticket"));
    awb_tile_kernel<<<kAwbTiles, kAwbThreads, 0, ctx->stream>>>(a, (AwbTile*)s, (unsigned*)(s + kTicketOff),
                                                                (float*)(s + kOutOff));
    ctx->launches++;
    GLS_CHECK(check_launch(ctx, "autoWhiteBalance"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(ctx->host_pinned, s + kOutOff, 4 * sizeof(float),
                                              cudaMemcpyDeviceToHost, ctx->stream), "copy white balance"));
    GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "synchronize"));
    for (int c = 0; c < 3; c++) wb_out[c] = ctx->host_pinned[c];
    if (highlights) *highlights = ctx->host_pinned[3];
    return GLS_OK;
}
