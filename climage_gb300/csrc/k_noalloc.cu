// k_noalloc.cu -- GuidedFilter::filter over a scratch area that is part of the library image.
//
// gls_guided_filter takes its ten intermediate images (box-blurred means, products, inverse
// covariances, transposed temporaries) from the context's scratch, which grows by
// cudaFree + cudaMalloc whenever a larger image arrives.  gls_guided_filter_noalloc runs the
// same launches over a fixed static device array instead, so a call allocates nothing.
//
// The array lives in this translation unit alone: its module, and with it the 16 MiB, is
// loaded on a device only when the first call on that device looks up its address.
#include <mutex>

#include "gls_internal.h"
#include "gls_stages.h"

namespace gls {
namespace {

// The scratch: room for the guided filter of an image of up to
// GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS pixels (n * 144 bytes + 256-byte alignment padding of
// each of the ten buffers).
static __device__ __align__(256) unsigned char g_guided_scratch[GLS_GUIDED_FILTER_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
std::atomic<void*> g_scratch_ptr[kMaxDevices];

// Address of the array on the current device, looked up once per device.
gls_status static_scratch(gls_ctx* ctx, void** out) {
    int dev = -1;
    GLS_CHECK(check_cuda(ctx, cudaGetDevice(&dev), "cudaGetDevice"));
    if (dev != ctx->device)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT,
                         "guidedFilter (no allocation): device %d is current, the context's device %d must be", dev,
                         ctx->device);
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(ctx, GLS_ERR_UNSUPPORTED, "guidedFilter (no allocation): device %d >= %d", dev, kMaxDevices);
    void* p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lock(g_setup_mu);
        p = g_scratch_ptr[dev].load(std::memory_order_relaxed);
        if (!p) {
            GLS_CHECK(check_cuda(ctx, cudaGetSymbolAddress(&p, g_guided_scratch),
                                 "cudaGetSymbolAddress(guided filter static scratch)"));
            g_scratch_ptr[dev].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return GLS_OK;
}

}  // namespace
}  // namespace gls

using namespace gls;

extern "C" gls_status gls_guided_filter_noalloc(gls_ctx* ctx, const gls_image_desc* in, int filter_size,
                                                const float eps[3], const gls_image_desc* out) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    GLS_CHECK(check_desc(ctx, in, "in", GLS_RGBA_F32, GLS_RGBA_F16));
    GLS_CHECK(check_desc(ctx, out, "out", GLS_RGBA_F32, GLS_RGBA_F16));
    if (in->width != out->width || in->height != out->height)
        return set_error(ctx, GLS_ERR_INVALID_SIZE, "GuidedFilter::filter: image sizes differ");
    if (fmt_is_half(in->format) != fmt_is_half(out->format))
        return set_error(ctx, GLS_ERR_FORMAT, "GuidedFilter::filter: storage precisions differ");
    if (!eps) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "eps is null");
    if (filter_size < 1) return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "filter_size must be >= 1");
    const long long pixels = (long long)in->width * in->height;
    const size_t need = guided_filter_scratch_bytes(in->width, in->height);
    if (pixels > GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS || need > sizeof(g_guided_scratch))
        return set_error(ctx, GLS_ERR_INVALID_SIZE,
                         "guidedFilter (no allocation): a %dx%d image (%lld pixels) needs %zu bytes of scratch; the "
                         "static scratch holds %zu bytes, at most %d pixels",
                         in->width, in->height, pixels, need, sizeof(g_guided_scratch),
                         (int)GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS);
    void* scratch = nullptr;
    GLS_CHECK(static_scratch(ctx, &scratch));
    // every buffer in the scratch is written in full before it is read: nothing to clear
    NlfArg e;
    e.dev = nullptr;
    for (int k = 0; k < 3; k++) {
        e.host[k] = 0.0f;
        e.host[3 + k] = eps[k];
    }
    for (int k = 0; k < 6; k++) e.mul[k] = 1.0f;
    const ImgRef ri{in->ptr, in->width, in->height, pitch_elems(in), fmt_is_half(in->format)};
    const ImgRef ro{out->ptr, out->width, out->height, pitch_elems(out), fmt_is_half(out->format)};
    launch_guided_filter(ctx, ri, ro, filter_size, e, scratch);
    return check_launch(ctx, "GuidedFilter::filter (no allocation)");
}
