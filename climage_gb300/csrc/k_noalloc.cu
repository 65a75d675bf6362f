// k_noalloc.cu -- GuidedFilter::filter over a scratch area that is part of the library image.
//
// gls_guided_filter takes its ten intermediate images (box-blurred means, products, inverse
// covariances, transposed temporaries) from the context's scratch, which grows by
// cudaFree + cudaMalloc whenever a larger image arrives.  gls_guided_filter_noalloc runs the
// same launches over a fixed static device array instead, so a call allocates nothing.
//
// The array lives in this translation unit alone.  Under CUDA's lazy module loading (the
// default since CUDA 12.2) its module, and with it the 16 MiB, is loaded on a device only
// when the first call on that device looks up its address; with CUDA_MODULE_LOADING=EAGER
// every context on every device reserves the 16 MiB when it is created, whether or not
// this entry point is ever called.
//
// The address is kept per device together with the identity of the CUDA context it was
// looked up in (cuCtxGetId, resolved through the runtime's driver entry points).  A device
// reset (cudaDeviceReset) or a new primary context makes a new context with a new id, and
// the next call looks the address up again instead of using one from the old context.
#include <cuda.h>

#include <mutex>

#include "gls_internal.h"
#include "gls_scratch_slot.h"
#include "gls_stages.h"

namespace gls {
namespace {

// The scratch: room for the guided filter of an image of up to
// GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS pixels (n * 144 bytes + 256-byte alignment padding of
// each of the ten buffers).
static __device__ __align__(256) unsigned char g_guided_scratch[GLS_GUIDED_FILTER_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;

std::mutex g_setup_mu;
ScratchSlot g_slots[kMaxDevices];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// cuCtxGetCurrent / cuCtxGetId from the driver the runtime uses (no link to libcuda)
bool driver_ctx_fns(CtxGetCurrentFn* cur, CtxGetIdFn* id) {
    static CtxGetCurrentFn s_cur = nullptr;
    static CtxGetIdFn s_id = nullptr;
    static bool s_tried = false;
    if (!s_tried) {
        s_tried = true;
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q0 == cudaDriverEntryPointSuccess && q1 == cudaDriverEntryPointSuccess) {
            s_cur = reinterpret_cast<CtxGetCurrentFn>(f0);
            s_id = reinterpret_cast<CtxGetIdFn>(f1);
        } else {
            cudaGetLastError();
        }
    }
    *cur = s_cur;
    *id = s_id;
    return s_cur && s_id;
}

// id of the context current on this thread (0 when none is current)
unsigned long long current_ctx_id(CtxGetCurrentFn cur, CtxGetIdFn id) {
    CUcontext c = nullptr;
    unsigned long long v = 0;
    if (cur(&c) != CUDA_SUCCESS || !c || id(c, &v) != CUDA_SUCCESS) return 0;
    return v;
}

// Address of the array in the context current on the context's device: looked up once per
// device and context (the set-up), reused while that context lives.
gls_status static_scratch(gls_ctx* ctx, void** out) {
    int dev = -1;
    GLS_CHECK(check_cuda(ctx, cudaGetDevice(&dev), "cudaGetDevice"));
    if (dev != ctx->device)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT,
                         "guidedFilter (no allocation): device %d is current, the context's device %d must be", dev,
                         ctx->device);
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(ctx, GLS_ERR_UNSUPPORTED, "guidedFilter (no allocation): device %d >= %d", dev, kMaxDevices);
    CtxGetCurrentFn cur;
    CtxGetIdFn idf;
    if (!driver_ctx_fns(&cur, &idf))
        return set_error(ctx, GLS_ERR_UNSUPPORTED,
                         "guidedFilter (no allocation): the driver offers no cuCtxGetCurrent/cuCtxGetId");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    gls_status st = GLS_OK;
    void* p = scratch_slot_get(g_slots[dev], current_ctx_id(cur, idf), [&](unsigned long long* id) -> void* {
        void* q = nullptr;
        // binds (and if need be creates) the device's primary context, loads the array there
        st = check_cuda(ctx, cudaGetSymbolAddress(&q, g_guided_scratch),
                        "cudaGetSymbolAddress(guided filter static scratch)");
        if (st != GLS_OK) return nullptr;
        *id = current_ctx_id(cur, idf);
        if (*id == 0) st = set_error(ctx, GLS_ERR_CUDA, "guidedFilter (no allocation): no CUDA context is current");
        return q;
    });
    if (!p) return st != GLS_OK ? st : set_error(ctx, GLS_ERR_CUDA, "guidedFilter (no allocation): no scratch address");
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
