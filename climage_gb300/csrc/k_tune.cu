// k_tune.cu -- the process-wide cache of tuned launch shapes and its C API.
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "gls_tune.h"

namespace gls {
namespace {

struct Entry {
    int shape;
    float ms[kTuneMaxShapes];
};

struct Cache {
    std::mutex mu;
    std::map<std::tuple<int, int, int, int>, Entry> choice;
    int forced[kTuneKernels] = {-1, -1};
};

Cache& cache() {
    static Cache c;
    return c;
}

std::tuple<int, int, int, int> key_of(const TuneKey& k) { return std::make_tuple(k.kernel, k.w, k.h, k.flags); }

}  // namespace

int tune_lookup(const TuneKey& key) {
    if (key.kernel < 0 || key.kernel >= kTuneKernels) return 0;
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    if (c.forced[key.kernel] >= 0) return c.forced[key.kernel];
    auto it = c.choice.find(key_of(key));
    return it == c.choice.end() ? -1 : it->second.shape;
}

void tune_store(const TuneKey& key, int shape, const float* ms) {
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    Entry e{};
    e.shape = shape;
    for (int v = 0; v < kTuneMaxShapes; v++) e.ms[v] = v < kTuneShapes[key.kernel] ? ms[v] : 0.0f;
    c.choice[key_of(key)] = e;
}

bool tune_can_time(gls_ctx* ctx) {
    static const bool enabled = [] {
        const char* e = std::getenv("GLS_TUNE");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    if (!enabled) return false;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &st) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return st == cudaStreamCaptureStatusNone;
}

}  // namespace gls

using namespace gls;

extern "C" {

gls_status gls_tune_force(int kernel, int shape) {
    if (kernel < 0 || kernel >= kTuneKernels || shape < -1 || shape >= kTuneShapes[kernel])
        return GLS_ERR_INVALID_ARGUMENT;
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    c.forced[kernel] = shape;
    return GLS_OK;
}

gls_status gls_tune_reset(void) {
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    c.choice.clear();
    for (int k = 0; k < kTuneKernels; k++) c.forced[k] = -1;
    return GLS_OK;
}

int gls_tune_count(void) {
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    return (int)c.choice.size();
}

gls_status gls_tune_entry(int index, int* kernel, int* width, int* height, int* flags, int* shape, float ms[4]) {
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    if (index < 0 || index >= (int)c.choice.size()) return GLS_ERR_INVALID_ARGUMENT;
    auto it = c.choice.begin();
    std::advance(it, index);
    if (kernel) *kernel = std::get<0>(it->first);
    if (width) *width = std::get<1>(it->first);
    if (height) *height = std::get<2>(it->first);
    if (flags) *flags = std::get<3>(it->first);
    if (shape) *shape = it->second.shape;
    if (ms)
        for (int v = 0; v < 4; v++) ms[v] = it->second.ms[v];
    return GLS_OK;
}

}  // extern "C"
