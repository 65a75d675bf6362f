// gls_tune.h -- choice among the compiled launch shapes of a kernel, per frame size.
//
// Some kernels are compiled for several tile shapes; every shape computes the same values
// (a tile only decides which block computes a pixel), and which one is fastest depends on
// the frame: small frames want more, smaller blocks to fill the 152 SMs, large frames the
// shape with the least halo.  On the first frame of a size the converter launches every
// shape of the kernel on that frame's own data, times them with CUDA events on its stream,
// and keeps the fastest for the process; later frames of the size launch that shape
// directly (another shape replaces the default only when it is 3 % faster, best of three
// timings each).  Nothing is timed while a stream is being captured into a graph (the default
// shape runs until a non-captured frame has tuned the size) or when GLS_TUNE=0 is set in the
// environment; gls_tune_force() pins a shape (tests compare every shape's output).
//
// The reference's counterpart is its work-group sizer (src/gls_cl.cpp:227-261,
// computeWorkGroupSizes), which picks an OpenCL local size per launch from fixed rules.
#ifndef GLS_TUNE_H
#define GLS_TUNE_H

#include <cuda_runtime.h>

#include "gls_internal.h"

namespace gls {

enum TuneKernel { kTuneDemosaic = 0, kTuneFinal = 1, kTuneKernels = 2 };
constexpr int kTuneMaxShapes = 4;
constexpr int kTuneShapes[kTuneKernels] = {4, 3};

struct TuneKey {
    int kernel, w, h, flags;  // flags: the kernel's variant bits (storage, input form, ...)
};

// The cached or forced shape for key, or -1.
int tune_lookup(const TuneKey& key);
// Records the timed choice (ms[v]: the best time of shape v).
void tune_store(const TuneKey& key, int shape, const float* ms);
// Whether shapes may be timed now on ctx's stream (tuning on, stream not capturing).
bool tune_can_time(gls_ctx* ctx);

// The shape to launch for key.  run(v) launches shape v on ctx->stream; every shape writes
// the same outputs from the same inputs, so timing them on the frame's data is harmless.
template <class F>
int tune_choose(gls_ctx* ctx, const TuneKey& key, F&& run) {
    const int known = tune_lookup(key);
    if (known >= 0) return known;
    if (!tune_can_time(ctx)) return 0;
    const int n = kTuneShapes[key.kernel];
    cudaEvent_t ev[kTuneMaxShapes + 1] = {};
    const int nev = n + 1;  // ev[v] .. ev[v + 1] brackets shape v
    for (int i = 0; i < nev; i++) {
        if (cudaEventCreate(&ev[i]) != cudaSuccess) {
            for (int j = 0; j < i; j++) cudaEventDestroy(ev[j]);
            cudaGetLastError();
            return 0;
        }
    }
    float best[kTuneMaxShapes];
    for (int v = 0; v < n; v++) {
        best[v] = 3.4e38f;
        run(v);  // first launch of each shape untimed
    }
    bool ok = true;
    for (int round = 0; round < 3 && ok; round++) {
        cudaEventRecord(ev[0], ctx->stream);
        for (int v = 0; v < n; v++) {
            run(v);
            cudaEventRecord(ev[1 + v], ctx->stream);
        }
        ok = cudaEventSynchronize(ev[n]) == cudaSuccess;
        for (int v = 0; v < n && ok; v++) {
            float ms = 0.0f;
            ok = cudaEventElapsedTime(&ms, ev[v], ev[1 + v]) == cudaSuccess;
            if (ok && ms < best[v]) best[v] = ms;
        }
    }
    for (int i = 0; i < nev; i++) cudaEventDestroy(ev[i]);
    if (!ok) return 0;  // a launch or event error: the caller's launch reports it
    // another shape must beat the default by 3 % (timings on a busy GPU carry a few % of
    // noise, and the default is the shape measured best on the bench's frames)
    int choice = 0;
    for (int v = 1; v < n; v++)
        if (best[v] < 0.97f * best[0] && best[v] < best[choice]) choice = v;
    tune_store(key, choice, best);
    return choice;
}

}  // namespace gls

#endif  // GLS_TUNE_H
