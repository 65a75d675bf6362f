// gls_internal.h -- host-side internals shared by the translation units of libgls_cuda.
#ifndef GLS_INTERNAL_H
#define GLS_INTERNAL_H

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/gls_cuda.h"

struct gls_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    std::string last_error;
    std::atomic<uint64_t> launches{0};
    // scratch for single-stage regressions
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    float* host_pinned = nullptr;  // small pinned buffer for returning values
};

namespace gls {

gls_status set_error(gls_ctx* ctx, gls_status s, const char* fmt, ...);
gls_status check_cuda(gls_ctx* ctx, cudaError_t e, const char* what);
gls_status check_launch(gls_ctx* ctx, const char* what);
gls_status ensure_scratch(gls_ctx* ctx, size_t bytes);

inline int fmt_channels(int fmt) {
    switch (fmt) {
        case GLS_R16_UNORM:
        case GLS_R_F32:
        case GLS_R_F16: return 1;
        case GLS_RGB8_UNORM: return 3;
        default: return 4;
    }
}

inline int fmt_bytes(int fmt) {
    switch (fmt) {
        case GLS_R16_UNORM: return 2;
        case GLS_R_F32: return 4;
        case GLS_R_F16: return 2;
        case GLS_RGBA_F32: return 16;
        case GLS_RGBA_F16: return 8;
        case GLS_RGBA8_UNORM: return 4;
        case GLS_RGB8_UNORM: return 3;
        default: return 0;
    }
}

inline bool fmt_is_half(int fmt) { return fmt == GLS_R_F16 || fmt == GLS_RGBA_F16; }

// Validates a descriptor: non-null pointer, positive size, pitch a multiple of the pixel
// size and at least one row, and (when fmt >= 0) the expected format.
gls_status check_desc(gls_ctx* ctx, const gls_image_desc* d, const char* name, int fmt0, int fmt1 = -1);

inline int pitch_elems(const gls_image_desc* d) { return d->stride_bytes / fmt_bytes(d->format); }

// Device-side parameter block of a noise-model fit.
struct NlfFit {
    double A[4], B[4], err2[4];
    double N1;  // number of pixels selected by pass 1
    int mode;  // 0 done, 1 needs the explicit error pass, 2 needs the refit pass
    int pad;
};

// Scratch layout for one regression.  The header holds the fit state, the block ticket and
// the running totals of passes 1 and 3, which every block adds its own sums to with integer
// atomics (exact, so in any order): per column three 64-bit limbs of the 128-bit fixed-point
// total, the pass-1 extremes as order-preserving words (atomic maximum; zero is the identity)
// and the NaN mask.  Pass 2 keeps per-block FP64 rows.  The header must be zero before a
// pass starts; the last block of every pass leaves it at zero (the fit state aside).
constexpr int kNlfMaxBlocks = 1024;
constexpr int kNlfK = 1 + 5 * 4;   // N + 5 sums x 4 channels
constexpr int kNlfKF = 4 * 4;      // min/max of m and v per channel
constexpr size_t kNlfTicketOff = 128;
constexpr size_t kNlfLimbOff = 256;                                  // [kNlfK][3] u64
constexpr size_t kNlfMmOff = kNlfLimbOff + 8 * 3 * (size_t)kNlfK;    // [kNlfKF] u32
constexpr size_t kNlfNanOff = kNlfMmOff + 4 * (size_t)kNlfKF;        // u32
constexpr size_t kNlfErrOff = kNlfNanOff + 4;                        // u32
constexpr size_t kNlfProbeOff = kNlfErrOff + 4;                      // u32, never written (wait probe)
constexpr size_t kNlfHeaderBytes = 1024;
constexpr size_t kNlfPartDBytes = sizeof(double) * (size_t)kNlfMaxBlocks * kNlfK;
constexpr size_t kNlfScratchBytes = kNlfHeaderBytes + kNlfPartDBytes;
static_assert(sizeof(NlfFit) <= kNlfTicketOff, "fit state overlaps the ticket");
static_assert(kNlfProbeOff + 4 <= kNlfHeaderBytes, "totals overflow the header");

struct NlfScratch {
    NlfFit* fit;
    unsigned* ticket;              // blocks of the current pass that have added their sums
    unsigned long long* tot_limb;  // [kNlfK][3]: bits 0-39, 40-79, and 80-127 (signed) of each block's sum
    unsigned* tot_mm;              // a fit of NC channels: [0, 2 NC) ~ord(minimum), [2 NC, 4 NC) ord(maximum)
    unsigned* tot_nan;             // bit k set when column k summed a NaN
    unsigned* err;                 // nonzero once a bounded wait of a statistics kernel ran out
    double* part_d;                // [block][kNlfK], pass 2
};

inline NlfScratch nlf_scratch_at(void* base) {
    char* p = reinterpret_cast<char*>(base);
    NlfScratch s;
    s.fit = reinterpret_cast<NlfFit*>(p);
    s.ticket = reinterpret_cast<unsigned*>(p + kNlfTicketOff);
    s.tot_limb = reinterpret_cast<unsigned long long*>(p + kNlfLimbOff);
    s.tot_mm = reinterpret_cast<unsigned*>(p + kNlfMmOff);
    s.tot_nan = reinterpret_cast<unsigned*>(p + kNlfNanOff);
    s.err = reinterpret_cast<unsigned*>(p + kNlfErrOff);
    s.part_d = reinterpret_cast<double*>(p + kNlfHeaderBytes);
    return s;
}

// Thresholds of computeNoiseStatistics (pyramidal_denoise.cpp:166-170) as the float
// bounds that select exactly the same fp32 statistics as the fp64 comparisons.
struct NlfThresholds {
    float m_lo, m_hi, v_lo, v_hi;
};
NlfThresholds nlf_thresholds();

// Launchers of the regression (k_nlf.cu).  Raw: statistics of 2x2 quads of a scaled raw
// image (fp32/fp16) or computed on the fly from uint16 raw; level: statistics of an RGBA
// image.  The fitted {A.., B..} floats are written to out_dev (8 or 6 floats).
// half_stats: the statistics rounded to binary16 before the fit (GLS_STORAGE_F16_STATS)
gls_status nlf_fit_raw_scaled(gls_ctx* ctx, const void* scaled, bool half, int w, int h, int pitch, int bayer,
                              NlfScratch s, float* out_dev, bool half_stats = false);
gls_status nlf_fit_raw_u16(gls_ctx* ctx, const uint16_t* raw, int w, int h, int pitch, int bayer,
                           const float scale_mul[4], float black, bool half_storage, NlfScratch s, float* out_dev,
                           bool half_stats = false);
gls_status nlf_fit_level(gls_ctx* ctx, const void* img, bool half, int w, int h, int pitch, NlfScratch s,
                         float* out_dev, bool half_stats = false);

}  // namespace gls

#define GLS_CHECK(expr)                 \
    do {                                \
        gls_status _s = (expr);         \
        if (_s != GLS_OK) return _s;    \
    } while (0)

#endif  // GLS_INTERNAL_H
