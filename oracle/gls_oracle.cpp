// gls_oracle.cpp -- CPU restatement of CLImage's RAW->RGB pipeline.
//
// TEST INFRASTRUCTURE ONLY (the checker): loaded by tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg, never by the product.  Every function follows the
// reference file:line named in its comment, statement by statement and in the same
// operation order, with these conventions for behaviour OpenCL leaves undefined:
//   * sampler-less image reads outside the image clamp to the edge;
//   * the linear sampler (normalised coordinates, CLAMP_TO_EDGE) computes its
//     interpolation fractions in float and quantises them to 8 fractional bits, as
//     texture units do, then blends the four texels in float;
//   * UNORM16 reads divide by 65535, UNORM8 writes saturate and round to nearest even,
//     fp16 image writes round to nearest even;
//   * built-ins (atan2pi, tanh, pow, smoothstep, ...) come from gls_clmath.h.
// The FP64 policy runs the same code in double without any fp16 rounding and with the
// platform libm: it is the error oracle for every result.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off, no -march flags).
#include "gls_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "../climage_gb300/csrc/gls_clmath.h"

namespace {

// ---------------------------------------------------------------------------------------
// Threading: rows are split into contiguous chunks, one per worker.
// ---------------------------------------------------------------------------------------
int g_threads = 0;

int num_threads() {
    if (g_threads > 0) return g_threads;
    const char* env = std::getenv("GLS_ORACLE_THREADS");
    if (env && std::atoi(env) > 0) return std::atoi(env);
    unsigned n = std::thread::hardware_concurrency();
    return n ? (int)n : 1;
}

void parallel_rows(int rows, const std::function<void(int, int)>& fn) {
    const int nt = std::min(num_threads(), std::max(rows, 1));
    if (nt <= 1 || rows < 64) {
        fn(0, rows);
        return;
    }
    std::vector<std::thread> pool;
    const int chunk = (rows + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        const int r0 = t * chunk, r1 = std::min(rows, r0 + chunk);
        if (r0 >= r1) break;
        pool.emplace_back([=, &fn] { fn(r0, r1); });
    }
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------------------
// Math policy: float uses the pinned OpenCL built-ins, double uses libm.
// ---------------------------------------------------------------------------------------
template <class C>
struct M;

template <>
struct M<float> {
    static float sqrt(float x) { return glsm::sqrt_(x); }
    static float div(float a, float b) { return glsm::div_(a, b); }
    static float atan2pi(float y, float x) { return glsm::atan2pi_(y, x); }
    static float tanh(float x) { return glsm::tanh_(x); }
    static float pow(float x, float y) { return glsm::pow_(x, y); }
    static float powr(float x, float y) { return glsm::powr_(x, y); }
    static float floor(float x) { return glsm::floor_(x); }
    static float fmax(float a, float b) { return glsm::fmax_(a, b); }
    static float fmin(float a, float b) { return glsm::fmin_(a, b); }
    static float fabs(float a) { return glsm::fabs_(a); }
};

template <>
struct M<double> {
    static double sqrt(double x) { return std::sqrt(x); }
    static double div(double a, double b) { return a / b; }
    static double atan2pi(double y, double x) { return std::atan2(y, x) / M_PI; }
    static double tanh(double x) { return std::tanh(x); }
    static double pow(double x, double y) { return std::pow(x, y); }
    static double powr(double x, double y) { return x < 0 ? NAN : std::pow(x, y); }
    static double floor(double x) { return std::floor(x); }
    static double fmax(double a, double b) { return a != a ? b : (b != b ? a : (a < b ? b : a)); }
    static double fmin(double a, double b) { return a != a ? b : (b != b ? a : (b < a ? b : a)); }
    static double fabs(double a) { return std::fabs(a); }
};

template <class C>
C clampc(C x, C lo, C hi) { return M<C>::fmin(M<C>::fmax(x, lo), hi); }
template <class C>
C mixc(C x, C y, C a) { return x + (y - x) * a; }
template <class C>
C smoothstepc(C e0, C e1, C x) {
    C t = clampc<C>(M<C>::div(x - e0, e1 - e0), C(0), C(1));
    return t * t * (C(3) - C(2) * t);
}
// step(edge, x) with NaN x giving 0 (the finite-math reading pinned in gls_clmath.h)
template <class C>
C stepc(C edge, C x) { return x >= edge ? C(1) : C(0); }
template <class C>
C mminc(C a, C b) { return a < b ? a : b; }
template <class C>
C mmaxc(C a, C b) { return a > b ? a : b; }
template <class C>
C mabsc(C a) { return a > 0 ? a : -a; }
template <class C>
C len2(C x, C y) { return M<C>::sqrt(x * x + y * y); }
template <class C>
C len3(C x, C y, C z) { return M<C>::sqrt(x * x + y * y + z * z); }
template <class C>
C len4(C x, C y, C z, C w) { return M<C>::sqrt(x * x + y * y + z * z + w * w); }

// Storage policy: how a value is rounded when written to an intermediate image, and
// how read_imageh converts a value to half.
struct Pol {
    int prec;
    bool half_storage() const { return prec == ORACLE_F16 || prec == ORACLE_F16_STATS; }
    bool half_reads() const { return prec != ORACLE_F64; }
};

template <class C>
C store(const Pol& p, C v) {
    if (p.half_storage()) return (C)glsm::round_half((float)v);
    return v;
}

template <class C>
C half_op(const Pol& p, C v) {
    if (p.half_reads()) return (C)glsm::round_half((float)v);
    return v;
}

// ---------------------------------------------------------------------------------------
// Images
// ---------------------------------------------------------------------------------------
template <class C>
struct Img {
    int w = 0, h = 0, c = 1;
    std::vector<C> d;
    Img() {}
    Img(int w_, int h_, int c_) : w(w_), h(h_), c(c_), d((size_t)w_ * h_ * c_, C(0)) {}
    C at(int x, int y, int k) const {
        x = x < 0 ? 0 : (x >= w ? w - 1 : x);
        y = y < 0 ? 0 : (y >= h ? h - 1 : y);
        return d[((size_t)y * w + x) * c + k];
    }
    C& ref(int x, int y, int k) { return d[((size_t)y * w + x) * c + k]; }
};

template <class C>
Img<C> from_float(const float* p, int w, int h, int c) {
    Img<C> im(w, h, c);
    for (size_t i = 0; i < im.d.size(); i++) im.d[i] = (C)p[i];
    return im;
}

template <class C>
void to_float(const Img<C>& im, float* p) {
    for (size_t i = 0; i < im.d.size(); i++) p[i] = (float)im.d[i];
}

// Kernel CFA table, demosaic.cl:29-34 (x, y) per {red, green, blue, green2}.
const int kBayer[4][4][2] = {
    {{1, 0}, {0, 0}, {0, 1}, {1, 1}},  // grbg
    {{0, 1}, {0, 0}, {1, 0}, {1, 1}},  // gbrg
    {{0, 0}, {0, 1}, {1, 1}, {1, 0}},  // rggb
    {{1, 1}, {0, 1}, {0, 0}, {1, 0}},  // bggr
};
enum { raw_red = 0, raw_green = 1, raw_blue = 2, raw_green2 = 3 };
enum { grbg = 0, gbrg = 1, rggb = 2, bggr = 3 };

// Linear sampler, normalised coordinates, CLAMP_TO_EDGE (demosaic_cl.cpp:163).
template <class C>
void sample_linear(const Img<C>& im, C u, C v, C* out) {
    const C fu = u * (C)im.w - C(0.5);
    const C fv = v * (C)im.h - C(0.5);
    const C i0f = M<C>::floor(fu), j0f = M<C>::floor(fv);
    C a = fu - i0f, b = fv - j0f;
    a = M<C>::floor(a * C(256) + C(0.5)) / C(256);
    b = M<C>::floor(b * C(256) + C(0.5)) / C(256);
    const int i0 = (int)i0f, j0 = (int)j0f;
    const C w00 = (C(1) - a) * (C(1) - b), w10 = a * (C(1) - b), w01 = (C(1) - a) * b, w11 = a * b;
    for (int k = 0; k < im.c; k++) {
        out[k] = w00 * im.at(i0, j0, k) + w10 * im.at(i0 + 1, j0, k) + w01 * im.at(i0, j0 + 1, k) +
                 w11 * im.at(i0 + 1, j0 + 1, k);
    }
}

// ---------------------------------------------------------------------------------------
// a4: scaleRawData, demosaic.cl:69-78 (binding demosaic_cl.cpp:26-44)
// ---------------------------------------------------------------------------------------
template <class C>
void scale_raw(const Pol& pol, const uint16_t* raw, int w, int h, int stride, int bayer, const float sm[4],
               float black, Img<C>& out) {
    out = Img<C>(w, h, 1);
    parallel_rows(h / 2, [&](int q0, int q1) {
        for (int qy = q0; qy < q1; qy++) {
            for (int qx = 0; qx < w / 2; qx++) {
                for (int c = 0; c < 4; c++) {
                    const int x = 2 * qx + kBayer[bayer][c][0], y = 2 * qy + kBayer[bayer][c][1];
                    const C v = M<C>::div((C)raw[(size_t)y * stride + x], C(65535));
                    const C r = (C)sm[c] * (v - (C)black);
                    out.ref(x, y, 0) = store(pol, r > C(0) ? r : C(0));
                }
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a5: rawNoiseStatistics + readRAWQuad, demosaic.cl:1288-1324
// ---------------------------------------------------------------------------------------
template <class C>
void raw_noise_statistics(const Img<C>& raw, int bayer, Img<C>& mean, Img<C>& var) {
    const int qw = raw.w / 2, qh = raw.h / 2;
    mean = Img<C>(qw, qh, 4);
    var = Img<C>(qw, qh, 4);
    parallel_rows(qh, [&](int y0, int y1) {
        for (int qy = y0; qy < y1; qy++) {
            for (int qx = 0; qx < qw; qx++) {
                C sum[4] = {0, 0, 0, 0}, sumSq[4] = {0, 0, 0, 0};
                for (int y = -2; y <= 2; y++) {
                    for (int x = -2; x <= 2; x++) {
                        for (int c = 0; c < 4; c++) {
                            const C s = raw.at(2 * (qx + x) + kBayer[bayer][c][0], 2 * (qy + y) + kBayer[bayer][c][1], 0);
                            sum[c] += s;
                            sumSq[c] += s * s;
                        }
                    }
                }
                for (int c = 0; c < 4; c++) {
                    mean.ref(qx, qy, c) = M<C>::div(sum[c], C(25));
                    var.ref(qx, qy, c) = M<C>::div(sumSq[c] - M<C>::div(sum[c] * sum[c], C(25)), C(25));
                }
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// Noise-model regression: computeNoiseStatistics / computeRawNoiseStatistics,
// pyramidal_denoise.cpp:161-256 and 259-362.  Three passes in FP64: fit, RMS error,
// refit on the pixels whose squared residual is <= the RMS (as the reference compares).
// The sums use compensated (Neumaier) accumulation so the result is the FP64 value of
// the exact sums, independent of summation order.
// ---------------------------------------------------------------------------------------
struct KSum {
    double s = 0, c = 0;
    void add(double x) {
        const double t = s + x;
        if (std::fabs(s) >= std::fabs(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
    }
    double value() const { return s + c; }
};

// The reference's gls::max(DVector, double) is std::max(v, a) == (v < a) ? a : v.
double refmax(double v, double a) { return (v < a) ? a : v; }

// mc: number of mean components (1 = luma mean broadcast, 4 = per CFA plane)
// nc: number of variance components
template <class GetMV>
void regress(long n, int mc, int nc, GetMV get, double* outA, double* outB) {
    const double varianceMax = 0.001, maxValue = 0.5, minValue = 0.001;
    auto in_range = [&](const double* m, const double* v) {
        for (int c = 0; c < mc; c++)
            if (m[c] < minValue || m[c] > maxValue) return false;
        for (int c = 0; c < nc; c++)
            if (v[c] < 0 || v[c] > varianceMax) return false;
        return true;
    };
    auto mof = [&](const double* m, int c) { return mc == 1 ? m[0] : m[c]; };

    KSum sx[4], sy[4], sxx[4], sxy[4];
    double N = 0;
    double m[4], v[4];
    for (long i = 0; i < n; i++) {
        get(i, m, v);
        if (!in_range(m, v)) continue;
        for (int c = 0; c < nc; c++) {
            const double mm = mof(m, c);
            sx[c].add(mm);
            sy[c].add(v[c]);
            sxx[c].add(mm * mm);
            sxy[c].add(mm * v[c]);
        }
        N++;
    }
    double A[4], B[4];
    for (int c = 0; c < nc; c++) {
        B[c] = refmax((N * sxy[c].value() - sx[c].value() * sy[c].value()) /
                          (N * sxx[c].value() - sx[c].value() * sx[c].value()),
                      1e-8);
        A[c] = refmax((sy[c].value() - B[c] * sx[c].value()) / N, 1e-8);
    }
    // Regression mean square error; gls::sqrt(Vector) evaluates sqrtf (gls_linalg.hpp:256-261)
    KSum e2[4];
    for (long i = 0; i < n; i++) {
        get(i, m, v);
        if (!in_range(m, v)) continue;
        for (int c = 0; c < nc; c++) {
            const double diff = (A[c] + B[c] * mof(m, c)) - v[c];
            e2[c].add(diff * diff);
        }
    }
    double err2[4];
    for (int c = 0; c < nc; c++) err2[c] = (double)sqrtf((float)(e2[c].value() / N));

    KSum sx2[4], sy2[4], sxx2[4], sxy2[4];
    double N2 = 0;
    for (long i = 0; i < n; i++) {
        get(i, m, v);
        if (!in_range(m, v)) continue;
        bool ok = true;
        for (int c = 0; c < nc; c++) {
            const double diff = (A[c] + B[c] * mof(m, c)) - v[c];
            if (!(diff * diff <= err2[c])) ok = false;
        }
        if (!ok) continue;
        for (int c = 0; c < nc; c++) {
            const double mm = mof(m, c);
            sx2[c].add(mm);
            sy2[c].add(v[c]);
            sxx2[c].add(mm * mm);
            sxy2[c].add(mm * v[c]);
        }
        N2++;
    }
    for (int c = 0; c < nc; c++) {
        const double b = refmax((N2 * sxy2[c].value() - sx2[c].value() * sy2[c].value()) /
                                    (N2 * sxx2[c].value() - sx2[c].value() * sx2[c].value()),
                                1e-8);
        const double a = refmax((sy2[c].value() - b * sx2[c].value()) / N2, 1e-8);
        outA[c] = a;
        outB[c] = b;
    }
}

// One statistic as the regression reads it: an fp32 value, or the fp16 one an rgba_pixel_float
// image of the shipped build holds (the host converts it to double exactly).
template <class C>
double stat_value(C v, bool half_stats) {
    return half_stats ? (double)glsm::round_half((float)v) : (double)(float)v;
}

template <class C>
void compute_raw_nlf(const Img<C>& scaled, int bayer, float out[8], bool half_stats = false) {
    Img<C> mean, var;
    raw_noise_statistics(scaled, bayer, mean, var);
    const long n = (long)mean.w * mean.h;
    double A[4], B[4];
    regress(n, 4, 4,
            [&](long i, double* m, double* v) {
                for (int c = 0; c < 4; c++) {
                    // statistics are kept in fp32 (the noise-model fit is an fp32 stage), or
                    // in fp16 as the shipped build's meanImage/varImage hold them
                    m[c] = stat_value(mean.d[(size_t)i * 4 + c], half_stats);
                    v[c] = stat_value(var.d[(size_t)i * 4 + c], half_stats);
                }
            },
            A, B);
    for (int c = 0; c < 4; c++) {
        out[c] = (float)A[c];
        out[4 + c] = (float)B[c];
    }
}

// ---------------------------------------------------------------------------------------
// a13: noiseStatistics, demosaic.cl:1267-1286
// ---------------------------------------------------------------------------------------
template <class C>
void noise_statistics(const Img<C>& in, Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int py = y0; py < y1; py++) {
            for (int px = 0; px < in.w; px++) {
                C sum[3] = {0, 0, 0}, sumSq[3] = {0, 0, 0};
                for (int y = -2; y <= 2; y++) {
                    for (int x = -2; x <= 2; x++) {
                        for (int k = 0; k < 3; k++) {
                            const C s = in.at(px + x, py + y, k);
                            sum[k] += s;
                            sumSq[k] += s * s;
                        }
                    }
                }
                C var[3];
                for (int k = 0; k < 3; k++) var[k] = M<C>::div(sumSq[k] - M<C>::div(sum[k] * sum[k], C(25)), C(25));
                out.ref(px, py, 0) = M<C>::div(sum[0], C(25));
                out.ref(px, py, 1) = var[0];
                out.ref(px, py, 2) = var[1];
                out.ref(px, py, 3) = var[2];
            }
        }
    });
}

template <class C>
void compute_nlf(const Img<C>& in, float out[6], bool half_stats = false) {
    Img<C> st;
    noise_statistics(in, st);
    const long n = (long)st.w * st.h;
    double A[4], B[4];
    regress(n, 1, 3,
            [&](long i, double* m, double* v) {
                m[0] = stat_value(st.d[(size_t)i * 4 + 0], half_stats);
                for (int c = 0; c < 3; c++) v[c] = stat_value(st.d[(size_t)i * 4 + 1 + c], half_stats);
            },
            A, B);
    for (int c = 0; c < 3; c++) {
        out[c] = (float)A[c];
        out[3 + c] = (float)B[c];
    }
}

// ---------------------------------------------------------------------------------------
// a6: high-noise raw branch, demosaic.cl:898-949, 530-553, 1187-1201
// ---------------------------------------------------------------------------------------
template <class C>
void bayer_to_rgba(const Pol& pol, const Img<C>& raw, int bayer, Img<C>& out) {
    out = Img<C>(raw.w / 2, raw.h / 2, 4);
    for (int qy = 0; qy < out.h; qy++)
        for (int qx = 0; qx < out.w; qx++)
            for (int c = 0; c < 4; c++)
                out.ref(qx, qy, c) = store(pol, raw.at(2 * qx + kBayer[bayer][c][0], 2 * qy + kBayer[bayer][c][1], 0));
}

template <class C>
void rgba_to_bayer(const Pol& pol, const Img<C>& rgba, int bayer, Img<C>& raw) {
    for (int qy = 0; qy < rgba.h; qy++)
        for (int qx = 0; qx < rgba.w; qx++)
            for (int c = 0; c < 4; c++)
                raw.ref(2 * qx + kBayer[bayer][c][0], 2 * qy + kBayer[bayer][c][1], 0) = store(pol, rgba.at(qx, qy, c));
}

template <class C>
void despeckle_rgba(const Pol& pol, const Img<C>& in, Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int py = y0; py < y1; py++) {
            for (int px = 0; px < in.w; px++) {
                for (int k = 0; k < 4; k++) {
                    C sample = 0, firstMax = 0, secMax = 0;
                    C firstMin = C(65535), secMin = C(65535);
                    for (int x = -1; x <= 1; x++) {
                        for (int y = -1; y <= 1; y++) {
                            const C v = in.at(px + x, py + y, k);
                            secMax = (v <= firstMax && v > secMax) ? v : secMax;
                            secMax = v > firstMax ? firstMax : secMax;
                            firstMax = v > firstMax ? v : firstMax;
                            secMin = (v >= firstMin && v < secMin) ? v : secMin;
                            secMin = v < firstMin ? firstMin : secMin;
                            firstMin = v < firstMin ? v : firstMin;
                            if (x == 0 && y == 0) sample = v;
                        }
                    }
                    out.ref(px, py, k) = store(pol, clampc<C>(sample, secMin, secMax));
                }
            }
        }
    });
}

template <class C>
void denoise_rgba(const Pol& pol, const Img<C>& in, const float rv[4], Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int py = y0; py < y1; py++) {
            for (int px = 0; px < in.w; px++) {
                C input[4], sigma[4], filtered[4] = {0, 0, 0, 0}, norm[4] = {0, 0, 0, 0};
                for (int k = 0; k < 4; k++) {
                    input[k] = in.at(px, py, k);
                    sigma[k] = M<C>::sqrt((C)rv[k] * input[k]);
                }
                for (int y = -2; y <= 2; y++) {
                    for (int x = -2; x <= 2; x++) {
                        C s[4], d[4];
                        for (int k = 0; k < 4; k++) {
                            s[k] = in.at(px + x, py + y, k);
                            d[k] = M<C>::div(s[k] - input[k], sigma[k]);
                        }
                        const C wgt = C(1) - stepc<C>(C(1), len4<C>(d[0], d[1], d[2], d[3]));
                        for (int k = 0; k < 4; k++) {
                            filtered[k] += wgt * s[k];
                            norm[k] += wgt;
                        }
                    }
                }
                for (int k = 0; k < 4; k++) out.ref(px, py, k) = store(pol, M<C>::div(filtered[k], norm[k]));
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a7: interpolateGreen + sobel + bilateralSobel, demosaic.cl:96-129, 160-227
// ---------------------------------------------------------------------------------------
template <class C>
void sobel(const Img<C>& im, int x, int y, C* gx, C* gy) {
    static const int kx[3][3] = {{1, 0, -1}, {2, 0, -2}, {1, 0, -1}};
    static const int ky[3][3] = {{1, 2, 1}, {0, 0, 0}, {-1, -2, -1}};
    C vx = 0, vy = 0;
    for (int j = -1; j <= 1; j++) {
        for (int i = -1; i <= 1; i++) {
            const C s = im.at(x + i, y + j, 0);
            vx += (C)kx[j + 1][i + 1] * s;
            vy += (C)ky[j + 1][i + 1] * s;
        }
    }
    const C r = M<C>::sqrt(C(4.5));
    *gx = M<C>::div(vx, r);
    *gy = M<C>::div(vy, r);
}

template <class C>
void bilateral_sobel(const Img<C>& im, int x, int y, C sigma, C* outx, C* outy) {
    C sx = 0, sy = 0, wx = 0, wy = 0;
    C cgx, cgy;
    sobel(im, x, y, &cgx, &cgy);
    cgx = mabsc(cgx);
    cgy = mabsc(cgy);
    const C lc = len2<C>(cgx, cgy);
    for (int j = -2; j <= 2; j++) {
        for (int i = -2; i <= 2; i++) {
            C gx, gy;
            sobel(im, x + i, y + j, &gx, &gy);
            gx = mabsc(gx);
            gy = mabsc(gy);
            const C w = C(1) - smoothstepc<C>(C(4) * sigma, C(16) * sigma, C(0.05) * mabsc(len2<C>(gx, gy) - lc));
            sx += w * gx;
            sy += w * gy;
            wx += w;
            wy += w;
        }
    }
    *outx = M<C>::div(sx, wx);
    *outy = M<C>::div(sy, wy);
}

template <class C>
void interpolate_green(const Pol& pol, const Img<C>& raw, int bayer, float lumaVariance_, Img<C>& green) {
    green = Img<C>(raw.w, raw.h, 1);
    const C lumaVariance = mmaxc<C>((C)lumaVariance_, C(1e-4));
    const int gx0 = kBayer[bayer][raw_green][0], gy0 = kBayer[bayer][raw_green][1];
    const C SQRT2 = sizeof(C) == 4 ? (C)1.41421356237309504880f : (C)1.41421356237309504880;
    parallel_rows(raw.h, [&](int r0, int r1) {
        for (int y = r0; y < r1; y++) {
            const int x0 = (y & 1) == (gy0 & 1) ? gx0 + 1 : gx0;
            for (int x = 0; x < raw.w; x++) {
                if ((x0 & 1) != (x & 1)) {
                    green.ref(x, y, 0) = store(pol, raw.at(x, y, 0));
                    continue;
                }
                const C g_left = raw.at(x - 1, y, 0), g_right = raw.at(x + 1, y, 0);
                const C g_up = raw.at(x, y - 1, 0), g_down = raw.at(x, y + 1, 0);
                const C c_xy = raw.at(x, y, 0);
                const C c_left = raw.at(x - 2, y, 0), c_right = raw.at(x + 2, y, 0);
                const C c_up = raw.at(x, y - 2, 0), c_down = raw.at(x, y + 2, 0);
                const C c2_tl = raw.at(x - 1, y - 1, 0), c2_tr = raw.at(x + 1, y - 1, 0);
                const C c2_bl = raw.at(x - 1, y + 1, 0), c2_br = raw.at(x + 1, y + 1, 0);
                const C c2_ave = M<C>::div(c2_tl + c2_tr + c2_bl + c2_br, C(4));

                const C g_ave = M<C>::div(g_left + g_right + g_up + g_down, C(4));
                const C lumaStdDev = M<C>::sqrt(lumaVariance * g_ave);
                C gradx, grady;
                bilateral_sobel(raw, x, y, lumaStdDev, &gradx, &grady);

                const C g_lf_x = M<C>::div(g_left + g_right, C(2)), g_lf_y = M<C>::div(g_up + g_down, C(2));
                const C g_hf_x = M<C>::div(C(2) * c_xy - (c_left + c_right), C(4));
                const C g_hf_y = M<C>::div(C(2) * c_xy - (c_up + c_down), C(4));

                const C whiteness = clampc<C>(M<C>::div(mminc<C>(c_xy, mminc<C>(g_ave, c2_ave)),
                                                        mmaxc<C>(c_xy, mmaxc<C>(g_ave, c2_ave))),
                                              C(0), C(1));
                const C glen = len2<C>(gradx, grady);
                const C lgt = smoothstepc<C>(lumaStdDev, C(4) * lumaStdDev, glen);
                const C hf_gain = lgt * mminc<C>(C(0.5) * whiteness + smoothstepc<C>(C(0), C(0.3), M<C>::div(glen, SQRT2)), C(1));
                const C g_est_x = g_lf_x + hf_gain * g_hf_x;
                const C g_est_y = g_lf_y + hf_gain * g_hf_y;

                C direction = C(2) * M<C>::atan2pi(grady, gradx);
                direction = direction < C(0.5)
                                ? mixc<C>(direction, C(0), C(1) - smoothstepc<C>(C(0.3) * lgt, C(0.45) * lgt, direction))
                                : mixc<C>(direction, C(1),
                                          smoothstepc<C>((C(1) - C(0.45)) * lgt, (C(1) - C(0.3)) * lgt, direction));
                direction = mixc<C>(C(0.5), direction, lgt);
                green.ref(x, y, 0) = store(pol, mixc<C>(g_est_y, g_est_x, direction));
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a8: interpolateRedBlue, demosaic.cl:229-318.  With rotate_180 the pixel (x, y) is written
// at (w - x, h - y) (demosaic.cl:310-313): the writes of column 0 and row 0 fall outside the
// image, and output column 0 and row 0 are never written -- they keep the image's initial
// contents, zero here (the convention the CUDA path follows).
// ---------------------------------------------------------------------------------------
template <class C>
void interpolate_red_blue(const Pol& pol, const Img<C>& raw, const Img<C>& gi, int bayer, float chromaVariance_,
                          Img<C>& rgb, bool rotate_180 = false) {
    rgb = Img<C>(raw.w, raw.h, 4);
    const C chromaVariance = mmaxc<C>((C)chromaVariance_, C(1e-6));
    const int rx = kBayer[bayer][raw_red][0], ry = kBayer[bayer][raw_red][1];
    const int gx = kBayer[bayer][raw_green][0], gy = kBayer[bayer][raw_green][1];
    const int bx = kBayer[bayer][raw_blue][0], by = kBayer[bayer][raw_blue][1];
    const int green_is_red_row = (bayer == bggr || bayer == grbg) ? raw_green : raw_green2;
    parallel_rows(raw.h, [&](int r0, int r1) {
        for (int y = r0; y < r1; y++) {
            for (int x = 0; x < raw.w; x++) {
                const int color = ((rx & 1) == (x & 1) && (ry & 1) == (y & 1))   ? raw_red
                                  : ((gx & 1) == (x & 1) && (gy & 1) == (y & 1)) ? raw_green
                                  : ((bx & 1) == (x & 1) && (by & 1) == (y & 1)) ? raw_blue
                                                                                 : raw_green2;
                const C green = gi.at(x, y, 0);
                C red = 0, blue = 0;
                if (color == raw_red || color == raw_blue) {
                    const C c1 = raw.at(x, y, 0);
                    const C g_tl = gi.at(x - 1, y - 1, 0), g_tr = gi.at(x + 1, y - 1, 0);
                    const C g_bl = gi.at(x - 1, y + 1, 0), g_br = gi.at(x + 1, y + 1, 0);
                    const C c2_tl = g_tl - raw.at(x - 1, y - 1, 0), c2_tr = g_tr - raw.at(x + 1, y - 1, 0);
                    const C c2_bl = g_bl - raw.at(x - 1, y + 1, 0), c2_br = g_br - raw.at(x + 1, y + 1, 0);
                    const C chromaStdDev = M<C>::sqrt(chromaVariance * green);
                    const C dvx = M<C>::fabs(c2_tl - c2_br), dvy = M<C>::fabs(c2_tr - c2_bl);
                    const C flatness = C(1) - smoothstepc<C>(C(0.25) * chromaStdDev, chromaStdDev, len2<C>(dvx, dvy));
                    const C alpha = mixc<C>(C(2) * M<C>::atan2pi(dvy, dvx), C(0.5), flatness);
                    const C c2 = green - mixc<C>(M<C>::div(c2_tr + c2_bl, C(2)), M<C>::div(c2_tl + c2_br, C(2)), alpha);
                    if (color == raw_red) {
                        red = c1;
                        blue = c2;
                    } else {
                        blue = c1;
                        red = c2;
                    }
                } else {
                    const C g_left = gi.at(x - 1, y, 0), g_right = gi.at(x + 1, y, 0);
                    const C g_up = gi.at(x, y - 1, 0), g_down = gi.at(x, y + 1, 0);
                    const C c1_left = g_left - raw.at(x - 1, y, 0), c1_right = g_right - raw.at(x + 1, y, 0);
                    const C c2_up = g_up - raw.at(x, y - 1, 0), c2_down = g_down - raw.at(x, y + 1, 0);
                    const C c1 = green - M<C>::div(c1_left + c1_right, C(2));
                    const C c2 = green - M<C>::div(c2_up + c2_down, C(2));
                    if (color == green_is_red_row) {
                        red = c1;
                        blue = c2;
                    } else {
                        blue = c1;
                        red = c2;
                    }
                }
                const int ox = rotate_180 ? raw.w - x : x, oy = rotate_180 ? raw.h - y : y;
                if (ox >= raw.w || oy >= raw.h) continue;  // the dropped writes of the rotation
                rgb.ref(ox, oy, 0) = store(pol, red);
                rgb.ref(ox, oy, 1) = store(pol, green);
                rgb.ref(ox, oy, 2) = store(pol, blue);
                rgb.ref(ox, oy, 3) = C(0);
            }
        }
    });
}

// a-extra: fastDebayer, demosaic.cl:320-334
template <class C>
void fast_debayer(const Pol& pol, const Img<C>& raw, int bayer, Img<C>& out) {
    out = Img<C>(raw.w / 2, raw.h / 2, 4);
    for (int qy = 0; qy < out.h; qy++) {
        for (int qx = 0; qx < out.w; qx++) {
            const C r = raw.at(2 * qx + kBayer[bayer][0][0], 2 * qy + kBayer[bayer][0][1], 0);
            const C g = raw.at(2 * qx + kBayer[bayer][1][0], 2 * qy + kBayer[bayer][1][1], 0);
            const C b = raw.at(2 * qx + kBayer[bayer][2][0], 2 * qy + kBayer[bayer][2][1], 0);
            const C g2 = raw.at(2 * qx + kBayer[bayer][3][0], 2 * qy + kBayer[bayer][3][1], 0);
            out.ref(qx, qy, 0) = store(pol, r);
            out.ref(qx, qy, 1) = store(pol, M<C>::div(g + g2, C(2)));
            out.ref(qx, qy, 2) = store(pol, b);
            out.ref(qx, qy, 3) = C(0);
        }
    }
}

// ---------------------------------------------------------------------------------------
// a9: blendHighlightsImage, demosaic.cl:338-380
// ---------------------------------------------------------------------------------------
template <class C>
void blend_highlights(const Pol& pol, const Img<C>& in, C clip, Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    const C S3 = sizeof(C) == 4 ? (C)1.7320508f : (C)1.7320508;
    const C trans[3][3] = {{1, 1, 1}, {S3, -S3, 0}, {-1, -1, 2}};
    const C itrans[3][3] = {{1, S3 / C(2), C(-0.5)}, {1, -S3 / C(2), C(-0.5)}, {1, 0, 1}};
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int y = y0; y < y1; y++) {
            for (int x = 0; x < in.w; x++) {
                C p[3] = {in.at(x, y, 0), in.at(x, y, 1), in.at(x, y, 2)};
                if (p[0] > clip || p[1] > clip || p[2] > clip) {
                    C cam[2][3];
                    for (int k = 0; k < 3; k++) {
                        cam[0][k] = p[k];
                        cam[1][k] = mminc<C>(p[k], clip);
                    }
                    C lab[2][3], sum[2];
                    for (int i = 0; i < 2; i++) {
                        for (int r = 0; r < 3; r++)
                            lab[i][r] = trans[r][0] * cam[i][0] + trans[r][1] * cam[i][1] + trans[r][2] * cam[i][2];
                        sum[i] = lab[i][1] * lab[i][1] + lab[i][2] * lab[i][2];
                    }
                    const C chratio = sum[0] > C(0) ? M<C>::sqrt(M<C>::div(sum[1], sum[0])) : C(1);
                    lab[0][1] *= chratio;
                    lab[0][2] *= chratio;
                    for (int r = 0; r < 3; r++)
                        p[r] = M<C>::div(itrans[r][0] * lab[0][0] + itrans[r][1] * lab[0][1] + itrans[r][2] * lab[0][2], C(3));
                }
                for (int k = 0; k < 3; k++) out.ref(x, y, k) = store(pol, p[k]);
                out.ref(x, y, 3) = C(0);
            }
        }
    });
}

// a10: transformImage, demosaic.cl:728-733
template <class C>
void transform(const Pol& pol, const Img<C>& in, const float m[9], Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int y = y0; y < y1; y++) {
            for (int x = 0; x < in.w; x++) {
                const C a = in.at(x, y, 0), b = in.at(x, y, 1), c = in.at(x, y, 2);
                for (int r = 0; r < 3; r++)
                    out.ref(x, y, r) = store(pol, (C)m[3 * r] * a + (C)m[3 * r + 1] * b + (C)m[3 * r + 2] * c);
                out.ref(x, y, 3) = C(0);
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a11: despeckleImage binds the kernel despeckleLumaMedianChromaImage
// (demosaic_cl.cpp:270-291 -> demosaic.cl:444-489): half-precision reads (read_imageh),
// luma clamped between its second extremes, chroma by a 3x3 median network.  Every
// half-precision operation is rounded to binary16.
// ---------------------------------------------------------------------------------------
template <class C>
void despeckle(const Pol& pol, const Img<C>& in, const float va[3], const float vb[3], Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    auto H = [&](C v) { return half_op(pol, v); };
    auto smin = [](C a, C b) { return a < b ? a : b; };
    auto smax = [](C a, C b) { return a > b ? a : b; };
    // s(a,b): temp = a; a = min(a,b); b = max(temp,b)
    auto S = [&](C& a, C& b) {
        const C t = a;
        a = smin(a, b);
        b = smax(t, b);
    };
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int py = y0; py < y1; py++) {
            for (int px = 0; px < in.w; px++) {
                C sample = 0, firstMax = 0, secMax = 0;
                const C hinf = pol.half_reads() ? H(C(65535)) : C(65535);
                C firstMin = hinf, secMin = hinf;
                auto rd = [&](int dx, int dy, C* cb, C* cr) {
                    const C v = H(in.at(px + dx, py + dy, 0));
                    *cb = H(in.at(px + dx, py + dy, 1));
                    *cr = H(in.at(px + dx, py + dy, 2));
                    secMax = (v <= firstMax && v > secMax) ? v : secMax;
                    secMax = v > firstMax ? firstMax : secMax;
                    firstMax = v > firstMax ? v : firstMax;
                    secMin = (v >= firstMin && v < secMin) ? v : secMin;
                    secMin = v < firstMin ? firstMin : secMin;
                    firstMin = v < firstMin ? v : firstMin;
                    if (dx == 0 && dy == 0) sample = v;
                };
                C a[6][2];
                rd(0, -1, &a[0][0], &a[0][1]);
                rd(1, -1, &a[1][0], &a[1][1]);
                rd(0, 0, &a[2][0], &a[2][1]);
                rd(1, 0, &a[3][0], &a[3][1]);
                rd(0, 1, &a[4][0], &a[4][1]);
                rd(1, 1, &a[5][0], &a[5][1]);
                for (int k = 0; k < 2; k++) {
                    S(a[0][k], a[1][k]); S(a[2][k], a[3][k]); S(a[4][k], a[5][k]);
                    S(a[0][k], a[2][k]); S(a[1][k], a[3][k]); S(a[0][k], a[4][k]); S(a[3][k], a[5][k]);
                }
                rd(-1, 1, &a[0][0], &a[0][1]);
                for (int k = 0; k < 2; k++) {
                    S(a[0][k], a[1][k]); S(a[2][k], a[3][k]); S(a[0][k], a[2][k]);
                    S(a[1][k], a[3][k]); S(a[0][k], a[4][k]); S(a[3][k], a[4][k]);
                }
                rd(-1, 0, &a[0][0], &a[0][1]);
                for (int k = 0; k < 2; k++) {
                    S(a[0][k], a[1][k]); S(a[2][k], a[3][k]); S(a[0][k], a[2][k]); S(a[1][k], a[3][k]);
                }
                rd(-1, -1, &a[0][0], &a[0][1]);
                for (int k = 0; k < 2; k++) {
                    S(a[0][k], a[1][k]); S(a[0][k], a[2][k]); S(a[1][k], a[2][k]);
                }
                // half arithmetic: every result rounded to binary16
                const C sigma = H(M<C>::sqrt((C)va[0] + (C)vb[0] * sample));
                const C four_sigma = H(C(4) * sigma);
                auto hsmooth = [&](C e0, C e1, C x) {
                    const C t = clampc<C>(H(M<C>::div(H(x - e0), H(e1 - e0))), C(0), C(1));
                    return H(H(t * t) * H(C(3) - H(C(2) * t)));
                };
                auto hmix = [&](C x, C y, C t) { return H(x + H(H(y - x) * t)); };
                const C minVal = hmix(secMin, firstMin, hsmooth(sigma, four_sigma, H(secMin - firstMin)));
                const C maxVal = hmix(secMax, firstMax, hsmooth(sigma, four_sigma, H(firstMax - secMax)));
                sample = clampc<C>(sample, minVal, maxVal);
                out.ref(px, py, 0) = store(pol, sample);
                out.ref(px, py, 1) = store(pol, a[1][0]);
                out.ref(px, py, 2) = store(pol, a[1][1]);
                out.ref(px, py, 3) = C(0);
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a12: downsampleImage, demosaic.cl:853-865
// ---------------------------------------------------------------------------------------
template <class C>
void downsample(const Pol& pol, const Img<C>& in, int ow, int oh, Img<C>& out) {
    out = Img<C>(ow, oh, 4);
    const C nx = M<C>::div(C(1), (C)ow), ny = M<C>::div(C(1), (C)oh);
    parallel_rows(oh, [&](int y0, int y1) {
        for (int y = y0; y < y1; y++) {
            for (int x = 0; x < ow; x++) {
                const C px = ((C)x + C(0.5)) * nx, py = ((C)y + C(0.5)) * ny;
                const C sx = C(0.5) * nx, sy = C(0.5) * ny;
                C t0[4], t1[4], t2[4], t3[4];
                sample_linear(in, px + -sx, py + -sy, t0);
                sample_linear(in, px + sx, py + -sy, t1);
                sample_linear(in, px + -sx, py + sy, t2);
                sample_linear(in, px + sx, py + sy, t3);
                for (int k = 0; k < 4; k++) out.ref(x, y, k) = store(pol, C(0.25) * (t0[k] + t1[k] + t2[k] + t3[k]));
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a14: denoiseImage (bilateral), demosaic.cl:735-765
// ---------------------------------------------------------------------------------------
template <class C>
void denoise_bilateral(const Pol& pol, const Img<C>& in, const float va[3], const float vb[3], float chromaBoost,
                       float gradientBoost, Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    const C SQRT2 = sizeof(C) == 4 ? (C)1.41421356237309504880f : (C)1.41421356237309504880;
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int py = y0; py < y1; py++) {
            for (int px = 0; px < in.w; px++) {
                C in3[3] = {in.at(px, py, 0), in.at(px, py, 1), in.at(px, py, 2)};
                C sigma[3];
                for (int k = 0; k < 3; k++) sigma[k] = M<C>::sqrt((C)va[k] + (C)vb[k] * in3[0]);
                C lumaBoost = 1;
                if ((C)gradientBoost > C(1)) {
                    C gx, gy;
                    sobel(in, px, py, &gx, &gy);
                    lumaBoost = (C)gradientBoost - ((C)gradientBoost - C(1)) *
                                                     smoothstepc<C>(C(0.5), C(2), len2<C>(M<C>::div(gx, sigma[0]), M<C>::div(gy, sigma[0])));
                }
                const C edge[3] = {lumaBoost * SQRT2, (C)chromaBoost * SQRT2, (C)chromaBoost * SQRT2};
                C filt[3] = {0, 0, 0}, norm[3] = {0, 0, 0};
                for (int y = -2; y <= 2; y++) {
                    for (int x = -2; x <= 2; x++) {
                        C s[3], d[3];
                        for (int k = 0; k < 3; k++) {
                            s[k] = in.at(px + x, py + y, k);
                            d[k] = M<C>::div(s[k] - in3[k], sigma[k]);
                        }
                        const C l = len3<C>(d[0], d[1], d[2]);
                        for (int k = 0; k < 3; k++) {
                            const C wk = C(1) - stepc<C>(edge[k], l);
                            filt[k] += wk * s[k];
                            norm[k] += wk;
                        }
                    }
                }
                for (int k = 0; k < 3; k++) out.ref(px, py, k) = store(pol, M<C>::div(filt[k], norm[k]));
                out.ref(px, py, 3) = C(0);
            }
        }
    });
}

// a15: denoiseImageGuided + denoiseLumaChromaGuided, demosaic.cl:767-851
template <class C>
void denoise_guided(const Pol& pol, const Img<C>& in, const float va[3], const float vb[3], Img<C>& out) {
    out = Img<C>(in.w, in.h, 4);
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int py = y0; py < y1; py++) {
            for (int px = 0; px < in.w; px++) {
                const C I[3] = {in.at(px, py, 0), in.at(px, py, 1), in.at(px, py, 2)};
                C eps[3];
                for (int k = 0; k < 3; k++) eps[k] = (C)va[k] + (C)vb[k] * I[0];
                const C norm = M<C>::div(C(1), C(25));
                C mI[3] = {0, 0, 0}, rr = 0, rg = 0, rb = 0, gg = 0, gb = 0, bb = 0;
                for (int y = -2; y <= 2; y++) {
                    for (int x = -2; x <= 2; x++) {
                        const C s0 = in.at(px + x, py + y, 0), s1 = in.at(px + x, py + y, 1), s2 = in.at(px + x, py + y, 2);
                        mI[0] += s0;
                        mI[1] += s1;
                        mI[2] += s2;
                        rr += s0 * s0;
                        rg += s0 * s1;
                        rb += s0 * s2;
                        gg += s1 * s1;
                        gb += s1 * s2;
                        bb += s2 * s2;
                    }
                }
                for (int k = 0; k < 3; k++) mI[k] *= norm;
                rr *= norm; rg *= norm; rb *= norm; gg *= norm; gb *= norm; bb *= norm;
                const C vrr = rr - mI[0] * mI[0], vrg = rg - mI[0] * mI[1], vrb = rb - mI[0] * mI[2];
                const C vgg = gg - mI[1] * mI[1], vgb = gb - mI[1] * mI[2], vbb = bb - mI[2] * mI[2];
                const C vrre = vrr + eps[0], vgge = vgg + eps[1], vbbe = vbb + eps[2];
                C invrr = vgge * vbbe - vgb * vgb;
                C invrg = vgb * vrb - vrg * vbbe;
                C invrb = vrg * vgb - vgge * vrb;
                C invgg = vrre * vbbe - vrb * vrb;
                C invgb = vrb * vrg - vrre * vgb;
                C invbb = vrre * vgge - vrg * vrg;
                const C invCovDet = M<C>::div(C(1), invrr * vrre + invrg * vrg + invrb * vrb);
                invrr *= invCovDet; invrg *= invCovDet; invrb *= invCovDet;
                invgg *= invCovDet; invgb *= invCovDet; invbb *= invCovDet;
                const C cr[3] = {vrr, vrg, vrb}, cg[3] = {vrg, vgg, vgb}, cb[3] = {vrb, vgb, vbb};
                C ar[3], ag[3], ab[3], b[3];
                for (int k = 0; k < 3; k++) {
                    ar[k] = invrr * cr[k] + invrg * cg[k] + invrb * cb[k];
                    ag[k] = invrg * cr[k] + invgg * cg[k] + invgb * cb[k];
                    ab[k] = invrb * cr[k] + invgb * cg[k] + invbb * cb[k];
                }
                for (int k = 0; k < 3; k++) b[k] = mI[k] - ar[k] * mI[0] - ag[k] * mI[1] - ab[k] * mI[2];
                for (int k = 0; k < 3; k++)
                    out.ref(px, py, k) = store(pol, ar[k] * I[0] + ag[k] * I[1] + ab[k] * I[2] + b[k]);
                out.ref(px, py, 3) = C(0);
            }
        }
    });
}

// a16: GuidedFilter::filter (guided_filter.cpp:195-225, guided_filter.cl:16-154).
// Intermediate images: mean_I in storage precision (pixel_float4), everything else fp32.
template <class C>
void box_blur(const Pol& pol, bool storage_rounded, const Img<C>& in, int fs, Img<C>& out) {
    // boxBlurX run twice through a transposed temporary (guided_filter.cpp:26-48)
    Img<C> tmp(in.h, in.w, in.c);
    for (int pass = 0; pass < 2; pass++) {
        const Img<C>& src = pass == 0 ? in : tmp;
        Img<C> dst(src.h, src.w, src.c);
        for (int y = 0; y < src.h; y++) {
            for (int x = 0; x < src.w; x++) {
                for (int k = 0; k < src.c; k++) {
                    C sum = 0;
                    for (int i = -fs / 2; i <= fs / 2; i++) sum += src.at(x + i, y, k);
                    sum = M<C>::div(sum, (C)fs);
                    dst.ref(y, x, k) = storage_rounded ? store(pol, sum) : sum;
                }
            }
        }
        if (pass == 0) tmp = dst;
        else out = dst;
    }
}

template <class C>
void guided_filter(const Pol& pol, const Img<C>& in, int fs, const float eps[3], Img<C>& out) {
    const int w = in.w, h = in.h;
    Img<C> meanI;
    box_blur(pol, true, in, fs, meanI);
    Img<C> p1(w, h, 4), p2(w, h, 2);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const C a = in.at(x, y, 0), b = in.at(x, y, 1), c = in.at(x, y, 2);
            p1.ref(x, y, 0) = a * a; p1.ref(x, y, 1) = a * b; p1.ref(x, y, 2) = a * c; p1.ref(x, y, 3) = b * b;
            p2.ref(x, y, 0) = b * c; p2.ref(x, y, 1) = c * c;
        }
    Img<C> p1b, p2b;
    box_blur(pol, false, p1, fs, p1b);
    box_blur(pol, false, p2, fs, p2b);
    Img<C> inv1(w, h, 4), inv2(w, h, 2);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const C m0 = meanI.at(x, y, 0), m1 = meanI.at(x, y, 1), m2 = meanI.at(x, y, 2);
            const C vrr = p1b.at(x, y, 0) - m0 * m0 + (C)eps[0] * m0;
            const C vrg = p1b.at(x, y, 1) - m0 * m1;
            const C vrb = p1b.at(x, y, 2) - m0 * m2;
            const C vgg = p1b.at(x, y, 3) - m1 * m1 + (C)eps[1];
            const C vgb = p2b.at(x, y, 0) - m1 * m2;
            const C vbb = p2b.at(x, y, 1) - m2 * m2 + (C)eps[2];
            C invrr = vgg * vbb - vgb * vgb;
            C invrg = vgb * vrb - vrg * vbb;
            C invrb = vrg * vgb - vgg * vrb;
            C invgg = vrr * vbb - vrb * vrb;
            C invgb = vrb * vrg - vrr * vgb;
            C invbb = vrr * vgg - vrg * vrg;
            const C det = invrr * vrr + invrg * vrg + invrb * vrb;
            inv1.ref(x, y, 0) = M<C>::div(invrr, det); inv1.ref(x, y, 1) = M<C>::div(invrg, det);
            inv1.ref(x, y, 2) = M<C>::div(invrb, det); inv1.ref(x, y, 3) = M<C>::div(invgg, det);
            inv2.ref(x, y, 0) = M<C>::div(invgb, det); inv2.ref(x, y, 1) = M<C>::div(invbb, det);
        }
    Img<C> ipr(w, h, 4), ipg(w, h, 4), ipb(w, h, 4);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const C p[3] = {in.at(x, y, 0), in.at(x, y, 1), in.at(x, y, 2)};
            for (int k = 0; k < 3; k++) {
                ipr.ref(x, y, k) = p[0] * p[k];
                ipg.ref(x, y, k) = p[1] * p[k];
                ipb.ref(x, y, k) = p[2] * p[k];
            }
        }
    Img<C> iprb, ipgb, ipbb;
    box_blur(pol, false, ipr, fs, iprb);
    box_blur(pol, false, ipg, fs, ipgb);
    box_blur(pol, false, ipb, fs, ipbb);
    Img<C> abr(w, h, 4), abg(w, h, 4), abb(w, h, 4);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const C mp[3] = {meanI.at(x, y, 0), meanI.at(x, y, 1), meanI.at(x, y, 2)};
            C cr[3], cg[3], cb[3];
            for (int k = 0; k < 3; k++) {
                cr[k] = iprb.at(x, y, k) - mp[0] * mp[k];
                cg[k] = ipgb.at(x, y, k) - mp[1] * mp[k];
                cb[k] = ipbb.at(x, y, k) - mp[2] * mp[k];
            }
            const C irr = inv1.at(x, y, 0), irg = inv1.at(x, y, 1), irb = inv1.at(x, y, 2), igg = inv1.at(x, y, 3);
            const C igb = inv2.at(x, y, 0), ibb = inv2.at(x, y, 1);
            C ar[3], ag[3], ab[3];
            for (int k = 0; k < 3; k++) {
                ar[k] = irr * cr[k] + irg * cg[k] + irb * cb[k];
                ag[k] = irg * cr[k] + igg * cg[k] + igb * cb[k];
                ab[k] = irb * cr[k] + igb * cg[k] + ibb * cb[k];
            }
            for (int k = 0; k < 3; k++) {
                abr.ref(x, y, k) = ar[k];
                abg.ref(x, y, k) = ag[k];
                abb.ref(x, y, k) = ab[k];
            }
            abr.ref(x, y, 3) = mp[0] - ar[0] * mp[0] - ag[0] * mp[1] - ab[0] * mp[2];
            abg.ref(x, y, 3) = mp[1] - ar[1] * mp[0] - ag[1] * mp[1] - ab[1] * mp[2];
            abb.ref(x, y, 3) = mp[2] - ar[2] * mp[0] - ag[2] * mp[1] - ab[2] * mp[2];
        }
    Img<C> abrb, abgb, abbb;
    box_blur(pol, false, abr, fs, abrb);
    box_blur(pol, false, abg, fs, abgb);
    box_blur(pol, false, abb, fs, abbb);
    out = Img<C>(w, h, 4);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const C I[3] = {in.at(x, y, 0), in.at(x, y, 1), in.at(x, y, 2)};
            const C bw[3] = {abrb.at(x, y, 3), abgb.at(x, y, 3), abbb.at(x, y, 3)};
            for (int k = 0; k < 3; k++)
                out.ref(x, y, k) = store(pol, abrb.at(x, y, k) * I[0] + abgb.at(x, y, k) * I[1] + abbb.at(x, y, k) * I[2] + bw[k]);
            out.ref(x, y, 3) = C(0);
        }
}

// ---------------------------------------------------------------------------------------
// a17: reassembleImage, demosaic.cl:867-896
// ---------------------------------------------------------------------------------------
template <class C>
void reassemble(const Pol& pol, const Img<C>& d0, const Img<C>& i1, const Img<C>& d1, float sharpening_, const float nlf[2],
                Img<C>& out) {
    Img<C> res(d0.w, d0.h, 4);
    const C nx = M<C>::div(C(1), (C)d0.w), ny = M<C>::div(C(1), (C)d0.h);
    parallel_rows(d0.h, [&](int y0, int y1) {
        for (int y = y0; y < y1; y++) {
            for (int x = 0; x < d0.w; x++) {
                const C ipx = ((C)x + C(0.5)) * nx, ipy = ((C)y + C(0.5)) * ny;
                C p1[4], pd1[4], dp[4];
                sample_linear(i1, ipx, ipy, p1);
                sample_linear(d1, ipx, ipy, pd1);
                for (int k = 0; k < 4; k++) dp[k] = d0.at(x, y, k) - (p1[k] - pd1[k]);
                C sharpening = (C)sharpening_;
                if (sharpening > C(1)) {
                    C a[4], b[4];
                    sample_linear(d1, ipx + nx, ipy + C(0) * ny, a);
                    sample_linear(d1, ipx - nx, ipy - C(0) * ny, b);
                    const C dx = M<C>::div(a[0] - b[0], C(2));
                    sample_linear(d1, ipx + C(0) * nx, ipy + ny, a);
                    sample_linear(d1, ipx - C(0) * nx, ipy - ny, b);
                    const C dy = M<C>::div(a[0] - b[0], C(2));
                    const C threshold = C(0.25) * M<C>::sqrt((C)nlf[0] + (C)nlf[1] * pd1[0]);
                    const C detail = smoothstepc<C>(C(0.25) * threshold, threshold, len2<C>(dx, dy)) *
                                     (C(1) - smoothstepc<C>(C(0.95), C(1), dp[0])) *
                                     (C(0.6) + C(0.4) * smoothstepc<C>(C(0), C(0.1), dp[0]));
                    sharpening = C(1) + (sharpening - C(1)) * detail;
                }
                dp[0] = mixc<C>(pd1[0], dp[0], sharpening);
                for (int k = 0; k < 4; k++) res.ref(x, y, k) = store(pol, dp[k]);
            }
        }
    });
    out = res;
}

// ---------------------------------------------------------------------------------------
// a18: localToneMappingMaskImage, demosaic.cl:1026-1107
// ---------------------------------------------------------------------------------------
template <class C>
void ltm_mask(const Pol& pol, const Img<C>& in, const Img<C>& guide, const oracle_ltm_params& lp, const float m[9],
              Img<C>& out) {
    out = Img<C>(in.w, in.h, 1);
    const C bw[9] = {C(0.16), C(0.16), C(0.08), C(0.16), C(0.16), C(0.08), C(0.08), C(0.08), C(0.04)};
    const C bo[9][2] = {{C(-1.5), C(-1.5)}, {C(0.5), C(-1.5)}, {C(2), C(-1.5)}, {C(-1.5), C(0.5)}, {C(0.5), C(0.5)},
                        {C(2), C(0.5)},     {C(-1.5), C(2)},   {C(0.5), C(2)},  {C(2), C(2)}};
    const C nx = M<C>::div(C(1), (C)in.w), ny = M<C>::div(C(1), (C)in.h);
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int y = y0; y < y1; y++) {
            for (int x = 0; x < in.w; x++) {
                const C px = (C)x * nx, py = (C)y * ny;
                C gs[9];
                C sum = 0, sumSq = 0;
                for (int i = 0; i < 9; i++) {
                    C t[4];
                    sample_linear(guide, px + (bo[i][0] + C(0.5)) * nx, py + (bo[i][1] + C(0.5)) * ny, t);
                    gs[i] = t[0];
                    const C s = bw[i] * t[0];
                    sum += s;
                    sumSq += s * s;
                }
                const C mean = sum, var = sumSq - sum * sum;
                C inp[4];
                sample_linear(in, px + C(0.5) * nx, py + C(0.5) * ny, inp);
                const C luma = inp[0];
                const C eps = (C)lp.guidedFilterEps;
                C filtered = 0, knorm = 0;
                for (int i = 0; i < 9; i++) {
                    const C s = gs[i];
                    const C wgt = bw[i] * (C(1) + M<C>::div((s - mean) * (luma - mean), var + eps));
                    filtered += wgt * s;
                    knorm += wgt;
                }
                const C illuminance = M<C>::div(filtered, knorm);
                const C reflectance = M<C>::div(luma, illuminance);
                C rgb[3];
                for (int r = 0; r < 3; r++) rgb[r] = (C)m[3 * r] * inp[0] + (C)m[3 * r + 1] * inp[1] + (C)m[3 * r + 2] * inp[2];
                const C hc = mminc<C>(len3<C>(M<C>::sqrt(C(2) * rgb[0]), M<C>::sqrt(C(2) * rgb[1]), M<C>::sqrt(C(2) * rgb[2])), C(1));
                const C tc = mixc<C>((C)lp.shadows, (C)lp.highlights, hc);
                const C v = M<C>::div(M<C>::pow(illuminance, M<C>::div(C(1), tc)) * M<C>::pow(reflectance, (C)lp.detail), luma);
                out.ref(x, y, 0) = store(pol, v);
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// a19: convertTosRGB + toneCurve/sigmoid/saturationBoost/contrastBoost, demosaic.cl:1380-1474
// ---------------------------------------------------------------------------------------
template <class C>
C sigmoid(C x, C s) { return C(0.5) * (M<C>::tanh(s * x - C(0.3) * s) + C(1)); }

template <class C>
C tone_curve(C x, C s) {
    // native_powr(0.95 * x, 0.5): evaluated as a square root
    return M<C>::div(sigmoid<C>(M<C>::sqrt(C(0.95) * x), s) - sigmoid<C>(C(0), s), sigmoid<C>(C(1), s) - sigmoid<C>(C(0), s));
}

template <class C>
void convert_srgb_pixel(const C in[3], const C* ltm, const float m[9], const oracle_rgb_params& rp, C out[3]) {
    C p[3] = {in[0], in[1], in[2]};
    const C eb = (C)rp.exposureBias != C(0) ? M<C>::powr(C(2), (C)rp.exposureBias) : C(1);
    for (int k = 0; k < 3; k++) p[k] *= eb;
    if ((C)rp.saturation != C(1)) {
        const C luma = C(0.2126) * p[0] + C(0.7152) * p[1] + C(0.0722) * p[2];
        for (int k = 0; k < 3; k++) {
            const C clip = smoothstepc<C>(C(0.75), C(2), p[k]);
            p[k] = mixc<C>(luma, p[k], mixc<C>((C)rp.saturation, C(1), clip));
        }
    }
    if ((C)rp.contrast != C(1)) {
        for (int k = 0; k < 3; k++) {
            const C clip = smoothstepc<C>(C(0.9), C(2), p[k]);
            p[k] = mixc<C>(C(0.2), p[k], mixc<C>((C)rp.contrast, C(1), clip));
        }
    }
    C rgb[3];
    for (int r = 0; r < 3; r++) rgb[r] = (C)m[3 * r] * p[0] + (C)m[3 * r + 1] * p[1] + (C)m[3 * r + 2] * p[2];
    for (int k = 0; k < 3; k++) rgb[k] = clampc<C>(tone_curve<C>(rgb[k], (C)rp.toneCurveSlope), C(0), C(1));
    if (rp.localToneMapping) {
        const C boost = *ltm;
        if (boost > C(1)) {
            const C luma = C(0.2126) * rgb[0] + C(0.7152) * rgb[1] + C(0.0722) * rgb[2];
            const C t = M<C>::pow(luma, C(0.5));
            for (int k = 0; k < 3; k++) {
                const C a = rgb[k] * boost;
                const C b = luma < C(1) ? C(1) - M<C>::div((C(1) - rgb[k]) * (C(1) - boost * luma), C(1) - luma) : rgb[k];
                rgb[k] = mixc<C>(a, b, t);
            }
        } else if (boost < C(1)) {
            for (int k = 0; k < 3; k++) rgb[k] *= boost;
        }
    }
    if ((C)rp.blacks > C(0)) {
        for (int k = 0; k < 3; k++) rgb[k] = M<C>::div(rgb[k] - (C)rp.blacks, C(1) - (C)rp.blacks);
    }
    for (int k = 0; k < 3; k++) out[k] = rgb[k];
}

template <class C>
void convert_srgb(const Img<C>& in, const Img<C>* ltm, const float m[9], const oracle_rgb_params& rp, uint8_t* o8,
                  float* of) {
    parallel_rows(in.h, [&](int y0, int y1) {
        for (int y = y0; y < y1; y++) {
            for (int x = 0; x < in.w; x++) {
                const C p[3] = {in.at(x, y, 0), in.at(x, y, 1), in.at(x, y, 2)};
                const C lv = (ltm && rp.localToneMapping) ? ltm->at(x, y, 0) : C(0);
                C rgb[3];
                convert_srgb_pixel<C>(p, &lv, m, rp, rgb);
                const size_t o = ((size_t)y * in.w + x) * 4;
                if (o8) {
                    for (int k = 0; k < 3; k++) o8[o + k] = glsm::to_unorm8((float)rgb[k]);
                    o8[o + 3] = 0;
                }
                if (of) {
                    for (int k = 0; k < 3; k++) of[o + k] = (float)rgb[k];
                    of[o + 3] = 0;
                }
            }
        }
    });
}

// ---------------------------------------------------------------------------------------
// Host colour math, restated from demosaic_utils.cpp:25-52, 809-822 and
// gls_linalg.hpp:347-556 (float, same operation order).
// ---------------------------------------------------------------------------------------
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
    // determinant(cofactor 2x2): 0 + (1*a)*d + (-1*b)*c
    float r = 0;
    r += 1.0f * a * d;
    r += -1.0f * b * c;
    return r;
}

void cofactor2(const M3 m, int p, int q, float out[4]) {
    int n = 0;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            if (r != p && c != q) out[n++] = m[r][c];
}

float det3(const M3 m) {
    float sign = 1, result = 0;
    for (int f = 0; f < 3; f++) {
        float c[4];
        cofactor2(m, 0, f, c);
        result += sign * m[0][f] * det2(c[0], c[1], c[2], c[3]);
        sign = -sign;
    }
    return result;
}

void inverse3(const M3 m, M3 out) {
    const float det = det3(m);
    M3 adj;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const float sign = ((i + j) % 2 == 0) ? 1.0f : -1.0f;
            float c[4];
            cofactor2(m, i, j, c);
            const float d = det2(c[0], c[1], c[2], c[3]);
            adj[j][i] = d != 0 ? sign * d : 0;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out[i][j] = adj[i][j] / det;
}

const M3 kXyzRgb = {{0.4124564f, 0.3575761f, 0.1804375f}, {0.2126729f, 0.7151522f, 0.0721750f}, {0.0193339f, 0.1191920f, 0.9503041f}};

void cam_ycbcr(const M3 rgb_cam, M3 out) {
    float cam_y[3];
    for (int i = 0; i < 3; i++) {
        float s = 0;
        for (int k = 0; k < 3; k++) s += kXyzRgb[1][k] * rgb_cam[k][i];
        cam_y[i] = s;
    }
    const float KR = cam_y[0], KG = cam_y[1], KB = cam_y[2];
    const M3 r = {{KR, KG, KB},
                  {-0.5f * KR / (1.0f - KB), -0.5f * KG / (1 - KB), 0.5f},
                  {0.5f, -0.5f * KG / (1 - KR), -0.5f * KB / (1 - KR)}};
    memcpy(out, r, sizeof(M3));
}

// ---------------------------------------------------------------------------------------
// Pipeline: RawConverter::demosaicImage (raw_converter.cpp:73-186) with
// PyramidalDenoise<levels>::denoise (pyramidal_denoise.cpp:104-149).
// ---------------------------------------------------------------------------------------
template <class C>
void denoise_level(const Pol& pol, int algo, bool coarsest, const Img<C>& in, const float np[6], const oracle_denoise_params& dp,
                   Img<C>& out) {
    const float va[3] = {np[0], np[1], np[2]}, vb[3] = {np[3], np[4], np[5]};
    if (algo == 0 || (algo == 1 && coarsest)) denoise_bilateral(pol, in, va, vb, dp.chromaBoost, dp.gradientBoost, out);
    else if (algo == 1) denoise_guided(pol, in, va, vb, out);
    else guided_filter(pol, in, 5, vb, out);
}

template <class C>
int demosaic(const uint16_t* raw, int w, int h, int stride, oracle_params* p, int prec, uint8_t* o8, float* of,
             oracle_taps* taps) {
    const int L = p->pyramid_levels;
    if (w <= 0 || h <= 0 || (w & 1) || (h & 1) || L < 4 || L > ORACLE_MAX_LEVELS) return -1;
    if ((w >> (L - 1)) < 1 || (h >> (L - 1)) < 1) return -1;
    const Pol pol{prec};
    const bool high_noise = p->noise_level > 0.6f;

    Img<C> scaled;
    scale_raw(pol, raw, w, h, stride, p->bayer_pattern, p->scale_mul, p->black_level / 0xffff, scaled);
    float raw_nlf[8];
    compute_raw_nlf(scaled, p->bayer_pattern, raw_nlf, prec == ORACLE_F16_STATS);
    for (int c = 0; c < 4; c++) p->raw_nlf[c] = raw_nlf[4 + c];

    if (high_noise) {
        Img<C> rgba, den;
        bayer_to_rgba(pol, scaled, p->bayer_pattern, rgba);
        despeckle_rgba(pol, rgba, den);
        denoise_rgba(pol, den, p->raw_nlf, rgba);
        rgba_to_bayer(pol, rgba, p->bayer_pattern, scaled);
    }
    if (taps && taps->scaled_raw) to_float(scaled, taps->scaled_raw);

    Img<C> green, lin, tmp;
    interpolate_green(pol, scaled, p->bayer_pattern, p->raw_nlf[1], green);
    if (taps && taps->green) to_float(green, taps->green);
    interpolate_red_blue(pol, scaled, green, p->bayer_pattern, (p->raw_nlf[0] + p->raw_nlf[2]) / 2, lin,
                         p->rotate_180 != 0);
    if (taps && taps->linear_rgb) to_float(lin, taps->linear_rgb);
    blend_highlights(pol, lin, C(1), tmp);

    M3 rgb_cam, cy, icy;
    memcpy(rgb_cam, p->rgb_cam, sizeof(M3));
    cam_ycbcr(rgb_cam, cy);
    transform(pol, tmp, &cy[0][0], lin);
    if (taps && taps->ycbcr) to_float(lin, taps->ycbcr);

    Img<C> image;
    {
        const float* np = p->pyramid_nlf[0];
        const float va[3] = {np[0], np[1], np[2]}, vb[3] = {np[3], np[4], np[5]};
        despeckle(pol, lin, va, vb, image);
    }
    if (taps && taps->level0) to_float(image, taps->level0);

    // PyramidalDenoise::denoise
    std::vector<Img<C>> pyr(L - 1), den(L);
    float calibrated[ORACLE_MAX_LEVELS][6];
    for (int i = 0; i < L; i++) {
        const Img<C>& src = i == 0 ? image : pyr[i - 1];
        if (i < L - 1) downsample(pol, src, w >> (i + 1), h >> (i + 1), pyr[i]);
        compute_nlf(src, p->pyramid_nlf[i], prec == ORACLE_F16_STATS);
        const float lm = p->denoise[i].luma * p->denoise[i].luma;
        const float cm = p->denoise[i].chroma * p->denoise[i].chroma;
        const float mul[6] = {lm, cm, cm, lm, cm, cm};
        for (int k = 0; k < 6; k++) calibrated[i][k] = p->pyramid_nlf[i][k] * mul[k];
    }
    denoise_level(pol, p->denoise_algorithm, true, pyr[L - 2], calibrated[L - 1], p->denoise[L - 1], den[L - 1]);
    for (int i = L - 2; i >= 0; i--) {
        const Img<C>& input = i > 0 ? pyr[i - 1] : image;
        denoise_level(pol, p->denoise_algorithm, false, input, calibrated[i], p->denoise[i], den[i]);
        const float nlf[2] = {calibrated[i][0], calibrated[i][3]};
        reassemble(pol, den[i], pyr[i], den[i + 1], p->denoise[i].sharpening, nlf, den[i]);
    }
    Img<C>& denoised = den[0];
    if (taps && taps->denoised0) to_float(denoised, taps->denoised0);

    inverse3(cy, icy);
    M3 icy_e;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) icy_e[i][j] = icy[i][j] * p->exposure_multiplier;

    Img<C> mask;
    if (p->rgb.localToneMapping) {
        ltm_mask(pol, denoised, den[3], p->ltm, &icy_e[0][0], mask);
        if (taps && taps->ltm_mask) to_float(mask, taps->ltm_mask);
    }
    Img<C> cam;
    transform(pol, denoised, &icy_e[0][0], cam);
    if (taps && taps->camera_rgb) to_float(cam, taps->camera_rgb);
    convert_srgb(cam, p->rgb.localToneMapping ? &mask : nullptr, p->rgb_cam, p->rgb, o8, of);
    return 0;
}

template <class C>
int fast_demosaic(const uint16_t* raw, int w, int h, int stride, const oracle_params* p, int prec, uint8_t* o8, float* of) {
    if (w <= 0 || h <= 0 || (w & 1) || (h & 1)) return -1;
    const Pol pol{prec};
    Img<C> scaled, rgb, hl;
    scale_raw(pol, raw, w, h, stride, p->bayer_pattern, p->scale_mul, p->black_level / 0xffff, scaled);
    fast_debayer(pol, scaled, p->bayer_pattern, rgb);
    blend_highlights(pol, rgb, C(1), hl);
    oracle_rgb_params rp = p->rgb;
    rp.localToneMapping = 0;  // the fast path binds a 1x1 placeholder mask (raw_converter.cpp:70-71)
    convert_srgb<C>(hl, nullptr, p->rgb_cam, rp, o8, of);
    return 0;
}

template <class F>
int dispatch(int prec, F&& f) {
    if (prec == ORACLE_F64) return f(double(0));
    return f(float(0));
}

}  // namespace

// ---------------------------------------------------------------------------------------
// autoWhiteBalance (demosaic_utils.cpp:857-1026), restated in the reference's operation
// order: 4x4 tiles of even size; per tile, over its 2x2 quads in raster order, the fp32
// running sums of the YCbCr image (M), of the absolute deviations from the mean (D) and,
// per luma bin of the near-white quads, of their normalised camera RGB.  Host CFA table
// (demosaic.hpp:83-88): {red, green, blue, green2} as (x, y).
// ---------------------------------------------------------------------------------------
namespace awb {

const int kHostBayer[4][4][2] = {
    {{1, 0}, {0, 0}, {0, 1}, {1, 1}},  // grbg
    {{0, 1}, {0, 0}, {1, 0}, {1, 1}},  // gbrg
    {{0, 0}, {1, 0}, {1, 1}, {0, 1}},  // rggb
    {{1, 1}, {1, 0}, {0, 0}, {0, 1}},  // bggr
};
constexpr int kBins = 128;

// readQuad (demosaic_utils.cpp:836-849): {red, (green + green2) / 2, blue}
inline void read_quad(const uint16_t* tile, int stride, int x, int y, int bayer, float q[3]) {
    const int (*o)[2] = kHostBayer[bayer];
    auto at = [&](int c) { return (float)tile[(size_t)(y + o[c][1]) * stride + x + o[c][0]]; };
    q[0] = at(0);
    q[1] = (at(1) + at(3)) / 2.0f;
    q[2] = at(2);
}

// rgb_ycbcr * v, each row accumulated from 0 (gls_linalg.hpp:353-372)
inline void mat_vec(const float m[9], const float v[3], float out[3]) {
    for (int j = 0; j < 3; j++) {
        float acc = 0;
        for (int k = 0; k < 3; k++) acc += m[3 * j + k] * v[k];
        out[j] = acc;
    }
}

// The camera RGB of a quad scaled by scale_mul and clipped at 1 (its YCbCr), and whether
// a channel sits in (0.5, 1] (demosaic_utils.cpp:861-881).
inline bool quad_ycbcr(const uint16_t* tile, int stride, int x, int y, int bayer, const float m[9],
                       const float smul[3], float black, float out[3]) {
    float q[3], rgb[3];
    read_quad(tile, stride, x, y, bayer, q);
    bool highlights = false;
    for (int c = 0; c < 3; c++) {
        rgb[c] = (smul[c] * (q[c] - black)) / (float)0xffff;
        if (rgb[c] > 1.0f) rgb[c] = 1.0f;
        else if (rgb[c] > 0.5f) highlights = true;
    }
    mat_vec(m, rgb, out);
    return highlights;
}

// Luma bin of (kBins - 1) * Y rounded half away from zero, clamped to [0, kBins - 1].  A
// negative rounded value lands in the top bin: the reference converts it to size_t before
// clamping, which on x86-64 wraps it to a huge value.
inline int luma_bin(float Y) {
    const float r = std::round((float)(kBins - 1) * Y);
    if (r < 0.0f || r > (float)(kBins - 1)) return kBins - 1;
    return (int)r;
}

struct TileResult {
    float gain[3];
    int highlights;
};

// autoWhiteBalanceKernel (demosaic_utils.cpp:851-966) over one tile of tw x th pixels.
TileResult tile(const uint16_t* t, int stride, int tw, int th, const float m[9], const float smul[3], float white,
                float black, int bayer, float fraction) {
    const int qw = tw / 2, qh = th / 2;
    int highlight_px = 0;
    float M[3] = {0, 0, 0};
    for (int y = 0; y < th; y += 2)
        for (int x = 0; x < tw; x += 2) {
            float p[3];
            if (quad_ycbcr(t, stride, x, y, bayer, m, smul, black, p)) highlight_px++;
            for (int c = 0; c < 3; c++) M[c] = M[c] + p[c];
        }
    const float n_quads = (float)th * tw / 4;
    for (int c = 0; c < 3; c++) M[c] = M[c] / n_quads;

    float D[3] = {0, 0, 0};
    for (int y = 0; y < qh; y++)
        for (int x = 0; x < qw; x++) {
            float p[3];
            quad_ycbcr(t, stride, 2 * x, 2 * y, bayer, m, smul, black, p);
            for (int c = 0; c < 3; c++) D[c] = D[c] + std::fabs(p[c] - M[c]);
        }
    const float n_yuv = (float)qh * qw;
    for (int c = 0; c < 3; c++) D[c] = D[c] / n_yuv;

    float bin_sum[kBins][3] = {};
    int bin_n[kBins] = {};
    const float Wr = 1.5f, WCr = 1.5f;
    int white_n = 0;
    float YMax = 0;
    for (int y = 0; y < qh; y++)
        for (int x = 0; x < qw; x++) {
            float p[3];
            quad_ycbcr(t, stride, 2 * x, 2 * y, bayer, m, smul, black, p);
            if (std::fabs(p[1] - (M[1] + std::copysign(D[1], M[1]))) < Wr * D[1] &&
                std::fabs(p[2] - (WCr * M[2] + std::copysign(D[2], M[2]))) < Wr * D[2]) {
                float q[3];
                read_quad(t, stride, 2 * x, 2 * y, bayer, q);
                const float Y = p[0];
                if (Y > YMax) YMax = Y;
                const int b = luma_bin(Y);
                for (int c = 0; c < 3; c++) bin_sum[b][c] = bin_sum[b][c] + (q[c] - black) / white;
                bin_n[b]++;
                white_n++;
            }
        }
    const int top = luma_bin(YMax);
    if (top == 0) return {{1, 1, 1}, 0};
    int n90 = 0;
    float avg[3] = {0, 0, 0};
    for (int i = top; i >= 0; i--) {
        for (int c = 0; c < 3; c++) avg[c] = avg[c] + bin_sum[i][c];
        n90 += bin_n[i];
        if ((float)n90 > fraction * (float)white_n) break;
    }
    TileResult r;
    float g[3];
    for (int c = 0; c < 3; c++) avg[c] = avg[c] / (float)n90;
    for (int c = 0; c < 3; c++) g[c] = YMax / avg[c];
    const float g1 = g[1];
    for (int c = 0; c < 3; c++) r.gain[c] = g[c] / g1;
    r.highlights = highlight_px;
    return r;
}

// autoWhiteBalance (demosaic_utils.cpp:976-1026): the mean of the 16 tiles' gains,
// normalised to green, and the fraction of quads with a channel in (0.5, 1].
void auto_white_balance(const uint16_t* raw, int w, int h, int stride, const float m[9], const float smul4[4],
                        float white, float black, int bayer, float wb[3], float* highlights) {
    const float s1 = smul4[1];
    const float smul[3] = {smul4[0] / s1, smul4[1] / s1, smul4[2] / s1};
    const int tw = 2 * ((w / 4) / 2), th = 2 * ((h / 4) / 2);
    float g[3] = {0, 0, 0};
    float hl = 0;
    for (int ty = 0; ty < 4; ty++)
        for (int tx = 0; tx < 4; tx++) {
            const TileResult r =
                tile(raw + (size_t)ty * th * stride + tx * tw, stride, tw, th, m, smul, white, black, bayer, 0.01f);
            for (int c = 0; c < 3; c++) g[c] = g[c] + r.gain[c];
            hl = hl + (float)r.highlights;
        }
    for (int c = 0; c < 3; c++) g[c] = g[c] / 16.0f;
    const float g1 = g[1];
    for (int c = 0; c < 3; c++) wb[c] = g[c] / g1;
    if (highlights) *highlights = hl / (float)(w * h / 4);
}

}  // namespace awb

// ---------------------------------------------------------------------------------------
// Colour-checker calibration (estimateRawParameters, demosaic_utils.cpp:686-785): per patch
// of a 6x4 ColorChecker chart, the fp32 mean and variance of each CFA channel over the
// patch's quads in raster order (colorCheckerRawStats, 411-533); the camera matrix and white
// point from the patch means (matrixFromColorChecker, 83-129, with dcraw's pseudoinverse,
// gls_linalg.hpp:559-590) and the raw noise slopes from the six neutral patches
// (linear_regression, 604-621: double sums of fp32 products).
// ---------------------------------------------------------------------------------------
namespace calib {

struct Rect {
    int x, y, w, h;
};

// alignToQuad (demosaic_utils.cpp:54-71)
Rect align_to_quad(Rect r) {
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

Rect patch_rect(const Rect& gmb, int row, int col) {
    const int pw = gmb.w / 6, ph = gmb.h / 4;
    return align_to_quad({gmb.x + col * pw + (int)(0.25 * pw), gmb.y + row * ph + (int)(0.25 * ph), (int)(0.5 * pw),
                          (int)(0.5 * ph)});
}

void patch_stats(const uint16_t* raw, int stride, float black, float white, int bayer, const Rect& gmb, int rotate,
                 float mean[24][4], float var[24][4]) {
    const int (*o)[2] = awb::kHostBayer[bayer];
    for (int row = 0; row < 4; row++)
        for (int col = 0; col < 6; col++) {
            const int idx = row * 6 + col;
            const Rect pr = patch_rect(gmb, row, col);
            const int samples = pr.w * pr.h / 4;
            auto px = [&](int y, int x, int c) {
                const float v = ((float)raw[(size_t)(y + o[c][1]) * stride + x + o[c][0]] - black) / white;
                return std::min(std::max(v, 0.0f), 1.0f);
            };
            float avg[4] = {0, 0, 0, 0};
            for (int y = 0; y < pr.h; y += 2)
                for (int x = 0; x < pr.w; x += 2)
                    for (int c = 0; c < 4; c++) avg[c] = avg[c] + px(pr.y + y, pr.x + x, c);
            for (int c = 0; c < 4; c++) avg[c] = avg[c] / (float)samples;
            float v[4] = {0, 0, 0, 0};
            for (int y = 0; y < pr.h; y += 2)
                for (int x = 0; x < pr.w; x += 2)
                    for (int c = 0; c < 4; c++) {
                        const float d = px(pr.y + y, pr.x + x, c) - avg[c];
                        v[c] = v[c] + d * d;
                    }
            for (int c = 0; c < 4; c++) {
                mean[idx][c] = avg[c];
                var[idx][c] = v[c] / (float)samples;
            }
        }
    if (rotate)
        for (int a = 0, b = 23; a < b; a++, b--)
            for (int c = 0; c < 4; c++) {
                std::swap(mean[a][c], mean[b][c]);
                std::swap(var[a][c], var[b][c]);
            }
}

// ColorChecker chart under D65 (xyY), matrixFromColorChecker
const float kGmbxyY[24][3] = {
    {0.400f, 0.350f, 10.1f}, {0.377f, 0.345f, 35.8f}, {0.247f, 0.251f, 19.3f}, {0.337f, 0.422f, 13.3f},
    {0.265f, 0.240f, 24.3f}, {0.261f, 0.343f, 43.1f}, {0.506f, 0.407f, 30.1f}, {0.211f, 0.175f, 12.0f},
    {0.453f, 0.306f, 19.8f}, {0.285f, 0.202f, 6.6f},  {0.380f, 0.489f, 44.3f}, {0.473f, 0.438f, 43.1f},
    {0.187f, 0.129f, 6.1f},  {0.305f, 0.478f, 23.4f}, {0.539f, 0.313f, 12.0f}, {0.448f, 0.470f, 59.1f},
    {0.364f, 0.233f, 19.8f}, {0.196f, 0.252f, 19.8f}, {0.310f, 0.316f, 90.0f}, {0.310f, 0.316f, 59.1f},
    {0.310f, 0.316f, 36.2f}, {0.310f, 0.316f, 19.8f}, {0.310f, 0.316f, 9.0f},  {0.310f, 0.316f, 3.1f}};

// pseudoinverse of a 24x3 matrix (gls_linalg.hpp:559-590, after dcraw)
void pseudoinverse(const float in[24][3], float out[24][3]) {
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

// {a, b} of the least-squares line through (x, y), six points
void regress6(const float x[6], const float y[6], float* a, float* b) {
    double sx = 0.0, sy = 0.0, sxx = 0.0, sxy = 0.0;
    for (int i = 0; i < 6; i++) sx = sx + x[i];
    for (int i = 0; i < 6; i++) sy = sy + y[i];
    for (int i = 0; i < 6; i++) sxx = sxx + (double)(x[i] * x[i]);
    for (int i = 0; i < 6; i++) sxy = sxy + (double)(x[i] * y[i]);
    const double n = 6.0;
    const double bb = (n * sxy - sx * sy) / (n * sxx - sx * sx);
    const double aa = (sy - bb * sx) / n;
    *a = (float)aa;
    *b = (float)bb;
}

// estimateRawParameters: cam_xyz (3x3), pre_mul (3), raw NLF slopes {r, g, b, g2}; false when
// cam_xyz_coeff rejects the matrix (a camera white at or below 1e-5)
bool estimate(const float mean[24][4], const float var[24][4], float cam_xyz[9], float pre_mul[3], float nlf[4]) {
    float xyz[24][3], inv[24][3];
    for (int q = 0; q < 24; q++) {
        const float x = kGmbxyY[q][0], y = kGmbxyY[q][1], Y = kGmbxyY[q][2];
        xyz[q][0] = Y * x / y;
        xyz[q][1] = Y;
        xyz[q][2] = Y * (1 - x - y) / y;
    }
    pseudoinverse(xyz, inv);
    float cx[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            float acc = 0;
            for (int k = 0; k < 24; k++) acc += mean[k][i] * inv[k][j];
            cx[3 * i + j] = acc;
        }
    // cam_xyz_coeff's white point (its matrix is dropped); it rejects a white <= 1e-5
    {
        M3 m, rgb_cam;
        memcpy(m, cx, sizeof(M3));
        mat_mul(m, kXyzRgb, rgb_cam);
        for (int i = 0; i < 3; i++) {
            float s = 0;
            for (int k = 0; k < 3; k++) s += rgb_cam[i][k] * 1.0f;
            if (!((double)s > 0.00001)) return false;
            pre_mul[i] = 1 / s;
        }
    }
    const float norm = cx[3] + cx[4] + cx[5];
    for (int k = 0; k < 9; k++) cam_xyz[k] = cx[k] / norm;
    const float p1 = pre_mul[1];
    for (int k = 0; k < 3; k++) pre_mul[k] = pre_mul[k] / p1;
    const int order[6] = {23, 22, 21, 20, 19, 18};  // Black, Neutral 3.5, 5, 6.5, 8, White
    for (int c = 0; c < 4; c++) {
        float x[6], y[6], a;
        for (int i = 0; i < 6; i++) {
            x[i] = mean[order[i]][c];
            y[i] = var[order[i]][c];
        }
        regress6(x, y, &a, &nlf[c]);
    }
    return true;
}

}  // namespace calib

// ---------------------------------------------------------------------------------------
// Lossless JPEG (ITU-T T.81 process 14, SOF3) as DNG stores raw tiles and strips: the
// decoder restates DecodeLosslessJPEG (src/gls_dng_lossless_jpeg.cpp:540-2142) -- marker
// parsing, Huffman decoding with its 8-bit lookup and its rules for invalid codes (17 bits
// consumed, category 0) and category 16 (-32768, no extra bits), predictors 0-7, restart
// intervals (bits dropped to the byte boundary, predictors reset); the encoder is test
// infrastructure of its own (any predictor, optional restart interval, length-limited
// Huffman tables built from the symbol counts) for streams the reference's encoder, which
// always writes predictor 1 without restarts, does not produce.
// ---------------------------------------------------------------------------------------
namespace lj92 {

struct Table {
    uint8_t bits[17] = {};
    uint8_t val[256] = {};
    int mincode[17] = {}, maxcode[18] = {}, valptr[17] = {};
    int look_n[256] = {}, look_v[256] = {};
    bool present = false;
};

// Figures C.1, C.2 and F.15 of T.81: canonical codes, decoding bounds, 8-bit lookup
void derive(Table& t) {
    int size[257], code[257], n = 0;
    for (int l = 1; l <= 16; l++)
        for (int i = 0; i < t.bits[l]; i++) size[n++] = l;
    size[n] = 0;
    int c = 0, si = size[0], p = 0;
    while (size[p]) {
        while (size[p] == si) code[p++] = c++;
        c <<= 1;
        si++;
    }
    p = 0;
    for (int l = 1; l <= 16; l++) {
        if (t.bits[l]) {
            t.valptr[l] = p;
            t.mincode[l] = code[p];
            p += t.bits[l];
            t.maxcode[l] = code[p - 1];
        } else {
            t.maxcode[l] = -1;
        }
    }
    t.maxcode[17] = 0xFFFFF;
    for (int k = 0; k < 256; k++) t.look_n[k] = 0;
    for (int q = 0; q < n; q++)
        if (size[q] <= 8) {
            const int lo = code[q] << (8 - size[q]), hi = lo | ((1 << (8 - size[q])) - 1);
            for (int k = lo; k <= hi; k++) {
                t.look_n[k] = size[q];
                t.look_v[k] = t.val[q];
            }
        }
}

// The bit reader of the reference (FillBitBuffer, gls_dng_lossless_jpeg.cpp:1315-1353):
// FF 00 is a data byte FF; FF followed by anything else is a marker, at which the reader
// steps back and supplies zero bytes; past the end of the buffer every byte reads as FF.
struct Reader {
    const uint8_t* d;
    size_t n, pos;
    uint64_t buf = 0;
    int left = 0;
    int get() { return pos < n ? d[pos++] : 0xFF; }
    void unget() {
        if (pos == 0) throw 1;
        pos--;
    }
    void fill(int need) {
        while (left < 25) {
            int c = get();
            if (c == 0xFF) {
                const int c2 = get();
                if (c2 != 0) {
                    unget();
                    unget();
                    if (left >= need) break;
                    c = 0;
                }
            }
            buf = (buf << 8) | (uint64_t)c;
            left += 8;
        }
    }
    int show8() {
        if (left < 8) fill(8);
        return (int)((buf >> (left - 8)) & 0xFF);
    }
    int bits(int k) {
        if (left < k) fill(k);
        left -= k;
        return (int)((buf >> left) & (0xFFFFu >> (16 - k)));
    }
    int bit() {
        if (!left) fill(1);
        left--;
        return (int)((buf >> left) & 1);
    }
};

int huff_decode(Reader& r, const Table& t) {
    int code = r.show8();
    if (t.look_n[code]) {
        r.left -= t.look_n[code];
        return t.look_v[code];
    }
    r.left -= 8;
    int l = 8;
    while (code > t.maxcode[l]) {
        code = (code << 1) | r.bit();
        l++;
    }
    if (l > 16) return 0;
    return t.val[t.valptr[l] + (code - t.mincode[l])];
}

int diff(Reader& r, const Table& t) {
    const int s = huff_decode(r, t);
    if (!s) return 0;
    if (s == 16) return -32768;
    if (s > 16) throw 1;
    int x = r.bits(s);
    if (x < (0x8000 >> (16 - s))) x += (-1 << s) + 1;
    return x;
}

struct Header {
    int precision = 0, width = 0, height = 0, ncomp = 0, ns = 0, ss = 0, pt = 0, restart = 0;
    int comp_id[4] = {}, scan_table[4] = {};
    size_t scan_pos = 0;
    Table tab[4];
};

struct Bytes {
    const uint8_t* d;
    size_t n, pos = 0;
    int get() {
        if (pos >= n) throw 1;
        return d[pos++];
    }
    int get2() {
        const int a = get();
        return (a << 8) | get();
    }
    void skip(size_t k) {
        if (pos + k >= n) throw 1;
        pos += k;
    }
    int marker() {
        int c;
        do {
            do c = get(); while (c != 0xFF);
            do c = get(); while (c == 0xFF);
        } while (c == 0);
        return c;
    }
};

// the marker segments up to the next frame, scan or image marker (ProcessTables)
int tables(Bytes& b, Header& h) {
    for (;;) {
        const int c = b.marker();
        if ((c >= 0xC0 && c <= 0xCF && c != 0xC4 && c != 0xCC) || c == 0xD8 || c == 0xD9 || c == 0xDA) return c;
        if (c == 0xC4) {  // DHT
            int len = b.get2() - 2;
            while (len > 0) {
                const int idx = b.get();
                if (idx < 0 || idx >= 4) throw 1;
                Table& t = h.tab[idx];
                t.present = true;
                int count = 0;
                t.bits[0] = 0;
                for (int i = 1; i <= 16; i++) count += (t.bits[i] = (uint8_t)b.get());
                if (count > 256) throw 1;
                for (int j = 0; j < count; j++) t.val[j] = (uint8_t)b.get();
                len -= 1 + 16 + count;
            }
        } else if (c == 0xDB || (c >= 0xD0 && c <= 0xD7) || c == 0x01) {
        } else if (c == 0xDD) {  // DRI
            if (b.get2() != 4) throw 1;
            h.restart = b.get2();
        } else {
            const int len = b.get2() - 2;
            b.skip((size_t)len);
        }
    }
}

Header parse(const uint8_t* d, size_t n) {
    Header h;
    Bytes b{d, n};
    if (b.get() != 0xFF || b.get() != 0xD8) throw 1;
    int c = tables(b, h);
    if (c != 0xC0 && c != 0xC1 && c != 0xC3) throw 1;
    const int len = b.get2();
    h.precision = b.get();
    h.height = b.get2();
    h.width = b.get2();
    h.ncomp = b.get();
    if (h.height <= 0 || h.width <= 0 || h.ncomp <= 0 || h.precision < 2 || h.precision > 16) throw 1;
    if (len != h.ncomp * 3 + 8) throw 1;
    int sampling[256];
    for (int i = 0; i < h.ncomp; i++) {
        const int id = b.get(), hv = b.get();
        b.get();
        if (i < 4) h.comp_id[i] = id;
        sampling[i] = hv;
    }
    for (int i = 0; i < h.ncomp; i++)
        if (sampling[i] != 0x11) throw 1;
    c = tables(b, h);
    if (c != 0xDA) throw 1;
    const int slen = b.get2() - 3;
    h.ns = b.get();
    if (slen != h.ns * 2 + 3 || h.ns < 1 || h.ns > 4) throw 1;
    for (int i = 0; i < h.ns; i++) {
        const int cc = b.get(), tt = b.get();
        int ci = 0;
        while (ci < h.ncomp && ci < 4 && h.comp_id[ci] != cc) ci++;
        if (ci >= h.ncomp || ci >= 4) throw 1;
        h.scan_table[i] = (tt >> 4) & 15;
    }
    h.ss = b.get();
    b.get();
    h.pt = b.get() & 0x0F;
    for (int i = 0; i < h.ns; i++) {
        const int t = h.scan_table[i];
        if (t > 3 || !h.tab[t].present) throw 1;
        derive(h.tab[t]);
    }
    h.scan_pos = b.pos;
    return h;
}

int predict(int ss, int left, int upper, int diag) {
    switch (ss) {
        case 0: return 0;
        case 1: return left;
        case 2: return upper;
        case 3: return diag;
        case 4: return left + upper - diag;
        case 5: return left + ((upper - diag) >> 1);
        case 6: return upper + ((left - diag) >> 1);
        case 7: return (left + upper) >> 1;
    }
    throw 1;
}

// DecodeImage: samples row by row, components interleaved; returns the sample count
long decode(const uint8_t* d, size_t n, uint16_t* out, long max_out, int info[8]) {
    Header h = parse(d, n);
    const int W = h.width, H = h.height, C = h.ns;
    const long total = (long)W * H * C;
    if (info) {
        info[0] = W, info[1] = H, info[2] = C, info[3] = h.precision;
        info[4] = h.ss, info[5] = h.pt, info[6] = h.restart, info[7] = h.ncomp;
    }
    if (total > max_out) return -2;
    Reader r{d, n, h.scan_pos};
    const int rows_per_restart = h.restart / W;
    int to_go = rows_per_restart, next_rst = 0;
    std::vector<uint16_t> prev((size_t)W * C), cur((size_t)W * C);
    auto first_row = [&](std::vector<uint16_t>& row) {
        for (int k = 0; k < C; k++)
            row[k] = (uint16_t)(diff(r, h.tab[h.scan_table[k]]) + (1 << (h.precision - h.pt - 1)));
        for (int x = 1; x < W; x++)
            for (int k = 0; k < C; k++)
                row[(size_t)x * C + k] = (uint16_t)(diff(r, h.tab[h.scan_table[k]]) + row[(size_t)(x - 1) * C + k]);
        if (rows_per_restart) to_go--;
    };
    first_row(prev);
    std::copy(prev.begin(), prev.end(), out);
    for (int y = 1; y < H; y++) {
        if (rows_per_restart) {
            if (to_go == 0) {  // ProcessRestart: drop the buffered bits, find RSTn
                r.pos -= r.left / 8;
                r.left = 0;
                r.buf = 0;
                int c;
                do {
                    do {
                        if (r.pos >= r.n) throw 1;
                        c = r.get();
                    } while (c != 0xFF);
                    do {
                        if (r.pos >= r.n) throw 1;
                        c = r.get();
                    } while (c == 0xFF);
                } while (c == 0);
                if (c != 0xD0 + next_rst) throw 1;
                next_rst = (next_rst + 1) & 7;
                to_go = rows_per_restart;
                first_row(cur);
                std::copy(cur.begin(), cur.end(), out + (size_t)y * W * C);
                std::swap(prev, cur);
                continue;
            }
            to_go--;
        }
        for (int k = 0; k < C; k++) cur[k] = (uint16_t)(diff(r, h.tab[h.scan_table[k]]) + prev[k]);
        for (int x = 1; x < W; x++)
            for (int k = 0; k < C; k++) {
                const size_t i = (size_t)x * C + k;
                const int p = predict(h.ss, cur[i - C], prev[i], prev[i - C]);
                cur[i] = (uint16_t)(diff(r, h.tab[h.scan_table[k]]) + p);
            }
        std::copy(cur.begin(), cur.end(), out + (size_t)y * W * C);
        std::swap(prev, cur);
    }
    return total;
}

// ---- test encoder ----
struct Writer {
    std::vector<uint8_t> out;
    uint64_t acc = 0;
    int nacc = 0;
    void put(int code, int len) {
        for (int i = len - 1; i >= 0; i--) {
            acc = (acc << 1) | ((code >> i) & 1);
            if (++nacc == 8) {
                const uint8_t b = (uint8_t)acc;
                out.push_back(b);
                if (b == 0xFF) out.push_back(0);
                acc = 0;
                nacc = 0;
            }
        }
    }
    void align() {  // pad with 1 bits
        while (nacc) put(1, 1);
    }
};

int category(int d) {
    int a = d < 0 ? -d : d, s = 0;
    while (a) {
        s++;
        a >>= 1;
    }
    return s;
}

// code lengths <= 16 for the used categories: Huffman lengths, then Annex K.3's
// adjustment; a reserved symbol of count 1 keeps the all-ones code out of use
void lengths(const long freq[17], uint8_t bits[17], uint8_t val[256], int* nval) {
    std::vector<std::pair<long, int>> sym;
    for (int s = 0; s <= 16; s++)
        if (freq[s]) sym.push_back({freq[s], s});
    sym.push_back({1, 256});
    const int n = (int)sym.size();
    std::vector<long> w(2 * n);
    std::vector<int> parent(2 * n, -1);
    std::vector<int> alive;
    for (int i = 0; i < n; i++) {
        w[i] = sym[i].first;
        alive.push_back(i);
    }
    int next = n;
    while (alive.size() > 1) {
        std::sort(alive.begin(), alive.end(), [&](int a, int b) { return w[a] != w[b] ? w[a] > w[b] : a > b; });
        const int a = alive.back();
        alive.pop_back();
        const int b = alive.back();
        alive.pop_back();
        w[next] = w[a] + w[b];
        parent[a] = parent[b] = next;
        alive.push_back(next++);
    }
    int count[40] = {};
    std::vector<int> len(n);
    for (int i = 0; i < n; i++) {
        int l = 0;
        for (int p = i; parent[p] >= 0; p = parent[p]) l++;
        len[i] = n == 1 ? 1 : l;
        count[len[i]]++;
    }
    for (int l = 39; l > 16; l--)  // K.3: move pairs up
        while (count[l] > 0) {
            int j = l - 2;
            while (count[j] == 0) j--;
            count[l] -= 2;
            count[l - 1]++;
            count[j + 1] += 2;
            count[j]--;
        }
    int l = 16;
    while (count[l] == 0) l--;
    count[l]--;  // drop the reserved symbol (one of the longest codes)
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const bool ra = sym[a].second == 256, rb = sym[b].second == 256;
        if (ra != rb) return rb;
        return sym[a].first != sym[b].first ? sym[a].first > sym[b].first : sym[a].second < sym[b].second;
    });
    int k = 0;
    bits[0] = 0;
    for (int q = 1; q <= 16; q++) {
        bits[q] = (uint8_t)count[q];
        for (int m = 0; m < count[q]; m++, k++) val[k] = (uint8_t)sym[order[k]].second;
    }
    *nval = k;
}

long encode(const uint16_t* src, int rows, int cols, int comps, int precision, int ss, int restart_rows,
            uint8_t* out, long cap) {
    if (comps < 1 || comps > 4 || ss < 1 || ss > 7 || precision < 2 || precision > 16) return -1;
    auto sample = [&](int y, int x, int k) { return (int)src[((size_t)y * cols + x) * comps + k]; };
    // the differences, as the decoder will predict them
    std::vector<int> dif((size_t)rows * cols * comps);
    for (int y = 0; y < rows; y++) {
        const bool first = y == 0 || (restart_rows && y % restart_rows == 0);
        for (int x = 0; x < cols; x++)
            for (int k = 0; k < comps; k++) {
                int p;
                if (first) p = x == 0 ? 1 << (precision - 1) : sample(y, x - 1, k);
                else if (x == 0) p = sample(y - 1, 0, k);
                else p = predict(ss, sample(y, x - 1, k), sample(y - 1, x, k), sample(y - 1, x - 1, k));
                int d = (sample(y, x, k) - p) & 0xFFFF;
                if (d >= 0x8000) d -= 0x10000;
                dif[((size_t)y * cols + x) * comps + k] = d;
            }
    }
    long freq[4][17] = {};
    for (size_t i = 0; i < dif.size(); i++) freq[i % comps][category(dif[i]) > 16 ? 16 : category(dif[i])]++;
    uint8_t bits[4][17], val[4][256];
    int nval[4], code[4][17] = {}, size[4][17] = {};
    for (int k = 0; k < comps; k++) {
        lengths(freq[k], bits[k], val[k], &nval[k]);
        int c = 0, p = 0;
        for (int l = 1; l <= 16; l++) {
            for (int m = 0; m < bits[k][l]; m++, p++) {
                code[k][val[k][p]] = c++;
                size[k][val[k][p]] = l;
            }
            c <<= 1;
        }
    }
    Writer w;
    auto put2 = [&](int v) {
        w.out.push_back((uint8_t)(v >> 8));
        w.out.push_back((uint8_t)v);
    };
    w.out = {0xFF, 0xD8};
    for (int k = 0; k < comps; k++) {
        w.out.push_back(0xFF);
        w.out.push_back(0xC4);
        put2(2 + 1 + 16 + nval[k]);
        w.out.push_back((uint8_t)k);
        for (int l = 1; l <= 16; l++) w.out.push_back(bits[k][l]);
        for (int m = 0; m < nval[k]; m++) w.out.push_back(val[k][m]);
    }
    if (restart_rows) {
        w.out.push_back(0xFF);
        w.out.push_back(0xDD);
        put2(4);
        put2(restart_rows * cols);
    }
    w.out.push_back(0xFF);
    w.out.push_back(0xC3);
    put2(8 + 3 * comps);
    w.out.push_back((uint8_t)precision);
    put2(rows);
    put2(cols);
    w.out.push_back((uint8_t)comps);
    for (int k = 0; k < comps; k++) {
        w.out.push_back((uint8_t)k);
        w.out.push_back(0x11);
        w.out.push_back(0);
    }
    w.out.push_back(0xFF);
    w.out.push_back(0xDA);
    put2(6 + 2 * comps);
    w.out.push_back((uint8_t)comps);
    for (int k = 0; k < comps; k++) {
        w.out.push_back((uint8_t)k);
        w.out.push_back((uint8_t)(k << 4));
    }
    w.out.push_back((uint8_t)ss);
    w.out.push_back(0);
    w.out.push_back(0);
    int rst = 0;
    for (int y = 0; y < rows; y++) {
        if (restart_rows && y > 0 && y % restart_rows == 0) {
            w.align();
            w.out.push_back(0xFF);
            w.out.push_back((uint8_t)(0xD0 + (rst++ & 7)));
        }
        for (int x = 0; x < cols; x++)
            for (int k = 0; k < comps; k++) {
                const int d = dif[((size_t)y * cols + x) * comps + k];
                const int s = category(d) > 16 ? 16 : category(d);
                w.put(code[k][s], size[k][s]);
                if (s && s < 16) w.put(d < 0 ? d + (1 << s) - 1 : d, s);
            }
    }
    w.align();
    w.out.push_back(0xFF);
    w.out.push_back(0xD9);
    if ((long)w.out.size() > cap) return -2;
    std::copy(w.out.begin(), w.out.end(), out);
    return (long)w.out.size();
}

}  // namespace lj92

extern "C" {

int oracle_threads(void) { return num_threads(); }
void oracle_set_threads(int n) { g_threads = n; }

int oracle_demosaic(const uint16_t* raw, int w, int h, int stride, oracle_params* p, int prec, uint8_t* o8, float* of,
                    oracle_taps* taps) {
    if (prec == ORACLE_F64) return demosaic<double>(raw, w, h, stride, p, prec, o8, of, taps);
    return demosaic<float>(raw, w, h, stride, p, prec, o8, of, taps);
}

int oracle_fast_demosaic(const uint16_t* raw, int w, int h, int stride, const oracle_params* p, int prec, uint8_t* o8,
                         float* of) {
    if (prec == ORACLE_F64) return fast_demosaic<double>(raw, w, h, stride, p, prec, o8, of);
    return fast_demosaic<float>(raw, w, h, stride, p, prec, o8, of);
}

int oracle_scale_raw(const uint16_t* raw, int w, int h, int stride, int bayer, const float sm[4], float black, int prec,
                     float* out) {
    Img<float> o;
    scale_raw(Pol{prec}, raw, w, h, stride, bayer, sm, black, o);
    to_float(o, out);
    return 0;
}

int oracle_raw_noise_statistics(const float* s, int w, int h, int bayer, float* mean, float* var) {
    Img<float> m, v;
    raw_noise_statistics(from_float<float>(s, w, h, 1), bayer, m, v);
    to_float(m, mean);
    to_float(v, var);
    return 0;
}

int oracle_compute_raw_nlf(const float* s, int w, int h, int bayer, float out[8]) {
    compute_raw_nlf(from_float<float>(s, w, h, 1), bayer, out);
    return 0;
}

int oracle_interpolate_green(const float* s, int w, int h, int bayer, float lv, int prec, float* g) {
    Img<float> o;
    interpolate_green(Pol{prec}, from_float<float>(s, w, h, 1), bayer, lv, o);
    to_float(o, g);
    return 0;
}

int oracle_interpolate_red_blue(const float* s, const float* g, int w, int h, int bayer, float cv, int prec, int rotate_180,
                                float* rgba) {
    Img<float> o;
    interpolate_red_blue(Pol{prec}, from_float<float>(s, w, h, 1), from_float<float>(g, w, h, 1), bayer, cv, o,
                         rotate_180 != 0);
    to_float(o, rgba);
    return 0;
}

int oracle_blend_highlights(const float* in, int w, int h, float clip, int prec, float* out) {
    Img<float> o;
    blend_highlights(Pol{prec}, from_float<float>(in, w, h, 4), clip, o);
    to_float(o, out);
    return 0;
}

int oracle_transform(const float* in, int w, int h, const float m[9], int prec, float* out) {
    Img<float> o;
    transform(Pol{prec}, from_float<float>(in, w, h, 4), m, o);
    to_float(o, out);
    return 0;
}

int oracle_despeckle(const float* in, int w, int h, const float va[3], const float vb[3], int prec, float* out) {
    Img<float> o;
    despeckle(Pol{prec}, from_float<float>(in, w, h, 4), va, vb, o);
    to_float(o, out);
    return 0;
}

int oracle_downsample(const float* in, int w, int h, int ow, int oh, int prec, float* out) {
    Img<float> o;
    downsample(Pol{prec}, from_float<float>(in, w, h, 4), ow, oh, o);
    to_float(o, out);
    return 0;
}

int oracle_noise_statistics(const float* in, int w, int h, float* out) {
    Img<float> o;
    noise_statistics(from_float<float>(in, w, h, 4), o);
    to_float(o, out);
    return 0;
}

int oracle_compute_nlf(const float* in, int w, int h, float out[6]) {
    compute_nlf(from_float<float>(in, w, h, 4), out);
    return 0;
}

int oracle_denoise_bilateral(const float* in, int w, int h, const float va[3], const float vb[3], float cb, float gb, int prec,
                             float* out) {
    Img<float> o;
    denoise_bilateral(Pol{prec}, from_float<float>(in, w, h, 4), va, vb, cb, gb, o);
    to_float(o, out);
    return 0;
}

int oracle_denoise_guided(const float* in, int w, int h, const float va[3], const float vb[3], int prec, float* out) {
    Img<float> o;
    denoise_guided(Pol{prec}, from_float<float>(in, w, h, 4), va, vb, o);
    to_float(o, out);
    return 0;
}

int oracle_guided_filter(const float* in, int w, int h, int fs, const float eps[3], int prec, float* out) {
    Img<float> o;
    guided_filter(Pol{prec}, from_float<float>(in, w, h, 4), fs, eps, o);
    to_float(o, out);
    return 0;
}

int oracle_reassemble(const float* d0, int w, int h, const float* i1, const float* d1, int w1, int h1, float sharpening,
                      const float nlf[2], int prec, float* out) {
    Img<float> o;
    reassemble(Pol{prec}, from_float<float>(d0, w, h, 4), from_float<float>(i1, w1, h1, 4), from_float<float>(d1, w1, h1, 4),
               sharpening, nlf, o);
    to_float(o, out);
    return 0;
}

int oracle_ltm_mask(const float* in, int w, int h, const float* guide, int gw, int gh, const oracle_ltm_params* ltm,
                    const float m[9], int prec, float* out) {
    Img<float> o;
    ltm_mask(Pol{prec}, from_float<float>(in, w, h, 4), from_float<float>(guide, gw, gh, 4), *ltm, m, o);
    to_float(o, out);
    return 0;
}

int oracle_convert_to_srgb(const float* in, const float* ltm, int w, int h, const float m[9], const oracle_rgb_params* rgb,
                           uint8_t* o8, float* of) {
    Img<float> mask;
    if (ltm) mask = from_float<float>(ltm, w, h, 1);
    convert_srgb(from_float<float>(in, w, h, 4), ltm ? &mask : nullptr, m, *rgb, o8, of);
    return 0;
}

int oracle_bayer_to_rgba(const float* s, int w, int h, int bayer, int prec, float* out) {
    Img<float> o;
    bayer_to_rgba(Pol{prec}, from_float<float>(s, w, h, 1), bayer, o);
    to_float(o, out);
    return 0;
}

int oracle_rgba_to_bayer(const float* rgba, int w, int h, int bayer, int prec, float* out) {
    Img<float> o(w, h, 1);
    rgba_to_bayer(Pol{prec}, from_float<float>(rgba, w / 2, h / 2, 4), bayer, o);
    to_float(o, out);
    return 0;
}

int oracle_despeckle_rgba(const float* in, int w, int h, int prec, float* out) {
    Img<float> o;
    despeckle_rgba(Pol{prec}, from_float<float>(in, w, h, 4), o);
    to_float(o, out);
    return 0;
}

int oracle_denoise_rgba(const float* in, int w, int h, const float rv[4], int prec, float* out) {
    Img<float> o;
    denoise_rgba(Pol{prec}, from_float<float>(in, w, h, 4), rv, o);
    to_float(o, out);
    return 0;
}

int oracle_fast_debayer(const float* s, int w, int h, int bayer, int prec, float* out) {
    Img<float> o;
    fast_debayer(Pol{prec}, from_float<float>(s, w, h, 1), bayer, o);
    to_float(o, out);
    return 0;
}

int oracle_regress(const float* m, const float* v, long n, int mc, int nc, float* out_ab) {
    double A[4], B[4];
    regress(n, mc, nc,
            [&](long i, double* mm, double* vv) {
                for (int c = 0; c < mc; c++) mm[c] = m[i * mc + c];
                for (int c = 0; c < nc; c++) vv[c] = v[i * nc + c];
            },
            A, B);
    for (int c = 0; c < nc; c++) {
        out_ab[c] = (float)A[c];
        out_ab[nc + c] = (float)B[c];
    }
    return 0;
}

void oracle_cam_xyz_coeff(const float cam_xyz[9], float pre_mul[3], float rgb_cam_out[9]) {
    M3 cx, rgb_cam;
    memcpy(cx, cam_xyz, sizeof(M3));
    mat_mul(cx, kXyzRgb, rgb_cam);
    float cam_white[3];
    for (int i = 0; i < 3; i++) {
        // rgb_cam * (1,1,1) via Matrix<3,1> product
        float s = 0;
        for (int k = 0; k < 3; k++) s += rgb_cam[i][k] * 1.0f;
        cam_white[i] = s;
    }
    M3 pm = {{1 / cam_white[0], 0, 0}, {0, 1 / cam_white[1], 0}, {0, 0, 1 / cam_white[2]}};
    for (int i = 0; i < 3; i++) pre_mul[i] = 1 / cam_white[i];
    M3 t, inv;
    mat_mul(pm, rgb_cam, t);
    inverse3(t, inv);
    memcpy(rgb_cam_out, inv, sizeof(M3));
}

void oracle_cam_ycbcr(const float rgb_cam[9], float out[9]) {
    M3 m, r;
    memcpy(m, rgb_cam, sizeof(M3));
    cam_ycbcr(m, r);
    memcpy(out, r, sizeof(M3));
}

void oracle_inverse3x3(const float m[9], float out[9]) {
    M3 a, r;
    memcpy(a, m, sizeof(M3));
    inverse3(a, r);
    memcpy(out, r, sizeof(M3));
}

void oracle_matmul3x3(const float a[9], const float b[9], float out[9]) {
    M3 x, y, r;
    memcpy(x, a, sizeof(M3));
    memcpy(y, b, sizeof(M3));
    mat_mul(x, y, r);
    memcpy(out, r, sizeof(M3));
}

long oracle_unpack_bits(const uint8_t* packed, long n_bytes, int bits, uint16_t* out, long max_out) {
    if (bits != 10 && bits != 12 && bits != 14 && bits != 16) return -1;
    const long n = (n_bytes * 8) / bits;
    long k = 0;
    for (; k < n && k < max_out; k++) {
        uint32_t v = 0;
        const long bit0 = k * bits;
        for (int b = 0; b < bits; b++) {
            const long bit = bit0 + b;
            const uint32_t byte = packed[bit >> 3];
            v = (v << 1) | ((byte >> (7 - (bit & 7))) & 1u);
        }
        out[k] = (uint16_t)v;
    }
    return k;
}

int oracle_auto_white_balance(const uint16_t* raw, int w, int h, int stride, const float rgb_ycbcr[9],
                               const float scale_mul[4], float white, float black, int bayer, float wb[3],
                               float* highlights) {
    if (w < 0 || h < 0 || stride < w || bayer < 0 || bayer > 3) return -1;
    awb::auto_white_balance(raw, w, h, stride, rgb_ycbcr, scale_mul, white, black, bayer, wb, highlights);
    return 0;
}

long oracle_lj92_decode(const uint8_t* data, long size, uint16_t* out, long max_out, int info[8]) {
    try {
        return lj92::decode(data, (size_t)size, out, max_out, info);
    } catch (...) {
        return -1;
    }
}

long oracle_lj92_encode(const uint16_t* src, int rows, int cols, int comps, int precision, int predictor,
                        int restart_rows, uint8_t* out, long cap) {
    return lj92::encode(src, rows, cols, comps, precision, predictor, restart_rows, out, cap);
}

int oracle_color_checker_raw_stats(const uint16_t* raw, int w, int h, int stride, float black, float white,
                                   int bayer, const int gmb[4], int rotate_180, float mean[96], float var[96]) {
    if (bayer < 0 || bayer > 3 || !gmb) return -1;
    (void)w;
    (void)h;
    calib::patch_stats(raw, stride, black, white, bayer, {gmb[0], gmb[1], gmb[2], gmb[3]}, rotate_180,
                       reinterpret_cast<float(*)[4]>(mean), reinterpret_cast<float(*)[4]>(var));
    return 0;
}

int oracle_estimate_raw_parameters(const uint16_t* raw, int w, int h, int stride, float black, float white, int bayer,
                                   const int gmb[4], int rotate_180, float cam_xyz[9], float pre_mul[3],
                                   float raw_nlf[4]) {
    float mean[24][4], var[24][4];
    if (oracle_color_checker_raw_stats(raw, w, h, stride, black, white, bayer, gmb, rotate_180, &mean[0][0],
                                       &var[0][0]) != 0)
        return -1;
    return calib::estimate(mean, var, cam_xyz, pre_mul, raw_nlf) ? 0 : -2;
}

float oracle_atan2pi(float y, float x) { return glsm::atan2pi_(y, x); }
float oracle_tanh(float x) { return glsm::tanh_(x); }
float oracle_exp2(float x) { return glsm::exp2_(x); }
float oracle_log2(float x) { return glsm::log2_(x); }
float oracle_pow(float x, float y) { return glsm::pow_(x, y); }
uint16_t oracle_f32_to_f16(float x) { return glsm::f32_to_f16_bits(x); }
float oracle_f16_to_f32(uint16_t h) { return glsm::f16_bits_to_f32(h); }

}  // extern "C"
