// ref_shim.cpp -- C entry points into the reference's own host code, compiled from the
// reference sources where they lie (oracle/Makefile, target _ref).  Test infrastructure:
// used only to pin the oracle's restatement of the host colour math and of the packed
// raw unpack; never shipped, never built on a machine without the reference sources.
#include <cstdint>
#include <cstring>
#include <vector>

#include "demosaic.hpp"

const char* BayerPatternName[4] = {"GRBG", "GBRG", "RGGB", "BGGR"};

// The 12/14-bit unpack routines are file-local (static inline) in gls_image_tiff.cpp,
// so that translation unit is included here; the libtiff entry points it references are
// never called from this shim.
#include "gls_image_tiff.cpp"

// colorCheckerRawStats dumps its channels as PNG files (demosaic_utils.cpp:528-531); the
// PNG writer is not part of the path, so the shim gives it an empty body.
namespace gls {
void write_png_file(const std::string&, int, int, int, int, bool, int, std::function<uint8_t*(int row)>) {}
}  // namespace gls

extern "C" {

void ref_cam_xyz_coeff(const float cam_xyz[9], float pre_mul[3], float rgb_cam[9]) {
    gls::Matrix<3, 3> cx;
    for (int i = 0; i < 9; i++) cx[i / 3][i % 3] = cam_xyz[i];
    gls::Vector<3> pm;
    const auto r = cam_xyz_coeff(&pm, cx);
    for (int i = 0; i < 3; i++) pre_mul[i] = pm[i];
    for (int i = 0; i < 9; i++) rgb_cam[i] = r[i / 3][i % 3];
}

void ref_cam_ycbcr(const float rgb_cam[9], float out[9]) {
    gls::Matrix<3, 3> m;
    for (int i = 0; i < 9; i++) m[i / 3][i % 3] = rgb_cam[i];
    const auto r = cam_ycbcr(m);
    for (int i = 0; i < 9; i++) out[i] = r[i / 3][i % 3];
}

void ref_inverse3x3(const float in[9], float out[9]) {
    gls::Matrix<3, 3> m;
    for (int i = 0; i < 9; i++) m[i / 3][i % 3] = in[i];
    const auto r = gls::inverse(m);
    for (int i = 0; i < 9; i++) out[i] = r[i / 3][i % 3];
}

void ref_matmul3x3(const float a[9], const float b[9], float out[9]) {
    gls::Matrix<3, 3> x, y;
    for (int i = 0; i < 9; i++) {
        x[i / 3][i % 3] = a[i];
        y[i / 3][i % 3] = b[i];
    }
    const auto r = x * y;
    for (int i = 0; i < 9; i++) out[i] = r[i / 3][i % 3];
}

void ref_matscale3x3(const float a[9], float s, float out[9]) {
    gls::Matrix<3, 3> x;
    for (int i = 0; i < 9; i++) x[i / 3][i % 3] = a[i];
    const auto r = x * s;
    for (int i = 0; i < 9; i++) out[i] = r[i / 3][i % 3];
}

// in_words: big-endian 16-bit words as stored in the file (the routine swaps them)
void ref_unpack12(const uint16_t* in_words, long n_words, uint16_t* out) {
    gls::unpack12BitsInto16Bits(out, in_words, (size_t)n_words);
}

void ref_unpack14(const uint16_t* in_words, long n_words, uint16_t* out) {
    gls::unpack14BitsInto16Bits(out, in_words, (size_t)n_words);
}

// autoWhiteBalance over a raw uint16 frame (row stride in pixels); the reference prints
// its result on stdout.
void ref_auto_white_balance(const uint16_t* raw, int w, int h, int stride, const float rgb_ycbcr[9],
                            const float scale_mul[4], float white, float black, int bayer, float wb[3],
                            float* highlights) {
    auto* px = reinterpret_cast<gls::luma_pixel_16*>(const_cast<uint16_t*>(raw));
    const gls::image<gls::luma_pixel_16> img(w, h, stride, std::span<gls::luma_pixel_16>(px, (size_t)stride * h));
    gls::Matrix<3, 3> m;
    for (int i = 0; i < 9; i++) m[i / 3][i % 3] = rgb_ycbcr[i];
    const gls::Vector<4> sm = {scale_mul[0], scale_mul[1], scale_mul[2], scale_mul[3]};
    const auto r = autoWhiteBalance(img, m, sm, white, black, (BayerPattern)bayer, highlights);
    for (int i = 0; i < 3; i++) wb[i] = r[i];
}

// DecodeLosslessJPEG (gls_dng_lossless_jpeg.cpp:3253-3275) over one stream: writes the
// decoded 16-bit samples (at most max_samples) and returns their count, -1 when the
// reference rejects the stream, -2 when out is too small.
long ref_lj92_decode(const uint8_t* data, long size, uint16_t* out, long max_samples) {
    try {
        std::vector<uint8_t> copy(data, data + size);
        gls::dng_stream stream(copy.data(), copy.size());
        gls::dng_spooler spooler;
        gls::DecodeLosslessJPEG(stream, spooler, 0, 0xFFFFFFFFu, false, (uint64_t)size);
        const long n = (long)(spooler.size() / 2);
        if (n > max_samples) return -2;
        memcpy(out, spooler.data(), n * 2);
        return n;
    } catch (...) {
        return -1;
    }
}

// EncodeLosslessJPEG (gls_dng_lossless_jpeg.cpp:3280-3287): predictor 1, one Huffman table
// per channel.  Returns the stream's length, or -1.
long ref_lj92_encode(const uint16_t* src, int rows, int cols, int channels, int bit_depth, uint8_t* out,
                     long capacity) {
    try {
        gls::dng_stream stream(out, (size_t)capacity);
        gls::EncodeLosslessJPEG(src, (uint32_t)rows, (uint32_t)cols, (uint32_t)channels, (uint32_t)bit_depth,
                                cols * channels, channels, stream);
        return (long)stream.Position();
    } catch (...) {
        return -1;
    }
}

// estimateRawParameters: returns 0, or -1 when the reference throws
int ref_estimate_raw_parameters(const uint16_t* raw, int w, int h, int stride, float black, float white, int bayer,
                                const int gmb[4], int rotate_180, float cam_xyz[9], float pre_mul[3],
                                float raw_nlf[4]) {
    try {
        auto* px = reinterpret_cast<gls::luma_pixel_16*>(const_cast<uint16_t*>(raw));
        const gls::image<gls::luma_pixel_16> img(w, h, stride, std::span<gls::luma_pixel_16>(px, (size_t)stride * h));
        gls::Matrix<3, 3> cx;
        gls::Vector<3> pm;
        const gls::rectangle r = {gmb[0], gmb[1], gmb[2], gmb[3]};
        const auto nlf = estimateRawParameters(img, &cx, &pm, black, white, (BayerPattern)bayer, r, rotate_180 != 0);
        for (int i = 0; i < 9; i++) cam_xyz[i] = cx[i / 3][i % 3];
        for (int i = 0; i < 3; i++) pre_mul[i] = pm[i];
        for (int i = 0; i < 4; i++) raw_nlf[i] = nlf[i];
        return 0;
    } catch (...) {
        return -1;
    }
}

}  // extern "C"
