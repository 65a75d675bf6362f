// gls_cuda.hpp -- header-only C++ layer over the C ABI (gls_cuda.h) that restores the
// reference's operator surface, so code written against CLImage's RAW pipeline ports by
// replacing gls::OpenCLContext with gls::CudaContext and cl_image_2d with cuda_image_2d:
//
//   gls::image<T>                 gls_image.hpp:230-453 (owned or borrowed storage,
//                                 stride in pixels, row access)
//   gls::cuda_image_2d<T>         gls_cl_image.hpp:38-107 (copyPixelsFrom/To, mapImage /
//                                 unmapImage through pinned staging, toImage)
//   free functions                demosaic_cl.hpp:23-129 (same names and arguments)
//   gls::RawConverter             raw_converter.hpp:22-62
//   autoWhiteBalance, colorCheckerRawStats, estimateRawParameters
//                                 demosaic.hpp:207-222 (raw frame on the host)
//   decodeLosslessJPEGTiles       the DNG reader's DecodeLosslessJPEG loop,
//                                 src/gls_image_tiff.cpp:369-440
//
// Errors: every failing status throws gls::cuda_error (the reference throws cl::Error).
#ifndef GLS_CUDA_HPP
#define GLS_CUDA_HPP

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "gls_cuda.h"

namespace gls {

struct cuda_error : std::runtime_error {
    gls_status status;
    cuda_error(gls_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

// ---- pixel types (gls_image.hpp:55-210) ----
template <typename T, int C>
struct basic_pixel {
    static constexpr int channels = C;
    typedef T dataType;
    std::array<T, C> v;
    T& operator[](int c) { return v[c]; }
    const T& operator[](int c) const { return v[c]; }
};

typedef basic_pixel<uint8_t, 1> luma_pixel;
typedef basic_pixel<uint8_t, 3> rgb_pixel;
typedef basic_pixel<uint8_t, 4> rgba_pixel;
typedef basic_pixel<uint16_t, 1> luma_pixel_16;
typedef basic_pixel<float, 1> luma_pixel_fp32;
typedef basic_pixel<float, 4> rgba_pixel_fp32;
typedef basic_pixel<__half, 1> luma_pixel_fp16;
typedef basic_pixel<__half, 4> rgba_pixel_fp16;

template <typename T>
struct pixel_format;
template <> struct pixel_format<luma_pixel_16> { static constexpr int value = GLS_R16_UNORM; };
template <> struct pixel_format<luma_pixel_fp32> { static constexpr int value = GLS_R_F32; };
template <> struct pixel_format<luma_pixel_fp16> { static constexpr int value = GLS_R_F16; };
template <> struct pixel_format<rgba_pixel_fp32> { static constexpr int value = GLS_RGBA_F32; };
template <> struct pixel_format<rgba_pixel_fp16> { static constexpr int value = GLS_RGBA_F16; };
template <> struct pixel_format<rgba_pixel> { static constexpr int value = GLS_RGBA8_UNORM; };
template <> struct pixel_format<rgb_pixel> { static constexpr int value = GLS_RGB8_UNORM; };

struct point {
    int x, y;
};
struct rectangle {
    int x, y, width, height;
};

enum BayerPattern { grbg = 0, gbrg = 1, rggb = 2, bggr = 3 };

inline void check(gls_status s, const char* what, gls_ctx* ctx = nullptr) {
    if (s != GLS_OK) {
        std::string msg = std::string(what) + ": " + gls_status_string(s);
        if (ctx) msg += std::string(" (") + gls_ctx_last_error(ctx) + ")";
        throw cuda_error(s, msg);
    }
}

// ---- host image (gls_image.hpp:230-453) ----
template <typename T>
class image {
   public:
    const int width, height, stride;
    typedef std::unique_ptr<image<T>> unique_ptr;

    image(int w, int h, int s)
        : width(w), height(h), stride(s), _store(std::make_unique<std::vector<T>>((size_t)s * h)),
          _data(_store->data(), _store->size()) {}
    image(int w, int h) : image(w, h, w) {}
    image(int w, int h, int s, std::span<T> data) : width(w), height(h), stride(s), _data(data) {}
    image(int w, int h, std::span<T> data) : image(w, h, w, data) {}

    T* operator[](int row) { return &_data[(size_t)stride * row]; }
    const T* operator[](int row) const { return &_data[(size_t)stride * row]; }
    std::span<T> pixels() const { return _data; }

   private:
    std::unique_ptr<std::vector<T>> _store;
    std::span<T> _data;
};

// ---- CudaContext: replaces gls::OpenCLContext ----
class CudaContext {
   public:
    explicit CudaContext(int device = 0, cudaStream_t stream = nullptr) {
        check(gls_ctx_create(device, &_ctx), "gls_ctx_create");
        gls_ctx_set_stream(_ctx, stream);
    }
    ~CudaContext() { gls_ctx_destroy(_ctx); }
    CudaContext(const CudaContext&) = delete;
    CudaContext& operator=(const CudaContext&) = delete;
    gls_ctx* ctx() const { return _ctx; }
    void synchronize() const { check(gls_ctx_synchronize(_ctx), "synchronize", _ctx); }

   private:
    gls_ctx* _ctx = nullptr;
};

// ---- device image (gls_cl_image.hpp:38-107) ----
template <typename T>
class cuda_image_2d {
   public:
    const int width, height;
    typedef std::unique_ptr<cuda_image_2d<T>> unique_ptr;

    cuda_image_2d(CudaContext* ctx, int w, int h) : width(w), height(h), _ctx(ctx) {
        if (cudaMallocPitch(&_ptr, &_pitch, (size_t)w * sizeof(T), h) != cudaSuccess)
            throw cuda_error(GLS_ERR_OUT_OF_MEMORY, "cudaMallocPitch");
    }
    cuda_image_2d(CudaContext* ctx, const image<T>& other) : cuda_image_2d(ctx, other.width, other.height) {
        copyPixelsFrom(other);
    }
    ~cuda_image_2d() { cudaFree(_ptr); }
    cuda_image_2d(const cuda_image_2d&) = delete;
    cuda_image_2d& operator=(const cuda_image_2d&) = delete;

    static unique_ptr fromImage(CudaContext* ctx, const image<T>& other) {
        return std::make_unique<cuda_image_2d<T>>(ctx, other);
    }

    // blocking copies, as enqueueWriteImage / enqueueReadImage with blocking = true
    void copyPixelsFrom(const image<T>& other) const {
        if (other.width != width || other.height != height) throw cuda_error(GLS_ERR_INVALID_SIZE, "copyPixelsFrom");
        cudaStream_t s = stream();
        check_rt(cudaMemcpy2DAsync(_ptr, _pitch, other.pixels().data(), (size_t)other.stride * sizeof(T),
                                   (size_t)width * sizeof(T), height, cudaMemcpyHostToDevice, s));
        check_rt(cudaStreamSynchronize(s));
    }
    void copyPixelsTo(image<T>* other) const {
        if (other->width != width || other->height != height) throw cuda_error(GLS_ERR_INVALID_SIZE, "copyPixelsTo");
        cudaStream_t s = stream();
        check_rt(cudaMemcpy2DAsync(other->pixels().data(), (size_t)other->stride * sizeof(T), _ptr, _pitch,
                                   (size_t)width * sizeof(T), height, cudaMemcpyDeviceToHost, s));
        check_rt(cudaStreamSynchronize(s));
    }
    typename image<T>::unique_ptr toImage() const {
        auto im = std::make_unique<image<T>>(width, height);
        copyPixelsTo(im.get());
        return im;
    }
    // mapImage: a host view of the pixels (pinned staging copy); unmapImage writes it back
    image<T> mapImage() const {
        if (!_map) {
            T* p = nullptr;
            check_rt(cudaMallocHost(&p, (size_t)width * height * sizeof(T)));
            _map.reset(p);
        }
        image<T> view(width, height, width, std::span<T>(_map.get(), (size_t)width * height));
        copyPixelsTo(&view);
        return view;
    }
    void unmapImage(const image<T>& mapped) const { copyPixelsFrom(mapped); }

    gls_image_desc desc() const {
        gls_image_desc d;
        d.ptr = _ptr;
        d.width = width;
        d.height = height;
        d.stride_bytes = (int)_pitch;
        d.format = pixel_format<T>::value;
        return d;
    }

   private:
    struct host_free {
        void operator()(T* p) const { cudaFreeHost(p); }
    };
    static void check_rt(cudaError_t e) {
        if (e != cudaSuccess) throw cuda_error(GLS_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaStream_t stream() const { return nullptr; }
    void* _ptr = nullptr;
    size_t _pitch = 0;
    CudaContext* _ctx;
    mutable std::unique_ptr<T, host_free> _map;
};

// ---- parameters (demosaic.hpp:32-81) ----
struct DenoiseParameters {
    float luma = 1.0, chroma = 1.0, chromaBoost = 1.0, gradientBoost = 1.0, sharpening = 1.0;
};
struct RGBConversionParameters {
    float contrast = 1.05, saturation = 1.0, toneCurveSlope = 3.5, exposureBias = 0, blacks = 0;
    int localToneMapping = 0;
};
struct LTMParameters {
    float guidedFilterEps = 0.01, shadows = 1.25, highlights = 1.0, detail = 1.1;
};
template <size_t levels = 5>
struct NoiseModelT {
    std::array<float, 4> rawNlf{};
    std::array<std::array<float, 6>, levels> pyramidNlf{};
};
template <size_t levels = 5>
struct DemosaicParametersT {
    BayerPattern bayerPattern = rggb;
    float black_level = 0, white_level = 65535, exposure_multiplier = 1;
    std::array<float, 4> scale_mul{1, 1, 1, 1};
    std::array<std::array<float, 3>, 3> rgb_cam{{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
    NoiseModelT<levels> noiseModel;
    std::array<DenoiseParameters, levels> denoiseParameters{};
    float noiseLevel = 0;
    RGBConversionParameters rgbConversionParameters;
    LTMParameters ltmParameters;
    int denoiseAlgorithm = GLS_DENOISE_BILATERAL;
    int storage = GLS_STORAGE_F32;

    gls_demosaic_params to_c() const {
        gls_demosaic_params p;
        std::memset(&p, 0, sizeof(p));
        p.bayer_pattern = bayerPattern;
        p.black_level = black_level;
        p.white_level = white_level;
        p.exposure_multiplier = exposure_multiplier;
        for (int i = 0; i < 4; i++) p.scale_mul[i] = scale_mul[i];
        for (int i = 0; i < 9; i++) p.rgb_cam[i] = rgb_cam[i / 3][i % 3];
        for (int i = 0; i < 4; i++) p.raw_nlf[i] = noiseModel.rawNlf[i];
        for (size_t l = 0; l < levels; l++) {
            for (int k = 0; k < 6; k++) p.pyramid_nlf[l][k] = noiseModel.pyramidNlf[l][k];
            const DenoiseParameters& d = denoiseParameters[l];
            p.denoise[l] = gls_denoise_params{d.luma, d.chroma, d.chromaBoost, d.gradientBoost, d.sharpening};
        }
        p.noise_level = noiseLevel;
        const RGBConversionParameters& r = rgbConversionParameters;
        p.rgb_conversion = gls_rgb_conversion_params{r.contrast, r.saturation, r.toneCurveSlope, r.exposureBias,
                                                     r.blacks, r.localToneMapping};
        p.ltm = gls_ltm_params{ltmParameters.guidedFilterEps, ltmParameters.shadows, ltmParameters.highlights,
                               ltmParameters.detail};
        p.pyramid_levels = (int)levels;
        p.denoise_algorithm = denoiseAlgorithm;
        p.storage = storage;
        p.rotate_180 = 0;
        return p;
    }
    void update_noise_model(const gls_demosaic_params& p) {
        for (int i = 0; i < 4; i++) noiseModel.rawNlf[i] = p.raw_nlf[i];
        for (size_t l = 0; l < levels; l++)
            for (int k = 0; k < 6; k++) noiseModel.pyramidNlf[l][k] = p.pyramid_nlf[l][k];
    }
};
typedef DemosaicParametersT<5> DemosaicParameters;

// ---- free functions (demosaic_cl.hpp:23-129) ----
template <typename TS>
void scaleRawData(CudaContext* c, const cuda_image_2d<luma_pixel_16>& raw, cuda_image_2d<TS>* scaled,
                  BayerPattern bayer, const std::array<float, 4>& scaleMul, float blackLevel) {
    const gls_image_desc a = raw.desc(), b = scaled->desc();
    check(gls_scale_raw_data(c->ctx(), &a, &b, bayer, scaleMul.data(), blackLevel), "scaleRawData", c->ctx());
}

template <typename TS>
void interpolateGreen(CudaContext* c, const cuda_image_2d<TS>& raw, cuda_image_2d<TS>* green, BayerPattern bayer,
                      float lumaVariance) {
    const gls_image_desc a = raw.desc(), b = green->desc();
    check(gls_interpolate_green(c->ctx(), &a, &b, bayer, lumaVariance), "interpolateGreen", c->ctx());
}

template <typename TS, typename T4>
void interpolateRedBlue(CudaContext* c, const cuda_image_2d<TS>& raw, const cuda_image_2d<TS>& green,
                        cuda_image_2d<T4>* rgb, BayerPattern bayer, float chromaVariance, bool rotate_180) {
    const gls_image_desc a = raw.desc(), g = green.desc(), o = rgb->desc();
    check(gls_interpolate_red_blue(c->ctx(), &a, &g, &o, bayer, chromaVariance, rotate_180), "interpolateRedBlue",
          c->ctx());
}

template <typename T4>
void blendHighlightsImage(CudaContext* c, const cuda_image_2d<T4>& in, float clip, cuda_image_2d<T4>* out) {
    const gls_image_desc a = in.desc(), b = out->desc();
    check(gls_blend_highlights(c->ctx(), &a, clip, &b), "blendHighlightsImage", c->ctx());
}

template <typename T4>
void transformImage(CudaContext* c, const cuda_image_2d<T4>& in, cuda_image_2d<T4>* out,
                    const std::array<std::array<float, 3>, 3>& m) {
    const gls_image_desc a = in.desc(), b = out->desc();
    float t[9];
    for (int i = 0; i < 9; i++) t[i] = m[i / 3][i % 3];
    check(gls_transform_image(c->ctx(), &a, &b, t), "transformImage", c->ctx());
}

template <typename T4>
void despeckleImage(CudaContext* c, const cuda_image_2d<T4>& in, const std::array<float, 3>& var_a,
                    const std::array<float, 3>& var_b, cuda_image_2d<T4>* out) {
    const gls_image_desc a = in.desc(), b = out->desc();
    check(gls_despeckle_image(c->ctx(), &a, var_a.data(), var_b.data(), &b), "despeckleImage", c->ctx());
}

template <typename T4>
void denoiseImage(CudaContext* c, const cuda_image_2d<T4>& in, const std::array<float, 3>& var_a,
                  const std::array<float, 3>& var_b, float chromaBoost, float gradientBoost, cuda_image_2d<T4>* out) {
    const gls_image_desc a = in.desc(), b = out->desc();
    check(gls_denoise_image(c->ctx(), &a, var_a.data(), var_b.data(), chromaBoost, gradientBoost, &b), "denoiseImage",
          c->ctx());
}

template <typename T4>
void resampleImage(CudaContext* c, const std::string& kernelName, const cuda_image_2d<T4>& in, cuda_image_2d<T4>* out) {
    if (kernelName != "downsampleImage") throw cuda_error(GLS_ERR_UNSUPPORTED, "resampleImage: " + kernelName);
    const gls_image_desc a = in.desc(), b = out->desc();
    check(gls_downsample_image(c->ctx(), &a, &b), "downsampleImage", c->ctx());
}

template <typename T4>
void reassembleImage(CudaContext* c, const cuda_image_2d<T4>& den0, const cuda_image_2d<T4>& img1,
                     const cuda_image_2d<T4>& den1, float sharpening, const std::array<float, 2>& nlf,
                     cuda_image_2d<T4>* out) {
    const gls_image_desc a = den0.desc(), b = img1.desc(), d = den1.desc(), o = out->desc();
    check(gls_reassemble_image(c->ctx(), &a, &b, &d, sharpening, nlf.data(), &o), "reassembleImage", c->ctx());
}

template <typename T4>
std::array<float, 6> computeNoiseStatistics(CudaContext* c, const cuda_image_2d<T4>& image) {
    const gls_image_desc a = image.desc();
    std::array<float, 6> r{};
    check(gls_compute_noise_statistics(c->ctx(), &a, r.data()), "computeNoiseStatistics", c->ctx());
    return r;
}

template <typename TS>
std::array<float, 8> computeRawNoiseStatistics(CudaContext* c, const cuda_image_2d<TS>& raw, BayerPattern bayer) {
    const gls_image_desc a = raw.desc();
    std::array<float, 8> r{};
    check(gls_compute_raw_noise_statistics(c->ctx(), &a, bayer, r.data()), "computeRawNoiseStatistics", c->ctx());
    return r;
}

// ---- raw-frame utilities (demosaic.hpp:207-222): the reference's arguments, the frame
// copied to the device; each call synchronises the context's stream ----
struct RawPatchStats {
    std::array<float, 4> mean;
    std::array<float, 4> variance;
};

inline std::array<float, 3> autoWhiteBalance(CudaContext* c, const image<luma_pixel_16>& rawImage,
                                             const std::array<std::array<float, 3>, 3>& rgb_ycbcr,
                                             const std::array<float, 4>& scale_mul, float white, float black,
                                             BayerPattern bayerPattern, float* highlights = nullptr) {
    cuda_image_2d<luma_pixel_16> raw(c, rawImage);
    const gls_image_desc r = raw.desc();
    float m[9];
    for (int i = 0; i < 9; i++) m[i] = rgb_ycbcr[i / 3][i % 3];
    std::array<float, 3> wb{};
    float hl = 0;
    check(gls_auto_white_balance(c->ctx(), &r, m, scale_mul.data(), white, black, bayerPattern, wb.data(), &hl),
          "autoWhiteBalance", c->ctx());
    if (highlights) *highlights = hl;
    return wb;
}

inline void colorCheckerRawStats(CudaContext* c, const image<luma_pixel_16>& rawImage, float black_level,
                                 float white_level, BayerPattern bayerPattern, const rectangle& gmb_position,
                                 bool rotate_180, std::array<RawPatchStats, 24>* stats) {
    cuda_image_2d<luma_pixel_16> raw(c, rawImage);
    const gls_image_desc r = raw.desc();
    const int g[4] = {gmb_position.x, gmb_position.y, gmb_position.width, gmb_position.height};
    float mean[96], var[96];
    check(gls_color_checker_raw_stats(c->ctx(), &r, black_level, white_level, bayerPattern, g, rotate_180, mean, var),
          "colorCheckerRawStats", c->ctx());
    for (int p = 0; p < 24; p++)
        for (int k = 0; k < 4; k++) {
            (*stats)[p].mean[k] = mean[4 * p + k];
            (*stats)[p].variance[k] = var[4 * p + k];
        }
}

// returns the raw noise slopes; cam_xyz and pre_mul as the reference fills them
inline std::array<float, 4> estimateRawParameters(CudaContext* c, const image<luma_pixel_16>& rawImage,
                                                  std::array<std::array<float, 3>, 3>* cam_xyz,
                                                  std::array<float, 3>* pre_mul, float black_level, float white_level,
                                                  BayerPattern bayerPattern, const rectangle& gmb_position,
                                                  bool rotate_180) {
    cuda_image_2d<luma_pixel_16> raw(c, rawImage);
    const gls_image_desc r = raw.desc();
    const int g[4] = {gmb_position.x, gmb_position.y, gmb_position.width, gmb_position.height};
    float m[9];
    std::array<float, 4> nlf{};
    check(gls_estimate_raw_parameters(c->ctx(), &r, black_level, white_level, bayerPattern, g, rotate_180, m,
                                      pre_mul->data(), nlf.data()),
          "estimateRawParameters", c->ctx());
    for (int i = 0; i < 9; i++) (*cam_xyz)[i / 3][i % 3] = m[i];
    return nlf;
}

// The DNG reader's lossless-JPEG loop (src/gls_image_tiff.cpp:369-440, DecodeLosslessJPEG per
// tile): the file's bytes, the tiles' (or the strip's) offsets and byte counts, into a device
// raw frame of the image's size.
inline void decodeLosslessJPEGTiles(CudaContext* c, const uint8_t* file, size_t file_size,
                                    const std::vector<uint64_t>& offsets, const std::vector<uint64_t>& byte_counts,
                                    int tile_width, int tile_height, cuda_image_2d<luma_pixel_16>* raw) {
    if (offsets.size() != byte_counts.size())
        throw cuda_error(GLS_ERR_INVALID_ARGUMENT, "decodeLosslessJPEGTiles: offsets and byte counts differ in number");
    const gls_image_desc r = raw->desc();
    check(gls_dng_decode_lossless_jpeg(c->ctx(), file, file_size, (int)offsets.size(), offsets.data(),
                                       byte_counts.data(), tile_width, tile_height, &r),
          "decodeLosslessJPEGTiles", c->ctx());
}

// ---- RawConverter (raw_converter.hpp:22-62) ----
class RawConverter {
   public:
    explicit RawConverter(CudaContext* ctx) : _ctx(ctx) {
        check(gls_raw_converter_create(ctx->ctx(), &_conv), "RawConverter", ctx->ctx());
    }
    ~RawConverter() { gls_raw_converter_destroy(_conv); }
    RawConverter(const RawConverter&) = delete;
    RawConverter& operator=(const RawConverter&) = delete;

    template <size_t L>
    cuda_image_2d<rgba_pixel>* demosaicImage(const image<luma_pixel_16>& rawImage, DemosaicParametersT<L>* params,
                                             const rectangle* gmb_position, bool rotate_180) {
        (void)gmb_position;  // the reference fits the noise model on every frame regardless
        if (!_raw || _raw->width != rawImage.width || _raw->height != rawImage.height) {
            _raw = std::make_unique<cuda_image_2d<luma_pixel_16>>(_ctx, rawImage.width, rawImage.height);
            _rgb = std::make_unique<cuda_image_2d<rgba_pixel>>(_ctx, rawImage.width, rawImage.height);
        }
        _raw->copyPixelsFrom(rawImage);
        gls_demosaic_params p = params->to_c();
        p.rotate_180 = rotate_180 ? 1 : 0;
        const gls_image_desc r = _raw->desc(), o = _rgb->desc();
        check(gls_raw_converter_demosaic(_conv, &r, &p, &o, 0), "RawConverter::demosaicImage", _ctx->ctx());
        params->update_noise_model(p);
        return _rgb.get();
    }

    template <size_t L>
    cuda_image_2d<rgba_pixel>* fastDemosaicImage(const image<luma_pixel_16>& rawImage,
                                                 const DemosaicParametersT<L>& params) {
        _raw = std::make_unique<cuda_image_2d<luma_pixel_16>>(_ctx, rawImage.width, rawImage.height);
        _fast = std::make_unique<cuda_image_2d<rgba_pixel>>(_ctx, rawImage.width / 2, rawImage.height / 2);
        _raw->copyPixelsFrom(rawImage);
        gls_demosaic_params p = params.to_c();
        const gls_image_desc r = _raw->desc(), o = _fast->desc();
        check(gls_raw_converter_fast_demosaic(_conv, &r, &p, &o), "RawConverter::fastDemosaicImage", _ctx->ctx());
        return _fast.get();
    }

    static std::unique_ptr<image<rgb_pixel>> convertToRGBImage(const cuda_image_2d<rgba_pixel>& rgba) {
        auto rgb = std::make_unique<image<rgb_pixel>>(rgba.width, rgba.height);
        auto mapped = rgba.mapImage();
        for (int y = 0; y < rgba.height; y++)
            for (int x = 0; x < rgba.width; x++) {
                const auto& p = mapped[y][x];
                (*rgb)[y][x] = rgb_pixel{{p[0], p[1], p[2]}};
            }
        return rgb;
    }

    gls_raw_converter* handle() const { return _conv; }

   private:
    CudaContext* _ctx;
    gls_raw_converter* _conv = nullptr;
    std::unique_ptr<cuda_image_2d<luma_pixel_16>> _raw;
    std::unique_ptr<cuda_image_2d<rgba_pixel>> _rgb, _fast;
};

}  // namespace gls

#endif  // GLS_CUDA_HPP
