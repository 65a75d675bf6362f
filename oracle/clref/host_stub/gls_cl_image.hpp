// gls_cl_image.hpp (stand-in) -- the few members of gls::cl_image_2d and gls::OpenCLContext
// that the reference's pipeline host code (pyramidal_denoise.cpp and its headers) uses,
// backed by host memory, so that its noise-model regressions compile and run on the CPU
// without an OpenCL runtime.  TEST INFRASTRUCTURE ONLY (oracle/clref/ref_regress.cpp).
#ifndef GLS_CL_IMAGE_STUB_HPP
#define GLS_CL_IMAGE_STUB_HPP

#include <cstring>
#include <memory>
#include <span>
#include <vector>

#include "gls_image.hpp"

namespace cl {
struct Context {};
}  // namespace cl

namespace gls {

class OpenCLContext {
   public:
    cl::Context clContext() { return {}; }
};

template <typename T>
class cl_image_2d {
   public:
    typedef std::unique_ptr<cl_image_2d<T>> unique_ptr;
    const int width, height;
    mutable std::vector<T> pixels;

    // A new image starts at zero.  The pixel types' own default constructors leave their
    // channels unset, and the reference reads texels that no kernel has written in one
    // place: with rotate_180, interpolateRedBlue never writes row 0 and column 0 of its
    // output (demosaic.cl:310-313), whose contents OpenCL leaves undefined; zero is the
    // convention the oracle and the CUDA path share.
    cl_image_2d(cl::Context, int w, int h) : width(w), height(h), pixels((size_t)w * h) {
        std::memset(static_cast<void*>(pixels.data()), 0, pixels.size() * sizeof(T));
    }
    image<T> mapImage() const { return image<T>(width, height, std::span<T>(pixels.data(), pixels.size())); }
    void copyPixelsFrom(const image<T>& other) const {
        for (int y = 0; y < height; y++)
            for (int x = 0; x < width; x++) pixels[(size_t)y * width + x] = other[y][x];
    }
    void unmapImage(const image<T>&) const {}
};

}  // namespace gls

#endif
