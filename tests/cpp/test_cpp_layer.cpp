// Drives the header-only C++ layer (include/gls_cuda.hpp) the way a port of CLImage's
// RawPipeline driver would: host gls::image<luma_pixel_16> in, RawConverter::demosaicImage,
// RawConverter::convertToRGBImage out, then autoWhiteBalance and colorCheckerRawStats on the
// same frame.  Reads a raw frame and its parameters from files written by
// tests/test_gpu_cpp_layer.py and writes the results next to them.
//
//   test_cpp_layer <dir>     reads <dir>/raw.u16 <dir>/params.txt, writes <dir>/rgb.u8,
//                            <dir>/nlf.txt, <dir>/awb.txt, <dir>/patches.f32
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/gls_cuda.hpp"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: test_cpp_layer <dir>\n";
        return 2;
    }
    const std::string dir = argv[1];
    std::ifstream pf(dir + "/params.txt");
    int w, h, bayer, levels, ltm;
    gls::DemosaicParametersT<4> p;
    pf >> w >> h >> bayer >> levels >> ltm;
    pf >> p.black_level >> p.white_level >> p.exposure_multiplier >> p.noiseLevel;
    for (auto& v : p.scale_mul) pf >> v;
    for (auto& r : p.rgb_cam)
        for (auto& v : r) pf >> v;
    for (auto& v : p.noiseModel.rawNlf) pf >> v;
    for (auto& r : p.noiseModel.pyramidNlf)
        for (auto& v : r) pf >> v;
    for (auto& d : p.denoiseParameters) pf >> d.luma >> d.chroma >> d.chromaBoost >> d.gradientBoost >> d.sharpening;
    auto& rc = p.rgbConversionParameters;
    pf >> rc.contrast >> rc.saturation >> rc.toneCurveSlope >> rc.exposureBias >> rc.blacks;
    rc.localToneMapping = ltm;
    pf >> p.ltmParameters.guidedFilterEps >> p.ltmParameters.shadows >> p.ltmParameters.highlights >>
        p.ltmParameters.detail;
    p.bayerPattern = (gls::BayerPattern)bayer;
    if (!pf || levels != 4) {
        std::cerr << "bad params\n";
        return 2;
    }
    gls::image<gls::luma_pixel_16> raw(w, h);
    {
        std::ifstream rf(dir + "/raw.u16", std::ios::binary);
        rf.read(reinterpret_cast<char*>(raw[0]), (std::streamsize)w * h * 2);
        if (!rf) {
            std::cerr << "bad raw\n";
            return 2;
        }
    }
    try {
        gls::CudaContext ctx(0);
        gls::RawConverter conv(&ctx);
        auto p_in = p;  // the parameters as read: demosaicImage updates the noise model in place
        auto* rgba = conv.demosaicImage(raw, &p, nullptr, false);
        auto rgb = gls::RawConverter::convertToRGBImage(*rgba);
        std::ofstream of(dir + "/rgb.u8", std::ios::binary);
        of.write(reinterpret_cast<const char*>((*rgb)[0]), (std::streamsize)w * h * 3);
        std::ofstream nf(dir + "/nlf.txt");
        nf.precision(9);
        for (float v : p.noiseModel.rawNlf) nf << v << " ";
        nf << "\n";
        // rotate_180: the frame turned by 180 degrees at interpolateRedBlue, as the reference does
        {
            auto* rot = conv.demosaicImage(raw, &p_in, nullptr, true);
            auto rrgb = gls::RawConverter::convertToRGBImage(*rot);
            std::ofstream rf(dir + "/rgb_rot.u8", std::ios::binary);
            rf.write(reinterpret_cast<const char*>((*rrgb)[0]), (std::streamsize)w * h * 3);
        }
        // autoWhiteBalance with the camera -> YCbCr matrix of the frame's rgb_cam
        float rgb_cam[9], cy[9];
        for (int i = 0; i < 9; i++) rgb_cam[i] = p.rgb_cam[i / 3][i % 3];
        gls::check(gls_cam_ycbcr(rgb_cam, cy), "cam_ycbcr");
        std::array<std::array<float, 3>, 3> rgb_ycbcr;
        for (int i = 0; i < 9; i++) rgb_ycbcr[i / 3][i % 3] = cy[i];
        float highlights = -1;
        const auto wb = gls::autoWhiteBalance(&ctx, raw, rgb_ycbcr, p.scale_mul, p.white_level, p.black_level,
                                              p.bayerPattern, &highlights);
        std::ofstream af(dir + "/awb.txt");
        af.precision(9);
        af << wb[0] << " " << wb[1] << " " << wb[2] << " " << highlights << "\n";
        // colorCheckerRawStats over a chart placed inside the frame
        std::array<gls::RawPatchStats, 24> stats;
        gls::colorCheckerRawStats(&ctx, raw, p.black_level, p.white_level, p.bayerPattern,
                                  gls::rectangle{12, 10, w - 30, h - 24}, false, &stats);
        std::ofstream sf(dir + "/patches.f32", std::ios::binary);
        for (const auto& s : stats) {
            sf.write(reinterpret_cast<const char*>(s.mean.data()), 16);
            sf.write(reinterpret_cast<const char*>(s.variance.data()), 16);
        }
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
