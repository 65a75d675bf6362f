"""The oracle's whole pipeline against one assembled from the reference's own kernels: the
kernels of demosaic.cl and guided_filter.cl run on the CPU (oracle/_ref/libclref.so), called
in the order and with the parameters of RawConverter::demosaicImage
(raw_converter.cpp:73-186) and PyramidalDenoise::denoise (pyramidal_denoise.cpp:104-149),
the noise models fitted by the reference's own computeRawNoiseStatistics /
computeNoiseStatistics (pyramidal_denoise.cpp, oracle/_ref/libref_regress.so) on the
statistics those kernels produce.  Only the order of the calls is written here; every value
comes from the reference's code.  The fitted noise models and every RGBA8 code must equal
the oracle's demosaic: this pins the oracle's sequencing, parameter plumbing and regressions,
the parts the kernel-by-kernel check leaves out.  Runs where the reference sources are
(skipped elsewhere)."""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import oracle_params

pytestmark = pytest.mark.skipif(orc.clref_lib() is None or orc.ref_regress_lib() is None,
                                reason="the reference's kernel files and host code are not built here")

F = np.float32


def nfl_multiplier(d):
    """nflMultiplier (pyramidal_denoise.cpp:97-101)."""
    luma, chroma = F(d["luma"]) * F(d["luma"]), F(d["chroma"]) * F(d["chroma"])
    return np.array([luma, chroma, chroma, luma, chroma, chroma], F)


def reference_pipeline(raw, spec):
    bayer, levels = spec["bayer_pattern"], spec["pyramid_levels"]
    h, w = raw.shape
    s = orc.clref_scale_raw(raw, bayer, spec["scale_mul"], F(spec["black_level"]) / F(65535))
    mean, var = orc.clref_raw_noise_statistics(s, bayer)
    raw_nlf = orc.ref_regress_raw(mean, var)[4:8]  # noiseModel.rawNlf = B (raw_converter.cpp:108-109)
    if spec["noise_level"] > 0.6:  # high_noise_image
        q = orc.clref_bayer_to_rgba(s, bayer)
        q = orc.clref_despeckle_rgba(q)
        q = orc.clref_denoise_rgba(q, raw_nlf)
        s = orc.clref_rgba_to_bayer(q, bayer)
    g = orc.clref_interpolate_green(s, bayer, raw_nlf[1])
    rgb = orc.clref_interpolate_red_blue(s, g, bayer, (raw_nlf[0] + raw_nlf[2]) / F(2))
    rgb = orc.clref_blend_highlights(rgb, 1.0)
    cy = gls.cam_ycbcr(np.array(spec["rgb_cam"], F).reshape(3, 3))
    y = orc.clref_transform(rgb, cy)
    np0 = np.array(spec["pyramid_nlf"][0], F)  # the call's input model, before the refit
    image = orc.clref_despeckle(y, np0[:3], np0[3:])
    # PyramidalDenoise::denoise (bilateral denoiser on every level)
    pyr, nlf, cal = [], [], []
    for i in range(levels):
        src = image if i == 0 else pyr[i - 1]
        if i < levels - 1:
            pyr.append(orc.clref_downsample(src, w >> (i + 1), h >> (i + 1)))
        nlf.append(orc.ref_regress_level(orc.clref_noise_statistics(src)))
        cal.append(nlf[i] * nfl_multiplier(spec["denoise"][i]))
    den = [None] * levels
    d = spec["denoise"][levels - 1]
    den[levels - 1] = orc.clref_denoise_bilateral(pyr[levels - 2], cal[-1][:3], cal[-1][3:], d["chromaBoost"],
                                                  d["gradientBoost"])
    for i in range(levels - 2, -1, -1):
        d = spec["denoise"][i]
        src = pyr[i - 1] if i > 0 else image
        den[i] = orc.clref_denoise_bilateral(src, cal[i][:3], cal[i][3:], d["chromaBoost"], d["gradientBoost"])
        den[i] = orc.clref_reassemble(den[i], pyr[i], den[i + 1], d["sharpening"], [cal[i][0], cal[i][3]])
    icy = (gls.inverse3x3(cy) * F(spec["exposure_multiplier"])).astype(F)
    r, l = spec["rgb"], spec["ltm"]
    if r["localToneMapping"]:
        mask = orc.clref_ltm_mask(den[0], den[3], (l["guidedFilterEps"], l["shadows"], l["highlights"], l["detail"]),
                                  icy)
    else:
        mask = np.zeros((h, w), F)
    cam = orc.clref_transform(den[0], icy)
    out = orc.clref_convert_to_srgb(cam, mask, np.array(spec["rgb_cam"], F).reshape(3, 3),
                                    (r["contrast"], r["saturation"], r["toneCurveSlope"], r["exposureBias"],
                                     r["blacks"]), r["localToneMapping"])
    return out, raw_nlf, np.array(nlf, F)


@pytest.mark.parametrize("bayer,noise_level,gain", [(2, 0.2, 2.0), (0, 0.45, 4.0), (3, 0.7, 16.0), (1, 0.2, 1.0)],
                         ids=["rggb", "grbg", "bggr_high_noise", "gbrg"])
def test_pipeline_equals_one_built_from_the_reference_kernels(bayer, noise_level, gain):
    raw, _, meta = synthetic.make_frame(160, 120, bayer=bayer, gain=gain, read_sigma=6.0, seed=80 + bayer)
    spec = configs.make_spec(meta, levels=4, noise_level=noise_level)
    out, raw_nlf, pyr_nlf = reference_pipeline(raw, spec)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))
    np.testing.assert_array_equal(raw_nlf, ref["raw_nlf"])
    np.testing.assert_array_equal(pyr_nlf, ref["pyramid_nlf"])
    np.testing.assert_array_equal(out[..., :3], ref["rgba8"][..., :3])


@pytest.mark.parametrize("seed,gain,sigma,bayer", [(3, 4.0, 3.0, 2), (5, 16.0, 12.0, 0), (7, 1.0, 2.0, 1)])
def test_oracle_regressions_equal_the_reference(seed, gain, sigma, bayer):
    """The oracle's noise-model fits (raw and per level) against the reference's own
    computeRawNoiseStatistics / computeNoiseStatistics on the same statistics images."""
    raw, _, meta = synthetic.make_frame(256, 192, bayer=bayer, gain=gain, read_sigma=sigma, seed=seed)
    spec = configs.make_spec(meta, levels=4)
    s = orc.scale_raw(raw, bayer, spec["scale_mul"], spec["black_level"] / 65535.0)
    m, v = orc.raw_noise_statistics(s, bayer)
    np.testing.assert_array_equal(orc.regress(m.reshape(-1, 4), v.reshape(-1, 4)).view(np.uint32),
                                  orc.ref_regress_raw(m, v).view(np.uint32))
    g = orc.interpolate_green(s, bayer, 1e-3)
    cy = gls.cam_ycbcr(np.array(spec["rgb_cam"], F).reshape(3, 3))
    st = orc.noise_statistics(orc.transform(orc.interpolate_red_blue(s, g, bayer, 5e-4), cy))
    np.testing.assert_array_equal(orc.regress(st.reshape(-1, 4)[:, 0], st.reshape(-1, 4)[:, 1:]).view(np.uint32),
                                  orc.ref_regress_level(st).view(np.uint32))


@pytest.mark.skipif(orc.ref_pipeline_lib() is None, reason="the reference's RawConverter is not built here")
@pytest.mark.parametrize("bayer,noise_level,gain", [(2, 0.2, 2.0), (0, 0.45, 4.0), (3, 0.7, 16.0), (1, 0.2, 1.0)],
                         ids=["rggb", "grbg", "bggr_high_noise", "gbrg"])
def test_oracle_equals_the_reference_raw_converter(bayer, noise_level, gain):
    """The reference's own RawConverter::demosaicImage (raw_converter.cpp, pyramidal_denoise.cpp,
    demosaic_utils.cpp compiled unmodified; its OpenCL bindings supplied by
    oracle/clref/ref_pipeline.cpp, each running its own demosaic.cl kernel on the CPU) against
    the oracle on the same frame: the fitted noise models and every RGBA8 code equal."""
    raw, _, meta = synthetic.make_frame(256, 192, bayer=bayer, gain=gain, read_sigma=6.0, seed=90 + bayer)
    spec = configs.make_spec(meta, levels=5, noise_level=noise_level)
    out, raw_nlf, pyr_nlf = orc.ref_raw_converter(raw, spec)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))
    np.testing.assert_array_equal(raw_nlf, ref["raw_nlf"])
    np.testing.assert_array_equal(pyr_nlf, ref["pyramid_nlf"])
    np.testing.assert_array_equal(out[..., :3], ref["rgba8"][..., :3])


@pytest.mark.skipif(orc.ref_pipeline_lib() is None, reason="the reference's RawConverter is not built here")
@pytest.mark.parametrize("bayer,noise_level", [(2, 0.2), (1, 0.7)], ids=["rggb", "gbrg_high_noise"])
def test_oracle_equals_the_reference_raw_converter_rotated(bayer, noise_level):
    """RawConverter::demosaicImage(..., rotate_180 = true): interpolateRedBlue writes pixel
    (x, y) at (w - x, h - y), so row 0 and column 0 of its image are never written and keep
    the converter's initial (zero) contents; every later stage reads the turned image.  The
    reference's own converter and the oracle agree on every RGBA8 code."""
    raw, _, meta = synthetic.make_frame(256, 192, bayer=bayer, gain=4.0, read_sigma=6.0, seed=95 + bayer)
    spec = configs.make_spec(meta, levels=5, noise_level=noise_level)
    spec["rotate_180"] = 1
    out, raw_nlf, pyr_nlf = orc.ref_raw_converter(raw, spec, rotate_180=True)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))
    np.testing.assert_array_equal(raw_nlf, ref["raw_nlf"])
    np.testing.assert_array_equal(pyr_nlf, ref["pyramid_nlf"])
    np.testing.assert_array_equal(out[..., :3], ref["rgba8"][..., :3])


@pytest.mark.skipif(orc.ref_pipeline_lib() is None, reason="the reference's RawConverter is not built here")
@pytest.mark.parametrize("width,height,bayer,noise_level,gain,sigma",
                         [(1024, 768, 2, 0.2, 2.0, 3.0), (4032, 3024, 2, 0.7, 16.0, 12.0)],
                         ids=["config1_1024x768", "bench_4032x3024_high_noise"])
def test_oracle_equals_the_reference_raw_converter_at_timed_sizes(width, height, bayer, noise_level, gain, sigma):
    """The same pin at the sizes the product is timed on: the small plain frame (1024x768
    RGGB 12-bit, read noise 3 DN, gain 2) and the bench's 4032x3024 frame at gain 16, which
    takes the high-noise raw branch.  The reference's RawConverter runs its fixed 5-level
    pyramid; about 5 s and 70 s of one CPU core."""
    raw, _, meta = synthetic.make_frame(width, height, bayer=bayer, gain=gain, read_sigma=sigma, seed=1000 + width)
    spec = configs.make_spec(meta, levels=5, noise_level=noise_level)
    out, raw_nlf, pyr_nlf = orc.ref_raw_converter(raw, spec)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))
    np.testing.assert_array_equal(raw_nlf, ref["raw_nlf"])
    np.testing.assert_array_equal(pyr_nlf, ref["pyramid_nlf"])
    np.testing.assert_array_equal(out[..., :3], ref["rgba8"][..., :3])


@pytest.mark.skipif(orc.ref_pipeline_lib(orc.F16) is None,
                    reason="the reference's RawConverter with fp16 storage is not built here")
@pytest.mark.parametrize("bayer,noise_level,gain", [(2, 0.2, 2.0), (0, 0.45, 4.0), (3, 0.7, 16.0), (1, 0.2, 1.0)],
                         ids=["rggb", "grbg", "bggr_high_noise", "gbrg"])
def test_oracle_equals_the_reference_raw_converter_with_fp16_storage(bayer, noise_level, gain):
    """The same RawConverter built with the image storage it ships with (USE_FP16_FLOATS,
    gls_image.hpp:32,189-200: every rgba_pixel_float / luma_pixel_float image in binary16).
    That build also keeps the noise-statistics images in fp16 (pyramidal_denoise.cpp:162,
    260-261), so the oracle's F16_STATS mode equals it bit for bit: noise models (NaN where a
    level has no pixel in the fit's range, on both sides) and every RGBA8 code.  The F16 mode,
    which fits on fp32 statistics as the CUDA pipeline does, stays within 2 codes of it."""
    raw, _, meta = synthetic.make_frame(256, 192, bayer=bayer, gain=gain, read_sigma=6.0, seed=90 + bayer)
    spec = configs.make_spec(meta, levels=5, noise_level=noise_level, storage=gls.STORAGE_F16)
    out, raw_nlf, pyr_nlf = orc.ref_raw_converter(raw, spec, orc.F16)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F16_STATS, want=("rgba8",))
    np.testing.assert_array_equal(raw_nlf, ref["raw_nlf"])
    np.testing.assert_array_equal(pyr_nlf, ref["pyramid_nlf"])
    np.testing.assert_array_equal(out[..., :3], ref["rgba8"][..., :3])
    f16 = orc.demosaic(raw, oracle_params(spec), orc.F16, want=("rgba8",))["rgba8"]
    assert int(np.abs(out[..., :3].astype(int) - f16[..., :3].astype(int)).max()) <= 2
