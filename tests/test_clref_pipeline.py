"""The oracle's whole pipeline against one assembled from the reference's own kernels: the
kernels of demosaic.cl and guided_filter.cl run on the CPU (oracle/_ref/libclref.so), called
in the order and with the parameters of RawConverter::demosaicImage
(raw_converter.cpp:73-186) and PyramidalDenoise::denoise (pyramidal_denoise.cpp:104-149),
the noise models fitted by the oracle's regression on the statistics those kernels produce
(computeRawNoiseStatistics / computeNoiseStatistics feed every pixel of the statistics
image to the fit).  The fitted noise models and every RGBA8 code must equal the oracle's
demosaic: this pins the oracle's sequencing and parameter plumbing, the part of the path the
kernel-by-kernel check leaves out.  Runs where the reference sources are (skipped elsewhere)."""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import oracle_params

pytestmark = pytest.mark.skipif(orc.clref_lib() is None, reason="the reference's kernel files are not built here")

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
    raw_nlf = orc.regress(mean.reshape(-1, 4), var.reshape(-1, 4))[4:8]
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
        stats = orc.clref_noise_statistics(src).reshape(-1, 4)
        nlf.append(orc.regress(stats[:, 0], stats[:, 1:]))
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
