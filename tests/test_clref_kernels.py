"""The oracle's restatement of the reference's kernels against the reference's own kernel
source: CLImage's demosaic.cl and guided_filter.cl, rewritten only where C++ syntax differs
(oracle/clref/transform.py), compiled as C++ against the OpenCL-C shim oracle/clref/cl_shim.h
and run on the CPU (oracle/_ref/libclref.so, `make -C oracle clref`).  Both sides use the same
conventions for what OpenCL leaves open (gls_clmath.h: edge clamping, the linear sampler's
8-bit fractions, IEEE fp32 without contraction, the transcendental fits), so every kernel
below must give the oracle's bits exactly, on every CFA phase and at two noise levels
(half-precision arithmetic rounds every operation to binary16, as an fp16 ALU does).  Runs
where the reference sources are (skipped elsewhere).  Not covered here: the kernels the
pipeline never binds (median filters, false-colour removal, sharpening)."""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc

pytestmark = pytest.mark.skipif(orc.clref_lib() is None, reason="the reference's kernel file is not built here")


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    if a.dtype == np.float32:
        nan = np.isnan(a) & np.isnan(b)
        bad = (a.view(np.uint32) != b.view(np.uint32)) & ~nan
    else:
        bad = a != b
    assert int(bad.sum()) == 0, "%d of %d values differ" % (int(bad.sum()), a.size)


@pytest.fixture(scope="module", params=[(0, 4.0, 3.0), (1, 1.0, 2.0), (2, 16.0, 12.0), (3, 2.0, 6.0)],
                ids=["grbg", "gbrg", "rggb", "bggr"])
def frame(request):
    bayer, gain, sigma = request.param
    raw, _, meta = synthetic.make_frame(96, 72, bayer=bayer, gain=gain, read_sigma=sigma, seed=70 + bayer)
    raw[10:20, 30:50] = meta["white"]  # a clipped highlight
    spec = configs.make_spec(meta, levels=4)
    s = orc.scale_raw(raw, bayer, spec["scale_mul"], spec["black_level"] / 65535.0)
    return raw, spec, bayer, s


def test_demosaic_kernels(frame):
    raw, spec, bayer, s = frame
    same(orc.clref_scale_raw(raw, bayer, spec["scale_mul"], spec["black_level"] / 65535.0), s)
    g = orc.interpolate_green(s, bayer, 0.001)
    same(orc.clref_interpolate_green(s, bayer, 0.001), g)
    rgb = orc.interpolate_red_blue(s, g, bayer, 0.0005)
    same(orc.clref_interpolate_red_blue(s, g, bayer, 0.0005), rgb)
    # rotate_180 (demosaic.cl:310-313): pixel (x, y) written at (w - x, h - y); the writes of
    # column 0 and row 0 fall outside the image, so output column 0 and row 0 keep the
    # image's initial contents, zero on both sides
    rot = orc.interpolate_red_blue(s, g, bayer, 0.0005, rotate_180=True)
    same(orc.clref_interpolate_red_blue(s, g, bayer, 0.0005, rotate_180=True), rot)
    h, w = s.shape
    assert not rot[0].any() and not rot[:, 0].any()
    same(rot[1:, 1:], rgb[:0:-1, :0:-1][:h - 1, :w - 1])
    same(orc.clref_fast_debayer(s, bayer), orc.fast_debayer(s, bayer))
    m, v = orc.raw_noise_statistics(s, bayer)
    cm, cv = orc.clref_raw_noise_statistics(s, bayer)
    same(cm, m)
    same(cv, v)


def test_raw_domain_kernels(frame):
    _, _, bayer, s = frame
    q = orc.bayer_to_rgba(s, bayer)
    same(orc.clref_bayer_to_rgba(s, bayer), q)
    same(orc.clref_rgba_to_bayer(q, bayer), orc.rgba_to_bayer(q, bayer))
    rv = [2e-4, 1e-4, 2.5e-4, 1e-4]
    same(orc.clref_denoise_rgba(q, rv), orc.denoise_rgba(q, rv))
    same(orc.clref_despeckle_rgba(q), orc.despeckle_rgba(q))  # float4 selects per component


def test_colour_and_denoise_kernels(frame):
    _, spec, bayer, s = frame
    g = orc.interpolate_green(s, bayer, 0.001)
    rgb = orc.interpolate_red_blue(s, g, bayer, 0.0005) * 1.8  # past the clip
    hl = orc.blend_highlights(rgb, 1.0)
    same(orc.clref_blend_highlights(rgb, 1.0), hl)
    cy = gls.cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
    y = orc.transform(hl, cy)
    same(orc.clref_transform(hl, cy), y)
    same(orc.clref_noise_statistics(y), orc.noise_statistics(y))
    va, vb = [1e-5, 2e-6, 2e-6], [3e-4, 1e-4, 1e-4]
    for cb, gb in ((1.0, 1.0), (2.0, 4.0)):
        same(orc.clref_denoise_bilateral(y, va, vb, cb, gb), orc.denoise_bilateral(y, va, vb, cb, gb))
    same(orc.clref_denoise_guided(y, va, vb), orc.denoise_guided(y, va, vb))
    # despeckleImage binds despeckleLumaMedianChromaImage: fp16 reads and fp16 arithmetic
    dsa, dsb = [2e-5, 1e-5, 1e-5], [4e-4, 2e-4, 2e-4]
    same(orc.clref_despeckle(y, dsa, dsb), orc.despeckle(y, dsa, dsb))
    # GuidedFilter::filter: guided_filter.cl's six kernels in the reference's host sequence
    for fs in (3, 5):
        same(orc.clref_guided_filter(y, fs, [1e-4, 1e-5, 1e-5]), orc.guided_filter(y, fs, [1e-4, 1e-5, 1e-5]))


def test_pyramid_ltm_and_srgb_kernels(frame):
    _, spec, bayer, s = frame
    g = orc.interpolate_green(s, bayer, 0.001)
    cy = gls.cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
    y = orc.transform(orc.blend_highlights(orc.interpolate_red_blue(s, g, bayer, 0.0005), 1.0), cy)
    h, w, _ = y.shape
    d1 = orc.downsample(y, w // 2, h // 2)
    same(orc.clref_downsample(y, w // 2, h // 2), d1)
    va, vb = [1e-5, 2e-6, 2e-6], [3e-4, 1e-4, 1e-4]
    den0 = orc.denoise_bilateral(y, va, vb, 1.0, 1.0)
    den1 = orc.denoise_bilateral(d1, va, vb, 1.0, 1.0)
    for sharpening in (1.0, 1.5):
        same(orc.clref_reassemble(den0, d1, den1, sharpening, [1e-5, 3e-4]),
             orc.reassemble(den0, d1, den1, sharpening, [1e-5, 3e-4]))
    guide = orc.downsample(orc.downsample(d1, w // 4, h // 4), w // 8, h // 8)
    ltm = orc.LTMParams()
    ltm.guidedFilterEps, ltm.shadows, ltm.highlights, ltm.detail = 0.01, 1.25, 1.0, 1.1
    icy = gls.inverse3x3(cy)
    mask = orc.ltm_mask(den0, guide, ltm, icy)
    same(orc.clref_ltm_mask(den0, guide, (0.01, 1.25, 1.0, 1.1), icy), mask)
    rgbp = orc.RGBParams()
    rgbp.contrast, rgbp.saturation, rgbp.toneCurveSlope, rgbp.exposureBias, rgbp.blacks = 1.05, 1.0, 3.5, 0.0, 0.0
    rgbp.localToneMapping = 1
    cam = orc.transform(den0, icy)
    rc = np.array(spec["rgb_cam"], np.float32).reshape(3, 3)
    o8 = orc.convert_to_srgb(cam, mask, rc, rgbp)
    o8 = o8[0] if isinstance(o8, tuple) else o8
    c8 = orc.clref_convert_to_srgb(cam, mask, rc, (1.05, 1.0, 3.5, 0.0, 0.0), 1)
    same(c8[..., :3], o8[..., :3])
