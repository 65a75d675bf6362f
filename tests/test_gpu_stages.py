"""Parity of every single-stage CUDA kernel (called through the C ABI) with the oracle.

Inputs are real intermediate images: the oracle runs the pipeline on a seeded synthetic
frame and its taps feed each stage on both sides.  The comparison is bit-exact: the
kernels and the oracle evaluate the same operations in the same order under the
conventions of gls_clmath.h.
"""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import mismatch, oracle_params

pytestmark = pytest.mark.gpu

SIZES = [(136, 104), (64, 48)]
ODD_SIZES = [(67, 45), (5, 3)]


def dev(a, half=False):
    import torch
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint16:
        return torch.from_numpy(a).cuda()
    return torch.from_numpy(a.astype(np.float16 if half else np.float32)).cuda()


def host(t):
    return t.float().cpu().numpy() if t.dtype in (__import__("torch").float16,) else t.cpu().numpy()


def empty(shape, half=False, dtype=None):
    import torch
    return torch.empty(shape, dtype=dtype or (torch.float16 if half else torch.float32), device="cuda")


def rnd_half(a, half):
    return a.astype(np.float16).astype(np.float32) if half else a.astype(np.float32)


@pytest.fixture(scope="module", params=[(136, 104, 2), (64, 48, 0), (136, 104, 1), (64, 48, 3)],
                ids=lambda p: "%dx%d-cfa%d" % p)
def frame(request):
    w, h, bayer = request.param
    raw, scene, meta = synthetic.make_frame(w, h, bayer=bayer, seed=w * 7 + bayer)
    spec = configs.make_spec(meta, levels=4)
    taps = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgbaf",),
                        taps=("scaled_raw", "green", "linear_rgb", "ycbcr", "level0", "denoised0"))
    return dict(raw=raw, spec=spec, taps=taps, bayer=bayer)


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_scale_raw(ctx, frame, half):
    import torch
    raw, spec, bayer = frame["raw"], frame["spec"], frame["bayer"]
    h, w = raw.shape
    black = np.float32(spec["black_level"]) / np.float32(0xFFFF)
    out = empty((h, w), half)
    ctx.scaleRawData(dev(raw), out, bayer, spec["scale_mul"], black)
    torch.cuda.synchronize()
    ref = orc.scale_raw(raw, bayer, spec["scale_mul"], black, orc.F16 if half else orc.F32)
    assert mismatch(host(out), ref) == 0


def test_unorm16_read_is_the_division(ctx):
    """Every uint16 code through scaleRawData with unit scale and zero black: the device's
    UNORM16 read (reciprocal and one correction step) equals the correctly rounded division
    v / 65535 for all 65536 codes."""
    import torch
    raw = np.arange(65536, dtype=np.uint16).reshape(256, 256)
    out = empty((256, 256), False)
    ctx.scaleRawData(dev(raw), out, 2, [1.0, 1.0, 1.0, 1.0], np.float32(0.0))
    torch.cuda.synchronize()
    want = raw.astype(np.float32) / np.float32(65535.0)
    assert np.array_equal(host(out).view(np.uint32), want.view(np.uint32))


def test_raw_noise_statistics(ctx, frame):
    import torch
    s = frame["taps"]["scaled_raw"]
    h, w = s.shape
    mean, var = empty((h // 2, w // 2, 4)), empty((h // 2, w // 2, 4))
    ctx.rawNoiseStatistics(dev(s), frame["bayer"], mean, var)
    torch.cuda.synchronize()
    rm, rv = orc.raw_noise_statistics(s, frame["bayer"])
    assert mismatch(host(mean), rm) == 0
    assert mismatch(host(var), rv) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_compute_raw_noise_statistics(ctx, frame, half):
    s = rnd_half(frame["taps"]["scaled_raw"], half)
    got = ctx.computeRawNoiseStatistics(dev(s, half), frame["bayer"])
    ref = orc.compute_raw_nlf(s, frame["bayer"])
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_interpolate_green(ctx, frame, half):
    import torch
    s = rnd_half(frame["taps"]["scaled_raw"], half)
    h, w = s.shape
    g = empty((h, w), half)
    ctx.interpolateGreen(dev(s, half), g, frame["bayer"], 3.7e-4)
    torch.cuda.synchronize()
    ref = orc.interpolate_green(s, frame["bayer"], 3.7e-4, orc.F16 if half else orc.F32)
    assert mismatch(host(g), ref) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_interpolate_red_blue(ctx, frame, half):
    import torch
    s = rnd_half(frame["taps"]["scaled_raw"], half)
    g = rnd_half(frame["taps"]["green"], half)
    h, w = s.shape
    out = empty((h, w, 4), half)
    ctx.interpolateRedBlue(dev(s, half), dev(g, half), out, frame["bayer"], 3.3e-4)
    torch.cuda.synchronize()
    ref = orc.interpolate_red_blue(s, g, frame["bayer"], 3.3e-4, orc.F16 if half else orc.F32)
    assert mismatch(host(out), ref) == 0
    # rotate_180 (demosaic.cl:310-313): the output turned by 180 degrees, row 0 and column 0 zero
    rot = empty((h, w, 4), half)
    rot.fill_(7.0)
    ctx.interpolateRedBlue(dev(s, half), dev(g, half), rot, frame["bayer"], 3.3e-4, rotate_180=True)
    torch.cuda.synchronize()
    ref_rot = orc.interpolate_red_blue(s, g, frame["bayer"], 3.3e-4, orc.F16 if half else orc.F32, rotate_180=True)
    assert mismatch(host(rot), ref_rot) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_rgba_pointwise(ctx, frame, half):
    import torch
    lin = rnd_half(frame["taps"]["linear_rgb"], half)
    h, w, _ = lin.shape
    prec = orc.F16 if half else orc.F32
    out = empty((h, w, 4), half)
    ctx.blendHighlightsImage(dev(lin, half), 1.0, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.blend_highlights(lin, 1.0, prec)) == 0
    m = np.array([[0.3, 0.5, 0.2], [-0.1, -0.4, 0.5], [0.5, -0.45, -0.05]], np.float32)
    ctx.transformImage(dev(lin, half), out, m)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.transform(lin, m, prec)) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_despeckle(ctx, frame, half):
    import torch
    y = rnd_half(frame["taps"]["ycbcr"], half)
    h, w, _ = y.shape
    out = empty((h, w, 4), half)
    va, vb = [2.1e-4, 1e-8, 8.2e-6], [2.6e-4, 3.9e-5, 9.0e-6]
    ctx.despeckleImage(dev(y, half), va, vb, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.despeckle(y, va, vb, orc.F16 if half else orc.F32)) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_downsample_and_stats(ctx, frame, half):
    import torch
    l0 = rnd_half(frame["taps"]["level0"], half)
    h, w, _ = l0.shape
    prec = orc.F16 if half else orc.F32
    for ow, oh in ((w // 2, h // 2), ((w + 1) // 3, (h + 1) // 3)):
        out = empty((oh, ow, 4), half)
        ctx.downsampleImage(dev(l0, half), out)
        torch.cuda.synchronize()
        assert mismatch(host(out), orc.downsample(l0, ow, oh, prec)) == 0
    st = empty((h, w, 4))
    ctx.noiseStatistics(dev(l0, half), st)
    torch.cuda.synchronize()
    assert mismatch(host(st), orc.noise_statistics(l0)) == 0
    np.testing.assert_array_equal(ctx.computeNoiseStatistics(dev(l0, half)), orc.compute_nlf(l0))


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
@pytest.mark.parametrize("boost", [(1.0, 1.0), (4.0, 2.0)], ids=["plain", "boosted"])
def test_denoise(ctx, frame, half, boost):
    import torch
    l0 = rnd_half(frame["taps"]["level0"], half)
    h, w, _ = l0.shape
    prec = orc.F16 if half else orc.F32
    va, vb = [3e-6, 2e-7, 5e-7], [4e-6, 1e-6, 1.2e-6]
    out = empty((h, w, 4), half)
    ctx.denoiseImage(dev(l0, half), va, vb, boost[0], boost[1], out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.denoise_bilateral(l0, va, vb, boost[0], boost[1], prec)) == 0
    ctx.denoiseImageGuided(dev(l0, half), va, vb, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.denoise_guided(l0, va, vb, prec)) == 0


@pytest.mark.parametrize("seed", range(4))
def test_denoise_taps_at_the_edge(ctx, seed):
    """Sample differences of sigma * sqrt(2) * (1 + t) with |t| of a few ulp put many taps of
    the bilateral filter on (or next to) the edge of its 0/1 weight, where the kernel's fast
    decision must hand over to the literal evaluation."""
    import torch
    rng = np.random.default_rng(100 + seed)
    h, w = 32, 48
    sig = np.float32(0.01)
    va, vb = [float(sig * sig), 2.5e-5, 4e-5], [0.0, 0.0, 0.0]
    img = np.zeros((h, w, 4), np.float32)
    t = rng.uniform(-6e-7, 6e-7, (h, w)).astype(np.float32)
    delta = (sig * np.float32(np.sqrt(2.0)) * (np.float32(1.0) + t)).astype(np.float32)
    img[..., 0] = np.float32(0.3) + np.where(rng.random((h, w)) < 0.5, delta, np.float32(0.0))
    img[..., 1] = np.float32(0.2) + np.where(rng.random((h, w)) < 0.3, np.float32(0.005) * (1 + t), np.float32(0.0))
    img[..., 2] = np.float32(0.25)
    out = empty((h, w, 4))
    for boost in ((1.0, 1.0), (1.0, 2.0)):
        ctx.denoiseImage(dev(img), va, vb, boost[0], boost[1], out)
        torch.cuda.synchronize()
        assert mismatch(host(out), orc.denoise_bilateral(img, va, vb, boost[0], boost[1])) == 0


@pytest.mark.parametrize("seed", range(3))
def test_denoise_raw_rgba_zeros_and_edges(ctx, seed):
    """denoiseRawRGBA where planes are zero (sigma = 0: the tap weight comes from NaN or
    infinite quotients) and where sample differences sit on the weight's edge."""
    import torch
    rng = np.random.default_rng(200 + seed)
    h, w = 24, 40
    rv = [1e-4, 2e-4, 1.5e-4, 3e-4]
    img = np.zeros((h, w, 4), np.float32)
    base = np.float32(0.25)
    sig0 = np.sqrt(np.float32(rv[0]) * base).astype(np.float32)
    t = rng.uniform(-8e-7, 8e-7, (h, w)).astype(np.float32)
    img[..., 0] = base + np.where(rng.random((h, w)) < 0.5, sig0 * (np.float32(1) + t), np.float32(0))
    img[..., 1] = np.where(rng.random((h, w)) < 0.4, np.float32(0), rng.uniform(0, 0.3, (h, w)).astype(np.float32))
    img[..., 2] = np.where(rng.random((h, w)) < 0.7, np.float32(0), np.float32(0.125))
    img[..., 3] = np.float32(0.3)
    out = empty((h, w, 4))
    ctx.denoiseRawRGBAImage(dev(img), rv, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.denoise_rgba(img, rv)) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_guided_filter(ctx, frame, half):
    import torch
    l0 = rnd_half(frame["taps"]["level0"], half)
    h, w, _ = l0.shape
    out = empty((h, w, 4), half)
    eps = [4e-6, 1e-6, 1.2e-6]
    ctx.guidedFilter(dev(l0, half), 5, eps, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.guided_filter(l0, 5, eps, orc.F16 if half else orc.F32)) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
@pytest.mark.parametrize("sharpening", [1.0, 1.5])
def test_reassemble(ctx, frame, half, sharpening):
    import torch
    l0 = rnd_half(frame["taps"]["level0"], half)
    h, w, _ = l0.shape
    prec = orc.F16 if half else orc.F32
    i1 = orc.downsample(l0, w // 2, h // 2, prec)
    d1 = rnd_half(i1 * np.float32(0.98) + np.float32(0.001), half)
    d0 = rnd_half(orc.denoise_bilateral(l0, [3e-6] * 3, [4e-6] * 3, 1.0, 1.0, prec), half)
    out = empty((h, w, 4), half)
    nlf = [3e-6, 4e-6]
    ctx.reassembleImage(dev(d0, half), dev(i1, half), dev(d1, half), sharpening, nlf, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.reassemble(d0, i1, d1, sharpening, nlf, prec)) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_ltm_and_srgb(ctx, frame, half):
    import torch
    den = rnd_half(frame["taps"]["denoised0"], half)
    h, w, _ = den.shape
    prec = orc.F16 if half else orc.F32
    guide = orc.downsample(orc.downsample(orc.downsample(den, w // 2, h // 2, prec), w // 4, h // 4, prec), w // 8, h // 8,
                           prec)
    spec = frame["spec"]
    cy = orc.cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
    icy = orc.inverse3x3(cy)
    ltm = gls.LTMParams(**spec["ltm"])
    mask = empty((h, w), half)
    ctx.localToneMappingMask(dev(den, half), dev(guide, half), ltm, icy, mask)
    torch.cuda.synchronize()
    ref_mask = orc.ltm_mask(den, guide, orc.LTMParams(**spec["ltm"]), icy, prec)
    assert mismatch(host(mask), ref_mask) == 0
    cam = orc.transform(den, icy, prec)
    for rgbp in (configs.RGB_LTM, configs.RGB_DEFAULT):
        rp = gls.RGBConversionParams(**rgbp)
        o8 = empty((h, w, 4), dtype=torch.uint8)
        of = empty((h, w, 4))
        m = dev(ref_mask, half) if rgbp["localToneMapping"] else None
        ctx.convertTosRGB(dev(cam, half), m, o8, spec["rgb_cam"], rp)
        ctx.convertTosRGB(dev(cam, half), m, of, spec["rgb_cam"], rp)
        torch.cuda.synchronize()
        r8, rf = orc.convert_to_srgb(cam, ref_mask if rgbp["localToneMapping"] else None,
                                     np.array(spec["rgb_cam"]), orc.RGBParams(**rgbp))
        assert mismatch(host(o8), r8) == 0
        assert mismatch(host(of), rf) == 0


@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_high_noise_raw_branch(ctx, frame, half):
    import torch
    s = rnd_half(frame["taps"]["scaled_raw"], half)
    h, w = s.shape
    prec = orc.F16 if half else orc.F32
    rgba = empty((h // 2, w // 2, 4), half)
    ctx.bayerToRawRGBA(dev(s, half), rgba, frame["bayer"])
    torch.cuda.synchronize()
    r_rgba = orc.bayer_to_rgba(s, frame["bayer"], prec)
    assert mismatch(host(rgba), r_rgba) == 0
    desp = empty((h // 2, w // 2, 4), half)
    ctx.despeckleRawRGBAImage(rgba, desp)
    torch.cuda.synchronize()
    r_desp = orc.despeckle_rgba(r_rgba, prec)
    assert mismatch(host(desp), r_desp) == 0
    rv = [3.4e-4, 3.7e-4, 9.4e-4, 3.7e-4]
    den = empty((h // 2, w // 2, 4), half)
    ctx.denoiseRawRGBAImage(desp, rv, den)
    torch.cuda.synchronize()
    r_den = orc.denoise_rgba(r_desp, rv, prec)
    assert mismatch(host(den), r_den) == 0
    back = empty((h, w), half)
    ctx.rawRGBAToBayer(den, back, frame["bayer"])
    torch.cuda.synchronize()
    assert mismatch(host(back), orc.rgba_to_bayer(r_den, frame["bayer"], prec)) == 0
    fd = empty((h // 2, w // 2, 4), half)
    ctx.fastDebayer(dev(s, half), fd, frame["bayer"])
    torch.cuda.synchronize()
    assert mismatch(host(fd), orc.fast_debayer(s, frame["bayer"], prec)) == 0


@pytest.mark.parametrize("w,h", ODD_SIZES)
def test_odd_sizes_rgba_stages(ctx, w, h):
    import torch
    rng = np.random.default_rng(w * 31 + h)
    img = rng.uniform(-0.05, 1.1, (h, w, 4)).astype(np.float32)
    img[..., 3] = 0
    out = empty((h, w, 4))
    va, vb = [3e-4, 2e-5, 5e-5], [4e-4, 1e-4, 1.2e-4]
    ctx.denoiseImage(dev(img), va, vb, 2.0, 2.0, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.denoise_bilateral(img, va, vb, 2.0, 2.0)) == 0
    ctx.despeckleImage(dev(img), va, vb, out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.despeckle(img, va, vb)) == 0
    ctx.guidedFilter(dev(img), 3, [4e-4, 1e-4, 1.2e-4], out)
    torch.cuda.synchronize()
    assert mismatch(host(out), orc.guided_filter(img, 3, [4e-4, 1e-4, 1.2e-4])) == 0
    ow, oh = max(1, w // 2), max(1, h // 2)
    ds = empty((oh, ow, 4))
    ctx.downsampleImage(dev(img), ds)
    torch.cuda.synchronize()
    assert mismatch(host(ds), orc.downsample(img, ow, oh)) == 0


def test_unpack(ctx):
    import torch
    rng = np.random.default_rng(5)
    for bits in (10, 12, 14, 16):
        samples = rng.integers(0, 1 << bits, 4099, dtype=np.uint32).astype(np.uint16)
        packed = synthetic.pack_bits(samples, bits)
        pk = torch.from_numpy(np.frombuffer(packed, np.uint8).copy()).cuda()
        out = torch.empty(samples.size, dtype=torch.uint16, device="cuda")
        ctx.unpackRawBits(pk, bits, out)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), samples)
        np.testing.assert_array_equal(orc.unpack_bits(packed, bits), samples)


def test_exact_shortcuts_selftest(ctx):
    """The kernels replace some literal operations by exact equivalents (shared-divisor
    division, clamped smoothstep, squared-length edge tests, hardware binary16 rounding);
    over 2^26 random and adversarial inputs each must equal the literal operation."""
    for seed in (1, 2):
        assert ctx.selftest(1 << 26, seed) == [0, 0, 0, 0]


def test_fast_reciprocal_is_correctly_rounded(ctx):
    """The shared-divisor division takes its reciprocal from the hardware approximation and
    one Newton step; for every divisor of its range (2^-60 <= |d| < 2^31, 1.5 G values) that
    equals the correctly rounded reciprocal, which the Markstein correction needs."""
    assert ctx.selftest_reciprocal() == 0


def test_invalid_arguments(ctx):
    import torch
    raw = torch.zeros((9, 8), dtype=torch.uint16, device="cuda")
    out = empty((9, 8))
    with pytest.raises(gls.GlsError) as e:
        ctx.scaleRawData(raw, out, 2, [1, 1, 1, 1], 0.0)
    assert e.value.status == 2
    raw = torch.zeros((8, 8), dtype=torch.uint16, device="cuda")
    with pytest.raises(gls.GlsError):
        ctx.scaleRawData(raw, empty((8, 8)), 7, [1, 1, 1, 1], 0.0)
    with pytest.raises(gls.GlsError):
        ctx.interpolateRedBlue(empty((8, 8)), empty((8, 8)), empty((8, 6, 4)), 2, 1e-4, rotate_180=True)
    with pytest.raises(gls.GlsError):
        ctx.unpackRawBits(torch.zeros(3, dtype=torch.uint8, device="cuda"), 11, torch.zeros(2, dtype=torch.uint16,
                                                                                            device="cuda"))
