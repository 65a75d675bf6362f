"""Whole-pipeline parity: RawConverter::demosaicImage on the GPU (through the C ABI) against
the oracle on the same seeded synthetic frames, for every CFA phase, both storage
precisions, the high-noise raw branch, the three denoisers and 4-6 pyramid levels.

Pass bar: the fitted noise model, every intermediate tap and the float output equal the
oracle's exactly; the RGBA8 product differs by at most 1 code (0.5 LSB of the float
result before quantisation) -- in practice it is identical.
"""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import LINEAR_MAX_ABS, U8_MAX_LSB, max_abs, mismatch, oracle_params

pytestmark = pytest.mark.gpu

TAPS = {0: "scaled_raw", 1: "green", 2: "level0", 3: "denoised0", 4: "ltm_mask"}


@pytest.fixture(params=[0, 1], ids=["fused", "staged"])
def mode(request):
    return request.param


def run_gpu(ctx, raw, spec, out_float=False, taps=True, mode=0):
    import torch
    h, w = raw.shape
    conv = gls.RawConverter(ctx)
    conv.setMode(mode)
    bufs = {}
    if taps:
        for k, name in TAPS.items():
            shape = (h, w) if name in ("scaled_raw", "green", "ltm_mask") else (h, w, 4)
            bufs[name] = torch.zeros(shape, dtype=torch.float32, device="cuda")
            conv.setTap(k, bufs[name])
    p = configs.to_gls_params(spec)
    out = torch.empty((h, w, 4), dtype=torch.float32 if out_float else torch.uint8, device="cuda")
    conv.demosaicImage(torch.from_numpy(raw).cuda(), p, out)
    torch.cuda.synchronize()
    res = {"out": out.cpu().numpy(), "raw_nlf": np.array(p.raw_nlf[:], np.float32),
           "pyramid_nlf": np.array([p.pyramid_nlf[i][:] for i in range(spec["pyramid_levels"])], np.float32)}
    for k, v in bufs.items():
        res[k] = v.cpu().numpy()
    conv.close()
    return res


def check(ctx, raw, spec, out_float=False, mode=0):
    prec = {gls.STORAGE_F16: orc.F16, gls.STORAGE_F16_STATS: orc.F16_STATS}.get(spec["storage"], orc.F32)
    ref = orc.demosaic(raw, oracle_params(spec), prec, want=("rgbaf" if out_float else "rgba8",),
                       taps=tuple(TAPS.values()))
    got = run_gpu(ctx, raw, spec, out_float, mode=mode)
    np.testing.assert_array_equal(got["raw_nlf"], ref["raw_nlf"])
    np.testing.assert_array_equal(got["pyramid_nlf"], ref["pyramid_nlf"])
    for name in TAPS.values():
        if name == "ltm_mask" and not spec["rgb"]["localToneMapping"]:
            continue
        assert mismatch(got[name], ref[name]) == 0, name
    if out_float:
        assert max_abs(got["out"], ref["rgbaf"]) <= LINEAR_MAX_ABS
        assert mismatch(got["out"], ref["rgbaf"]) == 0
    else:
        d = np.abs(got["out"].astype(int) - ref["rgba8"].astype(int))
        assert d.max() <= U8_MAX_LSB
        assert int((d > 0).sum()) == 0
    return got, ref


@pytest.mark.parametrize("bayer", [0, 1, 2, 3], ids=["grbg", "gbrg", "rggb", "bggr"])
def test_pipeline_cfa_phases(ctx, bayer, mode):
    raw, _, meta = synthetic.make_frame(256, 192, bayer=bayer, seed=100 + bayer)
    check(ctx, raw, configs.make_spec(meta, levels=4), mode=mode)


def test_pipeline_config1_float_output(ctx, mode):
    c = configs.CONFIG1
    raw, _, meta = synthetic.make_frame(c["width"], c["height"], bayer=c["bayer"], bits=c["bits"], black=c["black"],
                                        white=c["white"], wb=c["wb"], read_sigma=3.0, gain=2.0, seed=1)
    check(ctx, raw, configs.make_spec(meta, levels=4), out_float=True, mode=mode)


def test_pipeline_fp16_storage(ctx, mode):
    raw, _, meta = synthetic.make_frame(320, 240, bayer=0, bits=14, seed=3)
    check(ctx, raw, configs.make_spec(meta, levels=6, storage=gls.STORAGE_F16), mode=mode)


@pytest.mark.parametrize("bayer,noise_level,gain", [(0, 0.2, 2.0), (3, 0.7, 16.0)], ids=["grbg", "bggr_high_noise"])
def test_pipeline_fp16_statistics(ctx, mode, bayer, noise_level, gain):
    """GLS_STORAGE_F16_STATS: fp16 images and the noise statistics rounded to fp16 before the
    fits, as the reference ships -- equal to the oracle's F16_STATS mode, which the reference's
    own RawConverter built with fp16 storage equals on the CPU (test_clref_pipeline.py)."""
    raw, _, meta = synthetic.make_frame(256, 192, bayer=bayer, gain=gain, read_sigma=6.0, seed=150 + bayer)
    check(ctx, raw, configs.make_spec(meta, levels=5, storage=gls.STORAGE_F16_STATS, noise_level=noise_level),
          mode=mode)


def test_pipeline_high_noise_branch(ctx, mode):
    raw, _, meta = synthetic.make_frame(256, 192, bayer=2, gain=16.0, read_sigma=12.0, seed=4)
    check(ctx, raw, configs.make_spec(meta, levels=5, noise_level=0.7), mode=mode)


@pytest.mark.parametrize("algo", [1, 2], ids=["guided_fast", "guided_precise"])
def test_pipeline_guided_denoisers(ctx, algo, mode):
    raw, _, meta = synthetic.make_frame(192, 128, bayer=3, seed=5)
    check(ctx, raw, configs.make_spec(meta, levels=4, algorithm=algo), mode=mode)


def test_pipeline_strong_denoise_no_ltm(ctx, mode):
    raw, _, meta = synthetic.make_frame(256, 160, bayer=1, seed=6, gain=4.0, read_sigma=6.0)
    check(ctx, raw, configs.make_spec(meta, levels=5, ltm=False, denoise="strong"), mode=mode)


def test_pipeline_host_buffers_and_rgb(ctx):
    raw, _, meta = synthetic.make_frame(128, 96, bayer=2, seed=8)
    spec = configs.make_spec(meta, levels=4)
    conv = gls.RawConverter(ctx)
    out4 = np.zeros((96, 128, 4), np.uint8)
    out3 = np.zeros((96, 128, 3), np.uint8)
    conv.demosaicImageHost(raw, configs.to_gls_params(spec), out4)
    conv.demosaicImageHost(raw, configs.to_gls_params(spec), out3)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))["rgba8"]
    np.testing.assert_array_equal(out4, ref)
    np.testing.assert_array_equal(out3, ref[..., :3])


def test_pipeline_reused_converter_other_size(ctx):
    # the reference sizes its textures by the first frame only; this converter follows the frame
    import torch
    conv = gls.RawConverter(ctx)
    for (w, h, seed) in ((128, 96, 9), (96, 64, 10), (128, 96, 11)):
        raw, _, meta = synthetic.make_frame(w, h, bayer=2, seed=seed)
        spec = configs.make_spec(meta, levels=4)
        out = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
        conv.demosaicImage(torch.from_numpy(raw).cuda(), configs.to_gls_params(spec), out)
        ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))["rgba8"]
        np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_fast_demosaic(ctx):
    import torch
    raw, _, meta = synthetic.make_frame(160, 120, bayer=0, seed=12)
    spec = configs.make_spec(meta, levels=4)
    conv = gls.RawConverter(ctx)
    out = torch.empty((60, 80, 4), dtype=torch.uint8, device="cuda")
    conv.fastDemosaicImage(torch.from_numpy(raw).cuda(), configs.to_gls_params(spec), out)
    r8, _ = orc.fast_demosaic(raw, oracle_params(spec), orc.F32)
    np.testing.assert_array_equal(out.cpu().numpy(), r8)


def test_pipeline_rejects_bad_input(ctx):
    import torch
    conv = gls.RawConverter(ctx)
    raw, _, meta = synthetic.make_frame(64, 48, seed=13)
    spec = configs.make_spec(meta, levels=4)
    odd = torch.zeros((47, 64), dtype=torch.uint16, device="cuda")
    with pytest.raises(gls.GlsError):
        conv.demosaicImage(odd, configs.to_gls_params(spec), torch.empty((47, 64, 4), dtype=torch.uint8, device="cuda"))
    p = configs.to_gls_params(spec)
    p.pyramid_levels = 3
    with pytest.raises(gls.GlsError):
        conv.demosaicImage(torch.from_numpy(raw).cuda(), p, torch.empty((48, 64, 4), dtype=torch.uint8, device="cuda"))
    tiny = torch.zeros((4, 4), dtype=torch.uint16, device="cuda")
    with pytest.raises(gls.GlsError):
        conv.demosaicImage(tiny, configs.to_gls_params(spec), torch.empty((4, 4, 4), dtype=torch.uint8, device="cuda"))


@pytest.mark.parametrize("bayer,noise_level,gain", [(2, 0.2, 2.0), (1, 0.7, 16.0)], ids=["rggb", "gbrg_high_noise"])
def test_pipeline_rotate_180(ctx, bayer, noise_level, gain):
    """demosaicImage(..., rotate_180): interpolateRedBlue writes the frame turned by 180 degrees
    and every later stage reads the turned image (the converter runs its single-stage
    schedule for it); noise models, taps and output equal the oracle's, which the reference's
    own RawConverter equals on the CPU (test_clref_pipeline.py)."""
    raw, _, meta = synthetic.make_frame(200, 152, bayer=bayer, gain=gain, read_sigma=6.0, seed=140 + bayer)
    spec = configs.make_spec(meta, levels=5, noise_level=noise_level)
    spec["rotate_180"] = 1
    check(ctx, raw, spec)
    check(ctx, raw, spec, out_float=True)


def test_statistics_waits_run_out_and_report(ctx):
    """The statistics kernels' bounded waits (a TMA tile copy on its mbarrier, a coarser
    level's tile mark in the one-launch pyramid), made to run out on a mark that nothing sets
    and a barrier that nothing arrives at: the error word is set, status() raises
    GLS_ERR_TIMEOUT once, and the converter then converts frames as before."""
    import torch
    raw, _, meta = synthetic.make_frame(256, 192, bayer=2, seed=21)
    spec = configs.make_spec(meta, levels=5)
    conv = gls.RawConverter(ctx)
    p = configs.to_gls_params(spec)
    out = torch.empty((192, 256, 4), dtype=torch.uint8, device="cuda")
    conv.demosaicImage(torch.from_numpy(raw).cuda(), p, out)
    first = out.cpu().numpy()
    conv.status()
    conv.wait_probe(1 << 10)
    with pytest.raises(gls.GlsError) as err:
        conv.status()
    assert err.value.status == gls.GLS_ERR_TIMEOUT
    conv.status()  # reported once
    p = configs.to_gls_params(spec)
    conv.demosaicImage(torch.from_numpy(raw).cuda(), p, out)
    conv.status()
    np.testing.assert_array_equal(out.cpu().numpy(), first)
    with pytest.raises(gls.GlsError) as bad:
        conv.wait_probe(0)
    assert bad.value.status == gls.GLS_ERR_INVALID_ARGUMENT
    conv.close()
