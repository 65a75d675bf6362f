"""The learned stage inside the pipeline (RawConverter with a Cnn, through the C ABI).

- an all-zero network (residual 0, noise-model multiplier exactly 1) reproduces the plain
  pipeline bit for bit, in every configuration: the plumbing adds nothing;
- the network's input equals the oracle's image after interpolateRedBlue, and its sigma
  channel is sqrt(A1 + B1 * G) of the oracle's fitted raw noise model;
- a non-zero network changes the output and keeps it finite;
- the trained parameters shipped with the package beat the plain pipeline on held-out
  scenes (PSNR and Delta E against the noise-free scene through the plain pipeline).
"""
import numpy as np
import pytest

from climage_gb300 import configs, gls, learned, synthetic
from oracle import oracle as orc
from tests.helpers import oracle_params

pytestmark = pytest.mark.gpu


def run(conv, raw, spec, float_out):
    import torch
    h, w = raw.shape
    out = torch.empty((h, w, 4), dtype=torch.float32 if float_out else torch.uint8, device="cuda")
    conv.demosaicImage(torch.from_numpy(raw).cuda(), configs.to_gls_params(spec), out, defer_noise_model=True)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("storage,noise_level,float_out", [
    (gls.STORAGE_F32, 0.2, False), (gls.STORAGE_F32, 0.2, True), (gls.STORAGE_F16, 0.45, False),
    (gls.STORAGE_F32, 0.7, True)], ids=["f32-rgba8", "f32-float", "f16-rgba8", "high-noise-float"])
def test_zero_network_reproduces_plain(ctx, storage, noise_level, float_out):
    raw, _, meta = synthetic.make_frame(200, 152, bayer=1, gain=4.0 if noise_level < 0.6 else 16.0,
                                        read_sigma=6.0 if noise_level < 0.6 else 12.0, seed=21)
    spec = configs.make_spec(meta, levels=5, storage=storage, noise_level=noise_level)
    cnn = gls.Cnn(ctx)
    cnn.set_params(np.zeros(cnn.nparam, np.float32))
    plain, lrn = gls.RawConverter(ctx), gls.RawConverter(ctx)
    lrn.setCnn(cnn)
    a, b = run(plain, raw, spec, float_out), run(lrn, raw, spec, float_out)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    for c in (plain, lrn, cnn):
        c.close()


@pytest.mark.parametrize("bayer", [0, 2])
def test_network_input_matches_oracle(ctx, bayer):
    import torch
    raw, _, meta = synthetic.make_frame(136, 104, bayer=bayer, gain=4.0, read_sigma=6.0, seed=5 + bayer)
    spec = configs.make_spec(meta, levels=4)
    conv = gls.RawConverter(ctx)
    buf = torch.empty((104, 136, 4), dtype=torch.float32, device="cuda")
    conv.cnnInput(torch.from_numpy(raw).cuda(), configs.to_gls_params(spec), buf)
    torch.cuda.synchronize()
    got = buf.cpu().numpy()
    taps = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",), taps=("scaled_raw", "linear_rgb"))
    assert np.array_equal(got[..., :3], taps["linear_rgb"][..., :3])
    nlf = orc.compute_raw_nlf(taps["scaled_raw"], bayer)
    sig = np.sqrt(np.maximum(np.float32(nlf[1]) + np.float32(nlf[5]) * got[..., 1], np.float32(1e-8)))
    assert np.array_equal(got[..., 3], sig.astype(np.float32))
    conv.close()


def test_nonzero_network_changes_the_output(ctx):
    raw, _, meta = synthetic.make_frame(128, 96, bayer=2, gain=4.0, read_sigma=6.0, seed=8)
    spec = configs.make_spec(meta, levels=4)
    cnn = gls.Cnn(ctx)
    cnn.set_params(gls.cnn_init(2, head_std=0.05))
    plain, lrn = gls.RawConverter(ctx), gls.RawConverter(ctx)
    lrn.setCnn(cnn)
    a, b = run(plain, raw, spec, True), run(lrn, raw, spec, True)
    assert np.all(np.isfinite(b[..., :3]))
    assert not np.array_equal(a, b)
    lrn.setCnn(None)  # back to plain
    assert np.array_equal(run(lrn, raw, spec, True).view(np.uint8), a.view(np.uint8))
    for c in (plain, lrn, cnn):
        c.close()


def test_trained_network_beats_plain(ctx):
    params = learned.load_params()
    if params is None:
        pytest.skip("no trained parameters shipped")
    cnn = gls.Cnn(ctx)
    cnn.set_params(params)
    verdict = learned.judge(ctx, cnn, range(10**6 + 100, 10**6 + 103), width=512, height=384)
    cnn.close()
    assert verdict["learned"]["psnr_db"] > verdict["plain"]["psnr_db"], verdict
    assert verdict["learned"]["delta_e"] < verdict["plain"]["delta_e"], verdict
