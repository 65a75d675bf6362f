"""Whole-pipeline parity at the benchmark's own sizes, on the benchmark's seeded frames:
- the 4032x3024 RGGB 12-bit frames of the plain workload, fp32 storage, five levels, LTM
  on, RGBA8 out: the low-noise frame, and the high-gain frame that takes the raw-denoise
  branch;
- the 8064x6048 GRBG 14-bit frame of the precision form, fp16 storage, six levels.

Each goes through RawConverter::demosaicImage on the GPU and through the oracle on the
same frame.  Bar: the fitted noise models (raw and per level) are equal, and every RGBA8
code differs by at most 1 (0.5 LSB of the float result).  The count of differing codes is
reported; it has been zero."""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import U8_MAX_LSB, oracle_params

pytestmark = pytest.mark.gpu


def bench_frame(cfg, i):
    """Frame i of a workload, rendered as bench.py renders rank 0's frames."""
    sigma, gain, nl = cfg["noise"][i]
    raw, _, meta = synthetic.make_frame(cfg["width"], cfg["height"], bayer=cfg["bayer"], bits=cfg["bits"],
                                        black=cfg["black"], white=cfg["white"], wb=cfg["wb"], gain=gain,
                                        read_sigma=sigma, seed=i)
    return raw, configs.make_spec(meta, levels=cfg["levels"], storage=cfg["storage"], noise_level=nl)


def gpu_run(ctx, raw, spec):
    import torch
    h, w = raw.shape
    conv = gls.RawConverter(ctx)
    p = configs.to_gls_params(spec)
    out = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    conv.demosaicImage(torch.from_numpy(raw).cuda(), p, out)
    torch.cuda.synchronize()
    rgba8 = out.cpu().numpy()
    raw_nlf = np.array(p.raw_nlf[:], np.float32)
    pyr = np.array([p.pyramid_nlf[i][:] for i in range(spec["pyramid_levels"])], np.float32)
    conv.close()
    return rgba8, raw_nlf, pyr


def check(ctx, cfg, i, prec):
    raw, spec = bench_frame(cfg, i)
    got, raw_nlf, pyr = gpu_run(ctx, raw, spec)
    ref = orc.demosaic(raw, oracle_params(spec), prec, want=("rgba8",))
    np.testing.assert_array_equal(raw_nlf, ref["raw_nlf"])
    np.testing.assert_array_equal(pyr, ref["pyramid_nlf"])
    d = np.abs(got.astype(np.int16) - ref["rgba8"].astype(np.int16))
    assert int(d.max()) <= U8_MAX_LSB
    return int((d > 0).sum())


@pytest.mark.parametrize("i", [0, 2], ids=["read2_gain1", "read12_gain16_raw_denoise"])
def test_plain_workload_frame(ctx, i):
    assert configs.CONFIG2["storage"] == gls.STORAGE_F32
    differing = check(ctx, configs.CONFIG2, i, orc.F32)
    print("4032x3024 frame %d: %d RGBA8 codes differ by 1" % (i, differing))


def test_precision_form_frame(ctx):
    assert configs.CONFIG3["storage"] == gls.STORAGE_F16
    differing = check(ctx, configs.CONFIG3, 0, orc.F16)
    print("8064x6048 fp16 frame: %d RGBA8 codes differ by 1" % differing)
