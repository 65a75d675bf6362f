"""autoWhiteBalance on the GPU (gls_auto_white_balance, through the C ABI) against the
reference's own outputs (tests/golden/ref_awb.json) and the oracle: bit for bit on the
gains and the highlight fraction, at fixture sizes, at 4032x3024, on strided input and on
degenerate frames."""
import json
import os

import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests import awb_frames

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def f32(bits):
    return np.array(bits, np.uint32).view(np.float32)


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def gpu_awb(ctx, raw, m, sm, white, black, bayer):
    import torch
    t = raw if isinstance(raw, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(raw)).cuda()
    return ctx.autoWhiteBalance(t, m, sm, white, black, bayer)


def test_golden_cases(ctx):
    with open(os.path.join(GOLDEN, "ref_awb.json")) as f:
        golden = json.load(f)
    for case in awb_frames.CASES:
        fx = golden[case[0]]
        raw = awb_frames.make(case, orc.cam_ycbcr)[0]
        wb, hl = gpu_awb(ctx, raw, f32(fx["rgb_ycbcr"]), f32(fx["scale_mul"]), f32([fx["white"]])[0],
                         f32([fx["black"]])[0], fx["bayer"])
        assert bits_equal(wb, f32(fx["wb"])), (case[0], wb, f32(fx["wb"]))
        assert bits_equal(hl, f32([fx["highlights"]])[0]), (case[0], hl)


@pytest.mark.parametrize("bayer", [0, 1, 2, 3])
def test_full_size_frame(ctx, bayer):
    raw, _, meta = synthetic.make_frame(4032, 3024, bayer=bayer, gain=4.0, seed=40 + bayer)
    spec = configs.make_spec(meta, levels=5)
    m = gls.cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
    args = (m, spec["scale_mul"], float(meta["white"]), float(meta["black"]), bayer)
    wb, hl = gpu_awb(ctx, raw, *args)
    ref_wb, ref_hl = orc.auto_white_balance(raw, *args)
    assert bits_equal(wb, ref_wb) and bits_equal(hl, ref_hl), (wb, ref_wb, hl, ref_hl)


def test_strided_input(ctx):
    import torch
    full = awb_frames.crafted(700, 520, 8, sat=0.1, dark=0.2)
    view = torch.from_numpy(full).cuda()[:, 37:37 + 611]  # rows keep the 700-pixel pitch
    crop = np.ascontiguousarray(full[:, 37:37 + 611])
    m = orc.cam_ycbcr(np.eye(3, dtype=np.float32))
    args = (m, awb_frames.CRAFTED_SCALE_MUL, 65535.0, awb_frames.CRAFTED_BLACK, 1)
    wb, hl = gpu_awb(ctx, view, *args)
    ref_wb, ref_hl = orc.auto_white_balance(crop, *args)
    assert bits_equal(wb, ref_wb) and bits_equal(hl, ref_hl)


@pytest.mark.parametrize("shape,value", [((4, 4), 0), ((6, 10), 500), ((64, 48), 0), ((64, 48), 65535),
                                         ((3000, 8), 1000)])
def test_degenerate_frames(ctx, shape, value):
    """Tiles of zero quads (NaN means), black frames, saturated frames, one-quad-wide tiles."""
    raw = np.full(shape, value, np.uint16)
    m = orc.cam_ycbcr(np.eye(3, dtype=np.float32))
    args = (m, [1.5, 1.0, 1.2, 1.0], 65535.0, 256.0, 2)
    wb, hl = gpu_awb(ctx, raw, *args)
    ref_wb, ref_hl = orc.auto_white_balance(raw, *args)
    assert bits_equal(wb, ref_wb) and bits_equal(hl, ref_hl), (wb, ref_wb, hl, ref_hl)


def test_invalid_arguments(ctx):
    import torch
    raw = torch.from_numpy(np.zeros((64, 64), np.uint16)).cuda()
    m = np.eye(3, dtype=np.float32)
    with pytest.raises(gls.GlsError):
        ctx.autoWhiteBalance(raw, m, [1, 1, 1, 1], 65535.0, 0.0, 4)
    with pytest.raises(gls.GlsError):
        ctx.autoWhiteBalance(torch.zeros((64, 64), dtype=torch.float32, device="cuda"), m, [1, 1, 1, 1], 65535.0,
                             0.0, 2)
