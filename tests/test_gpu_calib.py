"""Colour-checker calibration on the GPU (gls_estimate_raw_parameters and
gls_color_checker_raw_stats, through the C ABI) against the reference's outputs
(tests/golden/ref_calib.json) and the oracle, bit for bit."""
import json
import os

import numpy as np
import pytest

from climage_gb300 import gls
from oracle import oracle as orc
from tests import calib_frames

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(a):
    return np.ravel(np.asarray(a, np.float32)).view(np.uint32)


@pytest.mark.parametrize("case", calib_frames.CASES, ids=[c[0] for c in calib_frames.CASES])
def test_matches_reference(ctx, case):
    import torch
    with open(os.path.join(GOLDEN, "ref_calib.json")) as f:
        fx = json.load(f)[case[0]]
    raw, black, white, bayer, gmb, rot = calib_frames.make(case)
    t = torch.from_numpy(raw).cuda()
    cx, pm, nlf = ctx.estimateRawParameters(t, black, white, bayer, gmb, rot)
    assert np.array_equal(bits(cx), np.array(fx["cam_xyz"], np.uint32))
    assert np.array_equal(bits(pm), np.array(fx["pre_mul"], np.uint32))
    assert np.array_equal(bits(nlf), np.array(fx["raw_nlf"], np.uint32))
    mean, var = ctx.colorCheckerRawStats(t, black, white, bayer, gmb, rot)
    om, ov = orc.color_checker_raw_stats(raw, black, white, bayer, gmb, rot)
    assert np.array_equal(bits(mean), bits(om)) and np.array_equal(bits(var), bits(ov))


def test_large_chart_and_strided_frame(ctx):
    """A chart filling most of a 4032x3024 frame (patches of ~80k quads), read through a
    strided view."""
    import torch
    case = ("big", 2016, 1512, 100, 80, 1800, 1300, 2, 12, 2.0, 3.0, 0, 9)
    raw, black, white, bayer, gmb, rot = calib_frames.make(case)
    full = np.zeros((1512, 2016 + 64), np.uint16)
    full[:, :2016] = raw
    view = torch.from_numpy(full).cuda()[:, :2016]
    cx, pm, nlf = ctx.estimateRawParameters(view, black, white, bayer, gmb, rot)
    ocx, opm, onlf = orc.estimate_raw_parameters(raw, black, white, bayer, gmb, rot)
    assert np.array_equal(bits(cx), bits(ocx)) and np.array_equal(bits(pm), bits(opm))
    assert np.array_equal(bits(nlf), bits(onlf))


def test_rejects_chart_outside_the_frame(ctx):
    import torch
    t = torch.from_numpy(np.zeros((64, 64), np.uint16)).cuda()
    with pytest.raises(gls.GlsError):
        ctx.estimateRawParameters(t, 0.0, 4095.0, 2, (40, 0, 48, 32))
