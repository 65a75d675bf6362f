"""The header-only C++ layer (include/gls_cuda.hpp): a C++ program written against the
reference's API (gls::image, RawConverter::demosaicImage, convertToRGBImage,
autoWhiteBalance, colorCheckerRawStats) produces the oracle's results."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from climage_gb300 import build, configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import oracle_params

pytestmark = pytest.mark.gpu


def test_cpp_layer_raw_converter(cuda):
    exe = build.build_cpp_test()
    raw, _, meta = synthetic.make_frame(192, 128, bayer=2, seed=31)
    spec = configs.make_spec(meta, levels=4)
    with tempfile.TemporaryDirectory() as d:
        raw.tofile(os.path.join(d, "raw.u16"))
        vals = [192, 128, spec["bayer_pattern"], 4, spec["rgb"]["localToneMapping"], spec["black_level"],
                spec["white_level"], spec["exposure_multiplier"], spec["noise_level"]]
        vals += spec["scale_mul"] + spec["rgb_cam"] + spec["raw_nlf"]
        for row in spec["pyramid_nlf"]:
            vals += row
        for dp in spec["denoise"]:
            vals += [dp["luma"], dp["chroma"], dp["chromaBoost"], dp["gradientBoost"], dp["sharpening"]]
        r = spec["rgb"]
        vals += [r["contrast"], r["saturation"], r["toneCurveSlope"], r["exposureBias"], r["blacks"]]
        l = spec["ltm"]
        vals += [l["guidedFilterEps"], l["shadows"], l["highlights"], l["detail"]]
        with open(os.path.join(d, "params.txt"), "w") as f:
            f.write(" ".join(repr(float(v)) if isinstance(v, float) else str(v) for v in vals))
        res = subprocess.run([exe, d], capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stderr
        got = np.fromfile(os.path.join(d, "rgb.u8"), np.uint8).reshape(128, 192, 3)
        got_rot = np.fromfile(os.path.join(d, "rgb_rot.u8"), np.uint8).reshape(128, 192, 3)
        nlf = np.array(open(os.path.join(d, "nlf.txt")).read().split(), np.float32)
        awb = np.array(open(os.path.join(d, "awb.txt")).read().split(), np.float32)
        patches = np.fromfile(os.path.join(d, "patches.f32"), np.float32).reshape(24, 2, 4)
    ref = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))
    np.testing.assert_array_equal(got, ref["rgba8"][..., :3])
    np.testing.assert_allclose(nlf, ref["raw_nlf"], rtol=1e-6)
    # demosaicImage(..., rotate_180 = true), the second call on the same converter
    rspec = dict(spec, rotate_180=1)
    ref_rot = orc.demosaic(raw, oracle_params(rspec), orc.F32, want=("rgba8",))
    np.testing.assert_array_equal(got_rot, ref_rot["rgba8"][..., :3])
    # autoWhiteBalance: the gains and the highlight fraction (printed with 9 digits: exact floats)
    cy = gls.cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
    owb, ohl = orc.auto_white_balance(raw, cy, spec["scale_mul"], spec["white_level"], spec["black_level"],
                                      spec["bayer_pattern"])
    np.testing.assert_array_equal(awb[:3], owb)
    assert awb[3] == np.float32(ohl)
    # colorCheckerRawStats over the chart rectangle the program used
    om, ov = orc.color_checker_raw_stats(raw, spec["black_level"], spec["white_level"], spec["bayer_pattern"],
                                         (12, 10, 192 - 30, 128 - 24))
    np.testing.assert_array_equal(patches[:, 0], om)
    np.testing.assert_array_equal(patches[:, 1], ov)
