"""The oracle pinned against the reference: colour math and packed-raw unpack equal the
reference's own compiled code (tests/golden, written by make_golden.py from
oracle/_ref), the noise-model regression meets known answers, and the stencils satisfy
the properties the reference's algorithms imply (constant images, CFA phase shifts).
autoWhiteBalance equals the reference's compiled code on seeded frames.  The reference has
no tests or golden vectors of its own for this path."""
import hashlib
import json
import os

import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from oracle import oracle as orc
from tests.helpers import oracle_params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def f32(bits):
    return np.array(bits, np.uint32).view(np.float32)


@pytest.fixture(scope="module")
def colour():
    with open(os.path.join(GOLDEN, "ref_colour.json")) as f:
        return json.load(f)


def test_colour_math_equals_reference(colour):
    for name, fx in colour.items():
        cam_xyz = f32(fx["cam_xyz"])
        for impl in (orc, gls):  # the oracle's and the product's restatements
            pre, rgb_cam = impl.cam_xyz_coeff(cam_xyz)
            np.testing.assert_array_equal(pre, f32(fx["pre_mul"]), err_msg=name)
            np.testing.assert_array_equal(rgb_cam.ravel(), f32(fx["rgb_cam"]), err_msg=name)
            cy = impl.cam_ycbcr(rgb_cam)
            np.testing.assert_array_equal(cy.ravel(), f32(fx["cam_ycbcr"]), err_msg=name)
            inv = impl.inverse3x3(cy)
            np.testing.assert_array_equal(inv.ravel(), f32(fx["inverse_cam_ycbcr"]), err_msg=name)
        np.testing.assert_array_equal(orc.matmul3x3(cy, inv).ravel(), f32(fx["cam_ycbcr_times_inverse"]))
        np.testing.assert_array_equal((inv * np.float32(0.8)).ravel(), f32(fx["inverse_times_0.8"]))


def test_unpack_equals_reference():
    fx = np.load(os.path.join(GOLDEN, "ref_unpack.npz"))
    for nbits in (12, 14):
        packed = fx["packed%d" % nbits].tobytes()
        np.testing.assert_array_equal(orc.unpack_bits(packed, nbits), fx["unpacked%d" % nbits])


@pytest.fixture(scope="module")
def awb_golden():
    with open(os.path.join(GOLDEN, "ref_awb.json")) as f:
        return json.load(f)


def awb_inputs(case, fx):
    """The case's frame (regenerated from its seed and checked against the fixture's hash)
    and the fixture's stored parameters."""
    from tests import awb_frames
    raw = awb_frames.make(case, orc.cam_ycbcr)[0]
    assert hashlib.sha256(raw.tobytes()).hexdigest() == fx["raw_sha256"], case[0]
    return raw, f32(fx["rgb_ycbcr"]), f32(fx["scale_mul"]), f32([fx["white"]])[0], f32([fx["black"]])[0], fx["bayer"]


def test_auto_white_balance_equals_reference(awb_golden):
    """Bit for bit, including crafted frames with clipped highlights and with dark quads
    whose negative luma bin the reference maps to the top bin (crafted_dark, crafted_mixed)."""
    from tests import awb_frames
    assert set(awb_golden) == {c[0] for c in awb_frames.CASES}
    for case in awb_frames.CASES:
        fx = awb_golden[case[0]]
        raw, m, sm, white, black, bayer = awb_inputs(case, fx)
        wb, hl = orc.auto_white_balance(raw, m, sm, white, black, bayer)
        np.testing.assert_array_equal(wb.view(np.uint32), np.array(fx["wb"], np.uint32), err_msg=case[0])
        assert int(np.float32(hl).view(np.uint32)) == fx["highlights"], case[0]


def lj92_fixture():
    with open(os.path.join(GOLDEN, "ref_lj92.json")) as f:
        meta = json.load(f)
    return np.load(os.path.join(GOLDEN, "ref_lj92.npz")), meta


def test_lj92_decode_equals_reference():
    """The oracle's lossless-JPEG decoder gives the reference decoder's samples on streams
    written by the reference's encoder and by the oracle's (predictors 2-7, restarts)."""
    streams, meta = lj92_fixture()
    for name, m in meta.items():
        dec, info = orc.lj92_decode(streams[name].tobytes())
        assert hashlib.sha256(dec.tobytes()).hexdigest() == m["samples_sha256"], name
        assert (info["height"], info["width"], info["components"]) == (m["rows"], m["cols"], m["components"])
        assert info["predictor"] == m["predictor"], name


def test_lj92_round_trip():
    from tests import lj92_cases
    for name, rows, cols, comps, prec, pred, rst, kind, seed in lj92_cases.CASES:
        x = lj92_cases.samples(rows, cols, comps, prec, kind, seed + 100)
        dec, _ = orc.lj92_decode(orc.lj92_encode(x, comps, prec, pred, rst))
        np.testing.assert_array_equal(dec, x, err_msg=name)


def test_estimate_raw_parameters_equals_reference():
    """The oracle's colour-checker calibration gives the reference's matrix, white point and
    noise slopes bit for bit (one chart rotated by 180 degrees, one at odd coordinates)."""
    from tests import calib_frames
    with open(os.path.join(GOLDEN, "ref_calib.json")) as f:
        golden = json.load(f)
    assert set(golden) == {c[0] for c in calib_frames.CASES}
    for case in calib_frames.CASES:
        fx = golden[case[0]]
        raw, black, white, bayer, gmb, rot = calib_frames.make(case)
        assert hashlib.sha256(raw.tobytes()).hexdigest() == fx["raw_sha256"], case[0]
        cx, pm, nlf = orc.estimate_raw_parameters(raw, black, white, bayer, gmb, rot)
        for got, key in ((cx, "cam_xyz"), (pm, "pre_mul"), (nlf, "raw_nlf")):
            np.testing.assert_array_equal(np.ravel(got).view(np.uint32), np.array(fx[key], np.uint32),
                                          err_msg=case[0] + " " + key)


def test_unpack_round_trip_all_depths():
    rng = np.random.default_rng(9)
    for nbits in (10, 12, 14, 16):
        s = rng.integers(0, 1 << nbits, 1001).astype(np.uint16)
        np.testing.assert_array_equal(orc.unpack_bits(synthetic.pack_bits(s, nbits), nbits), s)


def test_oracle_self_pins():
    """The oracle gives the same bits on every machine (x86-64 and aarch64)."""
    with open(os.path.join(GOLDEN, "oracle_pins.json")) as f:
        pins = json.load(f)
    for name, (w, h, bayer, prec, levels) in {
        "rggb_f32_4lvl": (256, 192, 2, orc.F32, 4),
        "grbg_f16_5lvl": (256, 192, 0, orc.F16, 5),
        "bggr_f32_highnoise": (192, 128, 3, orc.F32, 4),
    }.items():
        gain, sigma, nl = (16.0, 12.0, 0.7) if "highnoise" in name else (2.0, 3.0, 0.2)
        raw, _, meta = synthetic.make_frame(w, h, bayer=bayer, gain=gain, read_sigma=sigma, seed=77)
        assert hashlib.sha256(raw.tobytes()).hexdigest() == pins[name]["raw_sha256"], name
        spec = configs.make_spec(meta, levels=levels, noise_level=nl, storage=1 if prec == orc.F16 else 0)
        r = orc.demosaic(raw, oracle_params(spec), prec, want=("rgba8", "rgbaf"))
        np.testing.assert_array_equal(r["raw_nlf"], f32(pins[name]["raw_nlf"]))
        np.testing.assert_array_equal(r["pyramid_nlf"].ravel(), f32(pins[name]["pyramid_nlf"]))
        assert hashlib.sha256(r["rgba8"].tobytes()).hexdigest() == pins[name]["rgba8_sha256"], name
        assert hashlib.sha256(r["rgbaf"].tobytes()).hexdigest() == pins[name]["rgbaf_sha256"], name


def test_regression_known_answer():
    rng = np.random.default_rng(11)
    n = 20000
    A, B = np.array([1e-5, 2e-5, 3e-6]), np.array([4e-4, 1e-4, 2e-4])
    m = rng.uniform(0.002, 0.45, n)
    v = A[None] + B[None] * m[:, None] + rng.normal(0, 2e-6, (n, 3))
    ab = orc.regress(m, v)
    np.testing.assert_allclose(ab[:3], A, rtol=0.05, atol=2e-7)
    np.testing.assert_allclose(ab[3:], B, rtol=0.01)
    # statistics outside [0.001, 0.5] x [0, 0.001] are ignored
    m2 = np.concatenate([m, rng.uniform(0.6, 0.9, 500)])
    v2 = np.concatenate([v, np.full((500, 3), 5e-4)])
    np.testing.assert_array_equal(orc.regress(m2, v2), ab)
    # the refit keeps samples whose squared residual is <= the RMS residual (the reference
    # compares the squared residual with the un-squared RMS, pyramidal_denoise.cpp:225-230)
    m3 = np.array([0.1, 0.2, 0.3, 0.4], np.float32)
    v3 = np.stack([1e-5 + 2e-4 * m3] * 3, 1).astype(np.float32)
    ab3 = orc.regress(m3, v3)
    np.testing.assert_allclose(ab3[3:], 2e-4, rtol=1e-5)


def test_regression_degenerate_inputs_give_nan():
    # no sample in range: N = 0, the fit divides 0 by 0 as the reference does
    ab = orc.regress(np.full(10, 0.9, np.float32), np.zeros((10, 3), np.float32))
    assert np.isnan(ab).all()


def test_constant_frame_demosaics_to_constant():
    w, h = 64, 48
    for bayer in range(4):
        scaled = np.full((h, w), 0.3, np.float32)
        g = orc.interpolate_green(scaled, bayer, 3e-4)
        np.testing.assert_array_equal(g, scaled)
        rgb = orc.interpolate_red_blue(scaled, g, bayer, 3e-4)
        np.testing.assert_array_equal(rgb[..., :3], np.float32(0.3))


def test_cfa_phase_shift_equivariance():
    """Shifting a mosaic by one column turns RGGB into GRBG (and GBRG into BGGR); the
    interpolated planes shift with it away from the border."""
    rng = np.random.default_rng(12)
    scaled = rng.uniform(0.05, 0.6, (40, 66)).astype(np.float32)
    for p, q in ((2, 0), (1, 3)):
        g_p = orc.interpolate_green(scaled, p, 3e-4)
        g_q = orc.interpolate_green(scaled[:, 1:-1], q, 3e-4)
        np.testing.assert_array_equal(g_p[6:-6, 7:-7], g_q[6:-6, 6:-6])
        rb_p = orc.interpolate_red_blue(scaled, g_p, p, 3e-4)
        rb_q = orc.interpolate_red_blue(scaled[:, 1:-1], g_p[:, 1:-1], q, 3e-4)
        np.testing.assert_array_equal(rb_p[6:-6, 7:-7], rb_q[6:-6, 6:-6])


def test_fp64_error_oracle_close_to_fp32():
    raw, _, meta = synthetic.make_frame(192, 128, bayer=2, seed=21)
    spec = configs.make_spec(meta, levels=4)
    a = orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgbaf",))
    b = orc.demosaic(raw, oracle_params(spec), orc.F64, want=("rgbaf",))
    d = np.abs(a["rgbaf"].astype(np.float64) - b["rgbaf"])
    assert np.percentile(d, 99) < 5e-3
    mse = np.mean(np.clip(d, 0, 1) ** 2)
    assert 10 * np.log10(1.0 / max(mse, 1e-20)) > 50.0


def test_product_chart_fit_equals_reference():
    """The product's host-side fit (gls_fit_color_checker, no GPU needed), fed the oracle's
    patch statistics, gives the reference's matrix, white point and noise slopes bit for bit."""
    from tests import calib_frames
    with open(os.path.join(GOLDEN, "ref_calib.json")) as f:
        golden = json.load(f)
    for case in calib_frames.CASES:
        fx = golden[case[0]]
        raw, black, white, bayer, gmb, rot = calib_frames.make(case)
        mean, var = orc.color_checker_raw_stats(raw, black, white, bayer, gmb, rot)
        cx, pm, nlf = gls.fit_color_checker(mean, var)
        for got, key in ((cx, "cam_xyz"), (pm, "pre_mul"), (nlf, "raw_nlf")):
            np.testing.assert_array_equal(np.ravel(got).view(np.uint32), np.array(fx[key], np.uint32),
                                          err_msg=case[0] + " " + key)
    with pytest.raises(gls.GlsError):  # a chart with no signal has no white point
        gls.fit_color_checker(np.zeros((24, 4), np.float32), np.zeros((24, 4), np.float32))
