"""Writes the golden fixtures of tests/golden from the reference's own host code.

The reference's colour math (cam_xyz_coeff, cam_ycbcr, gls::inverse, matrix products from
CLImage/app/src/main/cpp/demosaic_utils.cpp and src/gls_linalg.hpp) and its packed-raw
unpack routines (src/gls_image_tiff.cpp:53-87) and autoWhiteBalance (demosaic_utils.cpp:
976-1026), estimateRawParameters (686-785) and the lossless-JPEG codec (src/gls_dng_lossless_jpeg.cpp) are compiled from the
reference sources into oracle/_ref/libref_host.so (make -C oracle ref); this script runs them
on fixed inputs and stores the results bit-exactly.  It also records hashes of the oracle's own
pipeline outputs on small seeded frames, which pin the oracle across machines.

    make -C oracle ref && python tests/golden/make_golden.py
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from climage_gb300 import configs, synthetic  # noqa: E402
from oracle import oracle as orc  # noqa: E402

# camera matrices: the Adobe-style matrix of raw_pipeline.cpp:77, the IMX571 and Sony a6400
# colour matrices used by the calibration drivers, and two synthetic well-conditioned ones
MATRICES = {
    "adobe_transcode": configs.CAM_XYZ,
    "imx571": [1.2594, -0.5333, -0.1138, -0.1404, 0.9717, 0.1688, 0.0342, 0.0969, 0.4330],
    "synthetic_a": [1.0, -0.2, -0.1, -0.15, 1.1, 0.05, 0.02, -0.12, 0.9],
    "synthetic_b": [0.8, -0.3, 0.05, -0.2, 1.2, 0.1, 0.05, 0.15, 0.7],
}


def bits(a):
    return [int(v) for v in np.asarray(a, np.float32).ravel().view(np.uint32)]


def colour_fixture(ref):
    f = ctypes.c_float
    out = {}
    for name, m in MATRICES.items():
        cx = (f * 9)(*m)
        pre, rgb_cam = (f * 3)(), (f * 9)()
        ref.ref_cam_xyz_coeff(cx, pre, rgb_cam)
        cy = (f * 9)()
        ref.ref_cam_ycbcr(rgb_cam, cy)
        inv = (f * 9)()
        ref.ref_inverse3x3(cy, inv)
        scaled = (f * 9)()
        ref.ref_matscale3x3(inv, f(0.8), scaled)
        prod = (f * 9)()
        ref.ref_matmul3x3(cy, inv, prod)
        out[name] = {"cam_xyz": bits(m), "pre_mul": bits(pre[:]), "rgb_cam": bits(rgb_cam[:]),
                     "cam_ycbcr": bits(cy[:]), "inverse_cam_ycbcr": bits(inv[:]),
                     "inverse_times_0.8": bits(scaled[:]), "cam_ycbcr_times_inverse": bits(prod[:])}
    return out


def unpack_fixture(ref):
    rng = np.random.default_rng(2024)
    res = {}
    for nbits, fn, group in ((12, ref.ref_unpack12, 3), (14, ref.ref_unpack14, 7)):
        n_words = group * 301
        raw_bytes = rng.integers(0, 256, 2 * n_words, dtype=np.uint8)
        words = raw_bytes.view(np.uint16).copy()  # file order: big-endian words, as read from disk
        out = np.zeros(n_words * 16 // nbits, np.uint16)
        fn(words.ctypes.data_as(ctypes.c_void_p), ctypes.c_long(n_words), out.ctypes.data_as(ctypes.c_void_p))
        res["packed%d" % nbits] = raw_bytes
        res["unpacked%d" % nbits] = out
    return res


def awb_fixture():
    """autoWhiteBalance of the reference (demosaic_utils.cpp:976-1026) on the seeded frames
    of tests/awb_frames.py.  The reference keeps its luma-bin sums in gls::Vector<3>, whose
    default constructor leaves the elements unset, so its histogram starts from whatever
    the stack held; oracle/Makefile builds it with -ftrivial-auto-var-init=zero, which gives
    the zeroed bins the code means."""
    from tests import awb_frames
    out = {}
    for case in awb_frames.CASES:
        raw, m, sm, white, black, bayer = awb_frames.make(case, orc.cam_ycbcr)
        wb, hl = orc.auto_white_balance(raw, m, sm, white, black, bayer, reference=True)
        out[case[0]] = {"raw_sha256": hashlib.sha256(raw.tobytes()).hexdigest(), "rgb_ycbcr": bits(m),
                        "scale_mul": bits(sm), "white": bits([white])[0], "black": bits([black])[0],
                        "bayer": bayer, "wb": bits(wb), "highlights": bits([hl])[0]}
    return out


def lj92_fixture():
    """Lossless-JPEG streams and the reference decoder's output (DecodeLosslessJPEG,
    gls_dng_lossless_jpeg.cpp:3253-3275): the "ref_" cases are written by the reference's
    EncodeLosslessJPEG, the "own_" cases (predictors 2-7, restart intervals, which that
    encoder never writes) by the oracle's test encoder."""
    from tests import lj92_cases
    streams, meta = {}, {}
    for name, rows, cols, comps, prec, pred, rst, kind, seed in lj92_cases.CASES:
        x = lj92_cases.samples(rows, cols, comps, prec, kind, seed)
        st = orc.lj92_encode(x, comps, prec, pred, rst, reference=name.startswith("ref_"))
        dec, info = orc.lj92_decode(st, reference=True)
        assert np.array_equal(dec, x), name
        streams[name] = np.frombuffer(st, np.uint8)
        meta[name] = {"rows": rows, "cols": cols, "components": comps, "precision": prec, "predictor": pred,
                      "restart_rows": rst, "samples_sha256": hashlib.sha256(dec.tobytes()).hexdigest()}
    return streams, meta


def calib_fixture():
    """estimateRawParameters of the reference (demosaic_utils.cpp:686-785) on the seeded chart
    frames of tests/calib_frames.py; its colorCheckerRawStats writes debug PNGs through a
    writer the shim leaves empty."""
    from tests import calib_frames
    out = {}
    for case in calib_frames.CASES:
        raw, black, white, bayer, gmb, rot = calib_frames.make(case)
        cx, pm, nlf = orc.estimate_raw_parameters(raw, black, white, bayer, gmb, rot, reference=True)
        out[case[0]] = {"raw_sha256": hashlib.sha256(raw.tobytes()).hexdigest(), "cam_xyz": bits(cx),
                        "pre_mul": bits(pm), "raw_nlf": bits(nlf)}
    return out


def oracle_pins():
    pins = {}
    for name, (w, h, bayer, prec, levels) in {
        "rggb_f32_4lvl": (256, 192, 2, orc.F32, 4),
        "grbg_f16_5lvl": (256, 192, 0, orc.F16, 5),
        "bggr_f32_highnoise": (192, 128, 3, orc.F32, 4),
    }.items():
        gain, sigma, nl = (16.0, 12.0, 0.7) if "highnoise" in name else (2.0, 3.0, 0.2)
        raw, _, meta = synthetic.make_frame(w, h, bayer=bayer, gain=gain, read_sigma=sigma, seed=77)
        spec = configs.make_spec(meta, levels=levels, noise_level=nl, storage=1 if prec == orc.F16 else 0)
        from tests.helpers import oracle_params
        r = orc.demosaic(raw, oracle_params(spec), prec, want=("rgba8", "rgbaf"))
        pins[name] = {"raw_sha256": hashlib.sha256(raw.tobytes()).hexdigest(),
                      "rgba8_sha256": hashlib.sha256(r["rgba8"].tobytes()).hexdigest(),
                      "rgbaf_sha256": hashlib.sha256(r["rgbaf"].tobytes()).hexdigest(),
                      "raw_nlf": bits(r["raw_nlf"]), "pyramid_nlf": bits(r["pyramid_nlf"])}
    return pins


def main():
    ref = orc.ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_host.so is missing: run make -C oracle ref on a machine with the reference")
    with open(os.path.join(HERE, "ref_colour.json"), "w") as f:
        json.dump(colour_fixture(ref), f, indent=1)
    np.savez_compressed(os.path.join(HERE, "ref_unpack.npz"), **unpack_fixture(ref))
    with open(os.path.join(HERE, "ref_awb.json"), "w") as f:
        json.dump(awb_fixture(), f, indent=1)
    streams, meta = lj92_fixture()
    np.savez_compressed(os.path.join(HERE, "ref_lj92.npz"), **streams)
    with open(os.path.join(HERE, "ref_lj92.json"), "w") as f:
        json.dump(meta, f, indent=1)
    with open(os.path.join(HERE, "ref_calib.json"), "w") as f:
        json.dump(calib_fixture(), f, indent=1)
    with open(os.path.join(HERE, "oracle_pins.json"), "w") as f:
        json.dump(oracle_pins(), f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
