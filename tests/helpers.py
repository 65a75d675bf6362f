"""Shared test helpers: spec -> oracle parameter block, tolerances."""
import numpy as np

from oracle import oracle as orc


def oracle_params(spec):
    p = orc.Params()
    p.bayer_pattern = spec["bayer_pattern"]
    p.black_level = spec["black_level"]
    p.white_level = spec["white_level"]
    p.exposure_multiplier = spec["exposure_multiplier"]
    for i in range(4):
        p.scale_mul[i] = spec["scale_mul"][i]
        p.raw_nlf[i] = spec["raw_nlf"][i]
    for i in range(9):
        p.rgb_cam[i] = spec["rgb_cam"][i]
    for i, row in enumerate(spec["pyramid_nlf"]):
        for k in range(6):
            p.pyramid_nlf[i][k] = row[k]
    for i, d in enumerate(spec["denoise"]):
        for k, v in d.items():
            setattr(p.denoise[i], k, v)
    p.noise_level = spec["noise_level"]
    for k, v in spec["rgb"].items():
        setattr(p.rgb, k, v)
    for k, v in spec["ltm"].items():
        setattr(p.ltm, k, v)
    p.pyramid_levels = spec["pyramid_levels"]
    p.denoise_algorithm = spec["denoise_algorithm"]
    p.rotate_180 = int(spec.get("rotate_180", 0))
    return p


# Tolerances of the parity tests (float outputs: max-abs 1e-3 on linear data; 8-bit
# outputs: within 0.5 LSB of the float result, i.e. codes differ by at most 1).
LINEAR_MAX_ABS = 1e-3
U8_MAX_LSB = 1


def max_abs(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b)
    d[both_nan] = 0
    return float(np.nanmax(d)) if d.size else 0.0


def mismatch(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        same = (a == b) | (np.isnan(a) & np.isnan(b))
    else:
        same = a == b
    return int((~same).sum())
