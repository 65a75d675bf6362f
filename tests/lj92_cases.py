"""Seeded sample arrays and stream parameters for the lossless-JPEG tests and fixtures."""
import numpy as np

# (name, rows, cols, components, precision, predictor, restart_rows, kind, seed); predictor 1
# without restarts is what the reference's encoder writes (those cases are encoded by it)
CASES = [
    ("ref_c1_12bit", 48, 64, 1, 12, 1, 0, "raw", 1),
    ("ref_c2_14bit", 33, 20, 2, 14, 1, 0, "raw", 2),
    ("ref_c4_16bit_random", 16, 24, 4, 16, 1, 0, "random", 3),
    ("ref_c1_16bit_halfscale", 9, 31, 1, 16, 1, 0, "halfscale", 4),
    ("ref_c3_8bit_flat", 7, 5, 3, 8, 1, 0, "flat", 5),
    ("ref_c1_1x1", 1, 1, 1, 12, 1, 0, "raw", 6),
    ("ref_c2_tall", 70, 1, 2, 12, 1, 0, "raw", 7),
    ("own_p2_restart3", 20, 17, 2, 12, 2, 3, "raw", 8),
    ("own_p3", 15, 23, 1, 14, 3, 0, "raw", 9),
    ("own_p4_restart1", 12, 9, 3, 16, 4, 1, "random", 10),
    ("own_p5", 18, 21, 2, 12, 5, 0, "raw", 11),
    ("own_p6_restart4", 25, 13, 1, 10, 6, 4, "raw", 12),
    ("own_p7", 14, 30, 4, 16, 7, 0, "halfscale", 13),
    ("own_p1_restart2", 11, 40, 2, 12, 1, 2, "raw", 14),
]


def samples(rows, cols, comps, precision, kind, seed):
    """(rows, cols * comps) uint16 samples of `precision` bits: raw-like (smooth rows plus
    noise), uniform random, values at 0 and half scale (differences of exactly 32768 at 16
    bits, category 16), or one flat value."""
    rng = np.random.default_rng(seed)
    top = (1 << precision) - 1
    if kind == "random":
        a = rng.integers(0, top + 1, (rows, cols * comps))
    elif kind == "halfscale":
        a = np.where(rng.integers(0, 2, (rows, cols * comps)) == 1, 1 << (precision - 1), 0)
    elif kind == "flat":
        a = np.full((rows, cols * comps), int(rng.integers(0, top + 1)))
    else:
        base = rng.uniform(0.1, 0.6) * top
        a = base + np.cumsum(rng.normal(0, top / 400, (rows, cols * comps)), axis=1) + rng.normal(0, top / 200, (rows, cols * comps))
        a = np.clip(np.rint(a), 0, top)
    return a.astype(np.uint16)
