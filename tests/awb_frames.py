"""Seeded raw frames for the autoWhiteBalance tests and fixtures.

Two kinds: scene frames (climage_gb300.synthetic, 12/14-bit, the camera matrix of the
pipeline tests) and crafted 16-bit frames that reach the corners of the algorithm: quads
clipped at 1 (highlights), quads whose luma rounds into the top bin, and dark quads below
the black level whose negative luma bin the reference maps to the top bin."""
import numpy as np

from climage_gb300 import configs, synthetic

# (name, kind, width, height, bayer, seed, options)
CASES = [
    ("scene_rggb", "scene", 640, 480, 2, 10, {}),
    ("scene_grbg_gain8", "scene", 1000, 750, 0, 11, {"gain": 8.0}),
    ("scene_gbrg_14bit", "scene", 512, 384, 1, 12, {"bits": 14}),
    ("scene_bggr_odd", "scene", 333, 250, 3, 13, {}),
    ("scene_rggb_tiny", "scene", 7, 9, 2, 14, {}),
    ("scene_gbrg_noisy", "scene", 402, 302, 1, 17, {"read_sigma": 30.0, "gain": 16.0}),
    ("crafted_sat", "crafted", 400, 300, 0, 1, {"sat": 0.1, "dark": 0.3}),
    ("crafted_sat_heavy", "crafted", 257, 183, 1, 2, {"sat": 0.3, "dark": 0.05}),
    ("crafted_dark", "crafted", 520, 260, 2, 3, {"sat": 0.02, "dark": 0.3}),
    ("crafted_mixed", "crafted", 96, 64, 3, 4, {"sat": 0.1, "dark": 0.05}),
    ("crafted_wide", "crafted", 1203, 97, 2, 5, {"sat": 0.3, "dark": 0.3}),
    ("crafted_small", "crafted", 12, 16, 0, 6, {"sat": 0.3, "dark": 0.3}),
]

CRAFTED_BLACK = 360.0
CRAFTED_SCALE_MUL = [1.02, 1.0, 1.03, 1.0]


def crafted(w, h, seed, sat, dark):
    """Near-neutral 16-bit quads (black level 360) with a fraction `sat` clipped at 65535
    and a fraction `dark` below black with a tint that keeps them near white."""
    rng = np.random.default_rng(seed)
    L = rng.uniform(0, 1, (h // 2, w // 2)) ** 2
    L[rng.uniform(size=L.shape) < dark] = -1.0
    L[rng.uniform(size=L.shape) < sat] = 1.2
    tint = 1 + 0.03 * rng.normal(size=(h // 2, w // 2, 4))
    quad = CRAFTED_BLACK + L[..., None] * (65535 - CRAFTED_BLACK) * tint
    low = L == -1.0
    quad[low] = np.array([200.0, 0.0, 250.0, 0.0]) + rng.uniform(0, 8, size=(int(low.sum()), 4))
    raw = np.zeros((h // 2 * 2, w // 2 * 2))
    raw[0::2, 0::2] = quad[..., 0]
    raw[0::2, 1::2] = quad[..., 1]
    raw[1::2, 1::2] = quad[..., 2]
    raw[1::2, 0::2] = quad[..., 3]
    return np.clip(np.rint(raw + rng.normal(0, 3, raw.shape)), 0, 65535).astype(np.uint16)


def make(case, cam_ycbcr):
    """(raw, rgb_ycbcr (3, 3), scale_mul[4], white, black, bayer) of a case; cam_ycbcr is
    the function that turns rgb_cam into the camera->YCbCr matrix."""
    name, kind, w, h, bayer, seed, opt = case
    if kind == "scene":
        raw, _, meta = synthetic.make_frame(w, h, bayer=bayer, seed=seed, **opt)
        spec = configs.make_spec(meta, levels=4)
        m = cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
        return raw, m, list(spec["scale_mul"]), float(meta["white"]), float(meta["black"]), bayer
    raw = crafted(w, h, seed, **opt)
    m = cam_ycbcr(np.eye(3, dtype=np.float32))
    return raw, m, CRAFTED_SCALE_MUL, 65535.0, CRAFTED_BLACK, bayer
