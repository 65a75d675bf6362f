"""Seeded raw frames with a ColorChecker chart, for the calibration tests and fixtures.

The chart's 24 patches carry the chart's D65 colours (xyY -> XYZ -> linear sRGB, clipped),
over a textured background, mosaicked with shot and read noise by climage_gb300.synthetic."""
import numpy as np

from climage_gb300 import synthetic

GMB_XYY = [(0.400, 0.350, 10.1), (0.377, 0.345, 35.8), (0.247, 0.251, 19.3), (0.337, 0.422, 13.3),
           (0.265, 0.240, 24.3), (0.261, 0.343, 43.1), (0.506, 0.407, 30.1), (0.211, 0.175, 12.0),
           (0.453, 0.306, 19.8), (0.285, 0.202, 6.6), (0.380, 0.489, 44.3), (0.473, 0.438, 43.1),
           (0.187, 0.129, 6.1), (0.305, 0.478, 23.4), (0.539, 0.313, 12.0), (0.448, 0.470, 59.1),
           (0.364, 0.233, 19.8), (0.196, 0.252, 19.8), (0.310, 0.316, 90.0), (0.310, 0.316, 59.1),
           (0.310, 0.316, 36.2), (0.310, 0.316, 19.8), (0.310, 0.316, 9.0), (0.310, 0.316, 3.1)]
XYZ_TO_SRGB = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560],
                        [0.0556434, -0.2040259, 1.0572252]])

# (name, width, height, chart x, y, w, h, bayer, bits, gain, read sigma, rotate_180, seed)
CASES = [
    ("rggb12", 640, 480, 80, 60, 480, 320, 2, 12, 2.0, 3.0, 0, 1),
    ("grbg14_odd_chart", 700, 520, 101, 77, 493, 331, 0, 14, 4.0, 6.0, 0, 2),
    ("bggr12_rotated", 512, 384, 40, 30, 430, 300, 3, 12, 1.0, 2.0, 1, 3),
    ("gbrg10_noisy", 600, 400, 60, 50, 470, 290, 1, 10, 8.0, 4.0, 0, 4),
]


def make(case):
    """(raw uint16, black, white, bayer, gmb (x, y, w, h), rotate_180)"""
    name, w, h, cx, cy, cw, ch, bayer, bits, gain, sigma, rot, seed = case
    scene = synthetic.make_scene(w, h, seed, n_rects=4) * 0.5 + 0.1
    pw, ph = cw // 6, ch // 4
    for q, (x, y, Y) in enumerate(GMB_XYY):
        r, c = divmod(q, 6)
        if rot:
            r, c = 3 - r, 5 - c
        X, Z = Y * x / y, Y * (1 - x - y) / y
        rgb = np.clip(XYZ_TO_SRGB @ np.array([X, Y, Z]) / 100.0, 0.002, 1.0)
        scene[cy + r * ph:cy + (r + 1) * ph, cx + c * pw:cx + (c + 1) * pw, :] = rgb
    black, white = {10: 16, 12: 64, 14: 256}[bits], (1 << bits) - 1
    raw = synthetic.mosaic(scene.astype(np.float32), bayer, black, white, (2.0, 1.0, 1.6), gain, sigma, seed)
    return raw, float(black), float(white), bayer, (cx, cy, cw, ch), rot
