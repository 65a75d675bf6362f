"""Seeded synthetic RAW frames: the stand-in for camera DNG inputs.

The reference ships no RAW sample (its Kodak round-trip set, raw_pipeline.cpp:148-214, is
not in the tree), so every workload here is rendered from a seeded linear-RGB scene:
smooth 2-D gradients, random axis-aligned rectangles with sharp edges (a few of them
brighter than the sensor clip, to drive highlight recovery) and oriented sinusoidal
texture.  The scene is mosaicked with the kernel CFA table (demosaic.cl:29-34), scaled to
DN = black + scene_c * (white - black) / wb_c so that the white-balance gains restore a
neutral scene, and degraded by Poisson shot noise (gain e-/DN) plus Gaussian read noise.

The random source is numpy's Philox-4x32-10 counter-based generator keyed by the seed, so
a frame is the same on every machine.
"""
import numpy as np

# Kernel CFA table (x, y) per {red, green, blue, green2}, demosaic.cl:29-34
BAYER_OFFSETS = {
    0: ((1, 0), (0, 0), (0, 1), (1, 1)),  # grbg
    1: ((0, 1), (0, 0), (1, 0), (1, 1)),  # gbrg
    2: ((0, 0), (0, 1), (1, 1), (1, 0)),  # rggb
    3: ((1, 1), (0, 1), (0, 0), (1, 0)),  # bggr
}
BAYER_NAMES = {"grbg": 0, "gbrg": 1, "rggb": 2, "bggr": 3}


def _rng(seed):
    return np.random.Generator(np.random.Philox(key=int(seed) & ((1 << 64) - 1)))


def make_scene(width, height, seed, n_rects=None, blur_sigma=0.7):
    """Linear RGB scene, float32 (height, width, 3), mostly in [0, 1].

    Colours are drawn as a grey level plus a moderate chroma offset (natural-scene
    saturation), and the scene is blurred by a small Gaussian standing in for the lens
    and optical low-pass filter, so that edges are sharp but not aliased.
    """
    rng = _rng(seed)
    y = np.linspace(0.0, 1.0, height, dtype=np.float32)[:, None]
    x = np.linspace(0.0, 1.0, width, dtype=np.float32)[None, :]
    scene = np.empty((height, width, 3), np.float32)
    a, bx, by, cxy = rng.uniform(0.15, 0.45), rng.uniform(-0.25, 0.25), rng.uniform(-0.25, 0.25), rng.uniform(-0.3, 0.3)
    base = a + bx * x + by * y + cxy * (x - 0.5) * (y - 0.5)
    for c in range(3):
        scene[:, :, c] = base * np.float32(rng.uniform(0.85, 1.15))
    if n_rects is None:
        n_rects = int(rng.integers(32, 257))
    for _ in range(n_rects):
        rw = int(rng.integers(max(2, width // 64), max(3, width // 4)))
        rh = int(rng.integers(max(2, height // 64), max(3, height // 4)))
        x0 = int(rng.integers(0, max(1, width - rw)))
        y0 = int(rng.integers(0, max(1, height - rh)))
        if rng.uniform() < 0.06:
            grey, sat = rng.uniform(0.8, 1.5), 0.1
        else:
            grey, sat = rng.uniform(0.0, 0.9) ** 1.5 + 0.005, 0.35
        color = grey * (1.0 + sat * rng.uniform(-1.0, 1.0, 3))
        scene[y0:y0 + rh, x0:x0 + rw, :] = np.maximum(color, 0.0).astype(np.float32)
    # oriented sinusoidal texture, 0.01 .. 0.25 cycles per pixel
    xx = np.arange(width, dtype=np.float32)[None, :]
    yy = np.arange(height, dtype=np.float32)[:, None]
    for _ in range(3):
        f = rng.uniform(0.01, 0.25)
        th = rng.uniform(0, np.pi)
        ph = rng.uniform(0, 2 * np.pi)
        amp = rng.uniform(0.02, 0.06)
        t = amp * np.sin((2 * np.pi * f) * (xx * np.float32(np.cos(th)) + yy * np.float32(np.sin(th))) + ph)
        gains = rng.uniform(0.8, 1.0, 3).astype(np.float32)
        scene += t[:, :, None].astype(np.float32) * gains[None, None, :]
    if blur_sigma > 0:
        scene = _blur(scene, blur_sigma)
    np.clip(scene, 0.0, 2.0, out=scene)
    return scene


def _blur(img, sigma):
    """Separable Gaussian blur (edge-replicated), float32."""
    r = int(np.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-r, r + 1, dtype=np.float64) / sigma) ** 2)
    k = (k / k.sum()).astype(np.float32)
    out = img
    for axis in (0, 1):
        pad = [(0, 0)] * out.ndim
        pad[axis] = (r, r)
        p = np.pad(out, pad, mode="edge")
        acc = np.zeros_like(out)
        n = out.shape[axis]
        for i, w in enumerate(k):
            sl = [slice(None)] * out.ndim
            sl[axis] = slice(i, i + n)
            acc += w * p[tuple(sl)]
        out = acc
    return out


def mosaic(scene, bayer, black, white, wb, gain, read_sigma, seed):
    """Bayer-mosaic a linear scene into uint16 DN with shot + read noise."""
    rng = _rng(seed ^ 0x5A5A5A5A)
    h, w, _ = scene.shape
    off = BAYER_OFFSETS[bayer]
    cfa_channel = (0, 1, 2, 1)
    dn = np.empty((h, w), np.float32)
    span = float(white - black)
    for c in range(4):
        ox, oy = off[c]
        ch = cfa_channel[c]
        dn[oy::2, ox::2] = scene[oy::2, ox::2, ch] * np.float32(span / wb[ch])
    signal = np.maximum(dn, 0.0)
    if gain > 0:
        electrons = rng.poisson(signal.astype(np.float64) * gain).astype(np.float32)
        signal = electrons / np.float32(gain)
    noisy = black + signal + rng.normal(0.0, read_sigma, size=(h, w)).astype(np.float32)
    return np.clip(np.rint(noisy), 0, white).astype(np.uint16)


def clean_reference(scene):
    """Ground-truth linear scene clipped to the sensor range (for PSNR against clean)."""
    return np.clip(scene, 0.0, 1.0)


def make_frame(width, height, bayer=2, bits=12, black=None, white=None, wb=(2.0, 1.0, 1.6), gain=2.0,
               read_sigma=3.0, seed=0):
    """One synthetic frame; returns (raw uint16 (h, w), scene float32 (h, w, 3), meta dict)."""
    if white is None:
        white = (1 << bits) - 1
    if black is None:
        black = {10: 16, 12: 64, 14: 256, 16: 1024}[bits]
    scene = make_scene(width, height, seed)
    raw = mosaic(scene, bayer, black, white, wb, gain, read_sigma, seed)
    meta = dict(bayer=bayer, black=black, white=white, wb=tuple(wb), gain=gain, read_sigma=read_sigma, bits=bits)
    return raw, scene, meta


def pack_bits(samples, bits):
    """uint16 samples -> MSB-first packed bytes (the DNG bit order unpacked by
    unpack12BitsInto16Bits / unpack14BitsInto16Bits, src/gls_image_tiff.cpp:53-87)."""
    s = np.ascontiguousarray(samples, dtype=np.uint32).ravel()
    n = s.size
    g = 8 // np.gcd(bits, 8)  # samples per whole number of bytes
    if n % g == 0 and g * bits <= 64:
        # groups of g samples fill g * bits / 8 bytes exactly: assemble each group in a uint64
        grp = s.reshape(-1, g).astype(np.uint64)
        acc = np.zeros(grp.shape[0], np.uint64)
        for j in range(g):
            acc = (acc << np.uint64(bits)) | grp[:, j]
        nb = g * bits // 8
        out = np.empty((grp.shape[0], nb), np.uint8)
        for k in range(nb):
            out[:, k] = ((acc >> np.uint64(8 * (nb - 1 - k))) & np.uint64(0xFF)).astype(np.uint8)
        return out.tobytes()
    total_bits = n * bits
    out = np.zeros((total_bits + 7) // 8, np.uint8)
    bitpos = np.arange(n, dtype=np.int64) * bits
    for b in range(bits):
        bit = (s >> (bits - 1 - b)) & 1
        pos = bitpos + b
        np.bitwise_or.at(out, pos >> 3, (bit << (7 - (pos & 7))).astype(np.uint8))
    return out.tobytes()
