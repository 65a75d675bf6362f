"""The DNG lossless-JPEG decoder on the GPU (gls_dng_decode_lossless_jpeg, through the C ABI)
against the reference decoder's output (tests/golden/ref_lj92.*, streams written by the
reference's own encoder and by the oracle's) and against the samples that were encoded:
single streams, tiled images clipped at the border, a 4032x3024 strip, every predictor,
restart intervals, and malformed streams."""
import hashlib
import json
import os

import numpy as np
import pytest

from climage_gb300 import gls, synthetic
from oracle import oracle as orc
from tests import lj92_cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def decode(ctx, streams, tile_w, tile_h, width, height):
    """Concatenate the streams in one host buffer and decode them into a (height, width) image."""
    import torch
    offs, sizes, parts, o = [], [], [], 0
    for s in streams:
        offs.append(o)
        sizes.append(len(s))
        parts.append(s)
        o += len(s) + 3  # a few unrelated bytes between the streams
        parts.append(b"\x00\xff\x00")
    out = torch.full((height, width), 0xABCD, dtype=torch.int32).to(torch.uint16).cuda()
    ctx.decodeLosslessJPEG(b"".join(parts), offs, sizes, tile_w, tile_h, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_golden_streams(ctx):
    with open(os.path.join(GOLDEN, "ref_lj92.json")) as f:
        meta = json.load(f)
    streams = np.load(os.path.join(GOLDEN, "ref_lj92.npz"))
    for name, m in meta.items():
        w, h = m["cols"] * m["components"], m["rows"]
        got = decode(ctx, [streams[name].tobytes()], w, h, w, h)
        assert hashlib.sha256(got.tobytes()).hexdigest() == m["samples_sha256"], name


@pytest.mark.parametrize("case", lj92_cases.CASES, ids=[c[0] for c in lj92_cases.CASES])
def test_round_trip_larger(ctx, case):
    name, rows, cols, comps, prec, pred, rst, kind, seed = case
    rows, cols = rows * 7 + 3, cols * 5 + 1
    x = lj92_cases.samples(rows, cols, comps, prec, kind, seed + 500)
    st = orc.lj92_encode(x, comps, prec, pred, rst)
    got = decode(ctx, [st], cols * comps, rows, cols * comps, rows)
    np.testing.assert_array_equal(got, x)


@pytest.mark.parametrize("comps", [1, 2])
def test_tiled_image_clipped_at_the_border(ctx, comps):
    """A 300x200 frame in 64x48 tiles (edge tiles padded to full size, as DNG writers do),
    each tile its own stream, decoded in one call."""
    raw, _, _ = synthetic.make_frame(300, 200, bayer=2, seed=4)
    tw, th = 64, 48
    ta, td = -(-300 // tw), -(-200 // th)
    padded = np.zeros((td * th, ta * tw), np.uint16)
    padded[:200, :300] = raw
    streams = []
    for ty in range(td):
        for tx in range(ta):
            tile = padded[ty * th:(ty + 1) * th, tx * tw:(tx + 1) * tw]
            streams.append(orc.lj92_encode(tile, comps, 12, 1, 0))
    got = decode(ctx, streams, tw, th, 300, 200)
    np.testing.assert_array_equal(got, raw)


def test_full_size_strip(ctx):
    """One 4032x3024 12-bit strip, one component: the layout the reference's DNG writer uses."""
    raw, _, _ = synthetic.make_frame(4032, 3024, bayer=2, gain=4.0, seed=12)
    st = orc.lj92_encode(raw, 1, 12, 1, 0)
    got = decode(ctx, [st], 4032, 3024, 4032, 3024)
    np.testing.assert_array_equal(got, raw)


def test_full_size_two_components_restarts(ctx):
    raw, _, _ = synthetic.make_frame(2016, 1512, bayer=1, gain=16.0, read_sigma=20.0, seed=13)
    st = orc.lj92_encode(raw, 2, 12, 1, 7)
    got = decode(ctx, [st], 2016, 1512, 2016, 1512)
    np.testing.assert_array_equal(got, raw)


@pytest.mark.parametrize("comps", [1, 2, 4])
def test_flat_areas(ctx, comps):
    """Clipped areas and a black border: long runs of zero differences (runs of zero bits in
    the stream, which a decode started inside them cannot place by itself)."""
    raw, _, _ = synthetic.make_frame(1024, 768, bayer=2, gain=2.0, seed=20 + comps)
    raw[100:400, 100:900] = 4095
    raw[500:, :] = 64
    raw[600:700, 300:310] = 1000
    st = orc.lj92_encode(raw, comps, 12, 1, 0)
    got = decode(ctx, [st], 1024, 768, 1024, 768)
    np.testing.assert_array_equal(got, raw)


def test_all_zero_frame(ctx):
    raw = np.zeros((512, 640), np.uint16)
    for comps in (1, 2):
        st = orc.lj92_encode(raw, comps, 14, 1, 0)
        np.testing.assert_array_equal(decode(ctx, [st], 640, 512, 640, 512), raw)


def test_malformed_streams(ctx):
    import torch
    x = lj92_cases.samples(16, 16, 1, 12, "raw", 1)
    st = orc.lj92_encode(x, 1, 12, 1, 0)
    out = torch.zeros((16, 16), dtype=torch.int32).to(torch.uint16).cuda()
    for bad in (st[:10], b"\x00\x00" + st[2:]):
        with pytest.raises(gls.GlsError) as e:
            ctx.decodeLosslessJPEG(bad, [0], [len(bad)], 16, 16, out)
        assert e.value.status == gls.GLS_ERR_BAD_STREAM
    with pytest.raises(gls.GlsError) as e:  # the stream decodes to 16x16, the tile is 16x8
        ctx.decodeLosslessJPEG(st, [0], [len(st)], 16, 8, out)
    assert e.value.status == gls.GLS_ERR_BAD_STREAM
