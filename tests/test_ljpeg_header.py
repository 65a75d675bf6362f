"""The DNG decoder's host-side header parser (gls_lossless_jpeg_info, no GPU needed): on the
golden streams it reads what the oracle's decoder reads (the oracle is pinned against the
reference's decoder); its tables-alike flag, which picks one-codeword decode units, agrees
with a separate reading of the streams' DHT segments; malformed headers are rejected."""
import json
import os

import numpy as np
import pytest

from climage_gb300 import gls, synthetic
from oracle import oracle as orc
from tests import lj92_cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def dht_tables(stream):
    """{table id: (bits[16], values)} of the DHT segments before the scan."""
    b = bytes(stream)
    i, out = 2, {}
    while i + 4 <= len(b) and b[i] == 0xFF:
        marker, length = b[i + 1], (b[i + 2] << 8) | b[i + 3]
        if marker == 0xC4:
            j = i + 4
            while j < i + 2 + length:
                bits = list(b[j + 1:j + 17])
                n = sum(bits)
                out[b[j] & 15] = (bits, list(b[j + 17:j + 17 + n]))
                j += 17 + n
        if marker == 0xDA:
            break
        i += 2 + length
    return out


def scan_tables(stream):
    """The table id of each scan component, in scan order."""
    b = bytes(stream)
    i = 2
    while b[i + 1] != 0xDA:
        i += 2 + ((b[i + 2] << 8) | b[i + 3])
    ns = b[i + 4]
    return [b[i + 6 + 2 * k] >> 4 for k in range(ns)]


def parse_alike(stream):
    """Whether every scan table splits bits alike: the same code lengths and, code by code,
    the same number of extra bits (category s reads s bits, 16 none, above 16 must match)."""
    tabs = dht_tables(stream)
    ids = scan_tables(stream)
    extra = lambda s: s if s < 16 else (0 if s == 16 else -s)
    b0, v0 = tabs[ids[0]]
    for t in ids[1:]:
        b, v = tabs[t]
        if b != b0 or [extra(s) for s in v] != [extra(s) for s in v0]:
            return False
    return True


def test_golden_streams_read_as_the_oracle_reads_them():
    with open(os.path.join(GOLDEN, "ref_lj92.json")) as f:
        meta = json.load(f)
    streams = np.load(os.path.join(GOLDEN, "ref_lj92.npz"))
    for name, m in meta.items():
        st = streams[name].tobytes()
        info = gls.lossless_jpeg_info(st)
        _, oinfo = orc.lj92_decode(st)
        assert (info["height"], info["width"], info["components"], info["predictor"]) == (
            oinfo["height"], oinfo["width"], oinfo["components"], oinfo["predictor"]), name
        assert (info["height"], info["width"], info["components"], info["precision"]) == (
            m["rows"], m["cols"], m["components"], m["precision"]), name
        assert info["restart_interval"] == m["restart_rows"] * m["cols"], name
        assert info["point_transform"] == 0
        assert info["tables_alike"] == int(parse_alike(st)), name


@pytest.mark.parametrize("comps", [1, 2, 4])
def test_tables_alike_flag(comps):
    """Whole-frame Bayer streams and small tiles, whose per-component tables may or may not
    parse alike: the flag follows the tables, and one component is always alike."""
    raw, _, _ = synthetic.make_frame(512, 384, bayer=2, gain=4.0, seed=60 + comps)
    seen = set()
    for img in (raw, raw[:64, :128], raw[128:192, 256:384]):
        st = orc.lj92_encode(np.ascontiguousarray(img), comps, 12, 1, 0)
        info = gls.lossless_jpeg_info(st)
        assert info["components"] == comps and info["width"] * comps == img.shape[1]
        assert info["tables_alike"] == int(parse_alike(st))
        seen.add(info["tables_alike"])
    if comps == 1:
        assert seen == {1}


def test_malformed_headers():
    x = lj92_cases.samples(16, 16, 1, 12, "raw", 1)
    st = orc.lj92_encode(x, 1, 12, 1, 0)
    assert gls.lossless_jpeg_info(st)["width"] == 16
    sof = st.index(b"\xff\xc3")
    bad = {
        "truncated": st[:10],
        "no SOI": b"\x00\x00" + st[2:],
        "2x2 sampling": st[:sof + 11] + b"\x22" + st[sof + 12:],
        "precision 1": st[:sof + 4] + b"\x01" + st[sof + 5:],
    }
    for what, b in bad.items():
        with pytest.raises(gls.GlsError) as e:
            gls.lossless_jpeg_info(b)
        assert e.value.status == gls.GLS_ERR_BAD_STREAM, what
