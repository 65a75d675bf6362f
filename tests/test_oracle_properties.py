"""Randomised pins of the oracle against the reference's own compiled code (oracle/_ref), on
the CPU: autoWhiteBalance on random frames (sizes, CFA phases, gains, noise, white-balance
multipliers) gives the same gains and highlight fraction bit for bit, and the reference's
lossless-JPEG decoder reads every stream the oracle's encoder writes (predictors 1-7,
restart intervals) back to the samples.  Runs where the reference's code was built."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings  # noqa: E402
from hypothesis import strategies as hs  # noqa: E402

from climage_gb300 import configs, gls, synthetic  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from tests import lj92_cases  # noqa: E402

pytestmark = pytest.mark.skipif(orc.ref_lib() is None, reason="the reference's host code is not built here")


@settings(max_examples=40, deadline=None)
@given(w=hs.integers(8, 40).map(lambda v: 8 * v), h=hs.integers(8, 30).map(lambda v: 8 * v),
       bayer=hs.integers(0, 3), gain=hs.floats(0.25, 16.0), read_sigma=hs.floats(0.5, 20.0),
       wb_r=hs.floats(1.0, 3.0), wb_b=hs.floats(1.0, 3.0), seed=hs.integers(0, 2**20))
def test_auto_white_balance_equals_reference(w, h, bayer, gain, read_sigma, wb_r, wb_b, seed):
    raw, _, meta = synthetic.make_frame(w, h, bayer=bayer, gain=gain, read_sigma=read_sigma,
                                        wb=(wb_r, 1.0, wb_b), seed=seed)
    spec = configs.make_spec(meta, levels=4)
    cy = gls.cam_ycbcr(np.array(spec["rgb_cam"], np.float32).reshape(3, 3))
    args = (cy, spec["scale_mul"], spec["white_level"], spec["black_level"], bayer)
    wb, hl = orc.auto_white_balance(raw, *args)
    rwb, rhl = orc.auto_white_balance(raw, *args, reference=True)
    np.testing.assert_array_equal(np.asarray(wb, np.float32).view(np.uint32), np.asarray(rwb, np.float32).view(np.uint32))
    assert np.float32(hl).view(np.uint32) == np.float32(rhl).view(np.uint32)


@settings(max_examples=80, deadline=None)
@given(rows=hs.integers(1, 24), cols=hs.integers(1, 24), comps=hs.integers(1, 4), precision=hs.integers(8, 16),
       predictor=hs.integers(1, 7), restart_rows=hs.integers(0, 4),
       kind=hs.sampled_from(["raw", "random", "halfscale", "flat"]), seed=hs.integers(0, 2**31 - 1))
def test_reference_decoder_reads_the_oracle_encoder(rows, cols, comps, precision, predictor, restart_rows, kind, seed):
    x = lj92_cases.samples(rows, cols, comps, precision, kind, seed)
    st = orc.lj92_encode(x, comps, precision, predictor, restart_rows)
    dec, info = orc.lj92_decode(st, reference=True)
    np.testing.assert_array_equal(dec, x)
    assert info["predictor"] == predictor
