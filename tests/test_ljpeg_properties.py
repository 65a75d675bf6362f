"""Randomised properties of the lossless-JPEG path on the CPU, over sizes, component counts,
precisions, predictors and restart intervals: the oracle's encoder and decoder round-trip
every sample array, and the product's host header parser (gls_lossless_jpeg_info) reads back
exactly the parameters the stream was written with."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings  # noqa: E402
from hypothesis import strategies as hs  # noqa: E402

from climage_gb300 import gls  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from tests import lj92_cases  # noqa: E402


@settings(max_examples=150, deadline=None)
@given(rows=hs.integers(1, 24), cols=hs.integers(1, 24), comps=hs.integers(1, 4), precision=hs.integers(8, 16),
       predictor=hs.integers(1, 7), restart_rows=hs.integers(0, 4),
       kind=hs.sampled_from(["raw", "random", "halfscale", "flat"]), seed=hs.integers(0, 2**31 - 1))
def test_round_trip_and_header(rows, cols, comps, precision, predictor, restart_rows, kind, seed):
    x = lj92_cases.samples(rows, cols, comps, precision, kind, seed)
    st = orc.lj92_encode(x, comps, precision, predictor, restart_rows)
    dec, _ = orc.lj92_decode(st)
    np.testing.assert_array_equal(dec, x)
    info = gls.lossless_jpeg_info(st)
    assert (info["height"], info["width"], info["components"], info["precision"]) == (rows, cols, comps, precision)
    assert info["predictor"] == predictor
    assert info["restart_interval"] == restart_rows * cols
    assert info["point_transform"] == 0
    if comps == 1:
        assert info["tables_alike"] == 1
