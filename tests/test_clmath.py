"""The OpenCL built-ins of gls_clmath.h against double-precision references.

These pin the approximations both the CUDA kernels and the oracle use: transcendentals
within a few ulp of the correctly rounded value, binary16 conversion identical to
numpy's round-to-nearest-even."""
import math

import numpy as np
import pytest

from oracle import oracle as orc


def ulp_err(got, ref):
    got = np.float32(got)
    ref64 = float(ref)
    if math.isnan(ref64):
        return 0.0 if math.isnan(float(got)) else float("inf")
    if math.isinf(ref64):
        return 0.0 if got == ref64 else float("inf")
    r = np.float32(ref64)
    ulp = float(np.spacing(np.abs(r))) if r != 0 else float(np.spacing(np.float32(0)))
    return abs(float(got) - ref64) / ulp


@pytest.fixture(scope="module")
def lib():
    return orc.lib()


def test_atan2pi(lib):
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(20000):
        y, x = (rng.standard_normal(2) * 10.0 ** rng.uniform(-6, 6, 2)).astype(np.float32)
        worst = max(worst, ulp_err(lib.oracle_atan2pi(float(y), float(x)), math.atan2(float(y), float(x)) / math.pi))
    assert worst <= 4.0, worst
    # special values (C99 atan2)
    assert lib.oracle_atan2pi(0.0, 0.0) == 0.0
    assert lib.oracle_atan2pi(0.0, -0.0) == 1.0
    assert lib.oracle_atan2pi(-0.0, -0.0) == -1.0
    assert lib.oracle_atan2pi(1.0, 0.0) == 0.5
    assert lib.oracle_atan2pi(float("inf"), float("inf")) == 0.25
    assert math.isnan(lib.oracle_atan2pi(float("nan"), 1.0))


def test_tanh(lib):
    xs = np.concatenate([np.linspace(-12, 12, 20001), np.float32(10.0) ** np.linspace(-8, 1, 2000)]).astype(np.float32)
    worst = max(ulp_err(lib.oracle_tanh(float(x)), math.tanh(float(x))) for x in xs)
    assert worst <= 4.0, worst


def test_exp2_log2(lib):
    xs = np.linspace(-140, 127.9, 40001).astype(np.float32)
    assert max(ulp_err(lib.oracle_exp2(float(x)), 2.0 ** float(x)) for x in xs if x > -126) <= 2.0
    rng = np.random.default_rng(2)
    ys = (2.0 ** rng.uniform(-149, 127, 40000)).astype(np.float32)
    worst = 0.0
    for y in ys:
        ref = math.log2(float(y))
        got = lib.oracle_log2(float(y))
        err = abs(got - ref) / max(float(np.spacing(np.float32(abs(ref)))), 1e-9) if abs(ref) > 1e-3 else abs(got - ref) / 1e-9
        worst = max(worst, err)
    assert worst <= 4.0, worst
    assert lib.oracle_log2(1.0) == 0.0 and lib.oracle_log2(2.0) == 1.0
    assert lib.oracle_log2(0.0) == -float("inf") and math.isnan(lib.oracle_log2(-1.0))


def test_pow(lib):
    rng = np.random.default_rng(3)
    xs = (10.0 ** rng.uniform(-4, 1, 20000)).astype(np.float32)
    ys = rng.uniform(-2, 2, 20000).astype(np.float32)
    worst = max(ulp_err(lib.oracle_pow(float(x), float(y)), float(x) ** float(y)) for x, y in zip(xs, ys))
    assert worst <= 64.0, worst
    assert lib.oracle_pow(0.25, 0.5) == 0.5
    assert lib.oracle_pow(-8.0, 1.0) == -8.0
    assert math.isnan(lib.oracle_pow(-0.5, 0.5))
    assert lib.oracle_pow(0.0, 0.5) == 0.0


def test_half_conversion_exhaustive(lib):
    halves = np.arange(1 << 16, dtype=np.uint16)
    ref = halves.view(np.float16).astype(np.float32)
    got = np.array([lib.oracle_f16_to_f32(int(h)) for h in halves], np.float32)
    same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
    assert same.all()


def test_float_to_half_rounding(lib):
    rng = np.random.default_rng(4)
    vals = np.concatenate([
        rng.standard_normal(30000).astype(np.float32) * np.float32(10.0) ** rng.uniform(-9, 5, 30000).astype(np.float32),
        np.array([65504, 65519.99, 65520, 65536, 6.1035156e-05, 6.097555e-05, 5.9604645e-08, 2.9802322e-08,
                  2.9802326e-08, 1e-10, 0.0, -0.0, 1.0009766, 1.0004883, 1.0014648], np.float32),
    ])
    got = np.array([lib.oracle_f32_to_f16(float(v)) for v in vals], np.uint16)
    ref = vals.astype(np.float16).view(np.uint16)
    assert (got == ref).all(), vals[got != ref][:10]
