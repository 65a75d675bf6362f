"""CPU-only checks of the C ABI: the library loads, exports every entry point that
include/gls_cuda.h declares, and its host colour math equals the oracle's and the
reference's own (pinned by tests/golden)."""
import ctypes
import os
import re

import numpy as np
import pytest

from climage_gb300 import configs, gls

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gls_cuda.h")).read()
    return sorted(set(re.findall(r"GLS_API\s+[\w\s\*]+?\b(gls_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gls_raw_converter_demosaic" in names and "gls_interpolate_green" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(gls.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol():
    bound = {s[0] for s in gls.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_status_strings_and_version():
    l = gls.lib()
    assert l.gls_status_string(0) == b"ok"
    assert b"sm_103a" in l.gls_version()


def test_no_gpu_context_creation_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    h = ctypes.c_void_p()
    assert gls.lib().gls_ctx_create(0, ctypes.byref(h)) != 0


def test_host_colour_math_matches_oracle():
    from oracle import oracle as orc
    pre_g, rc_g = gls.cam_xyz_coeff(configs.CAM_XYZ)
    pre_o, rc_o = orc.cam_xyz_coeff(configs.CAM_XYZ)
    np.testing.assert_array_equal(pre_g, pre_o)
    np.testing.assert_array_equal(rc_g, rc_o)
    np.testing.assert_array_equal(gls.cam_ycbcr(rc_g), orc.cam_ycbcr(rc_o))
    np.testing.assert_array_equal(gls.inverse3x3(gls.cam_ycbcr(rc_g)), orc.inverse3x3(orc.cam_ycbcr(rc_o)))


def test_tuner_cache_host_logic():
    """The launch-shape tuner's process-wide cache runs on the host: forcing a shape, the
    rejected shapes, reset, and an empty cache before any frame was converted."""
    gls.tune_reset()
    assert gls.tune_entries() == []
    l = gls.lib()
    for kernel, shapes in gls.TUNE_SHAPES.items():
        for shape in range(-1, len(shapes)):
            assert l.gls_tune_force(kernel, shape) == 0
        assert l.gls_tune_force(kernel, len(shapes)) != 0
        assert l.gls_tune_force(kernel, -2) != 0
    assert l.gls_tune_force(len(gls.TUNE_SHAPES), 0) != 0
    k, w, h, f, s = (ctypes.c_int() for _ in range(5))
    ms = (ctypes.c_float * 4)()
    assert l.gls_tune_entry(0, ctypes.byref(k), ctypes.byref(w), ctypes.byref(h), ctypes.byref(f), ctypes.byref(s),
                            ms) != 0  # no entry 0 in an empty cache
    gls.tune_reset()


def test_bench_shapes_option():
    """bench.py --shapes: 'kernel=shape' pairs by name reach the tuner's forced shapes; unknown
    kernels or shapes are rejected before anything runs."""
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "gls_bench_module", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    try:
        bench.force_shapes(gls, "demosaic=split, final=32x16")
        bench.force_shapes(gls, "")
        with pytest.raises(KeyError):
            bench.force_shapes(gls, "green=split")
        with pytest.raises(ValueError):
            bench.force_shapes(gls, "final=split")
    finally:
        gls.tune_reset()
