"""Randomised check of the product's host colour math (gls_cam_xyz_coeff, gls_cam_ycbcr,
gls_inverse3x3) against the reference's own compiled code (oracle/_ref): camera matrices
drawn around a real one (each entry scaled by up to +-25 %) give the same bits.  Runs where
the reference's code was built (skipped elsewhere)."""
import ctypes

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings  # noqa: E402
from hypothesis import strategies as hs  # noqa: E402
from hypothesis.extra import numpy as hnp  # noqa: E402

from climage_gb300 import configs, gls  # noqa: E402
from oracle import oracle as orc  # noqa: E402

REF = orc.ref_lib()
pytestmark = pytest.mark.skipif(REF is None, reason="the reference's host code is not built here")

F9 = ctypes.c_float * 9


def ref_m9(fn, m):
    out = F9()
    fn(F9(*[float(v) for v in np.ravel(m)]), out)
    return np.array(out[:], np.float32)


@settings(max_examples=200, deadline=None)
@given(scale=hnp.arrays(np.float32, (3, 3), elements=hs.floats(0.75, 1.25, width=32)))
def test_host_colour_math_equals_reference(scale):
    cam_xyz = (np.asarray(configs.CAM_XYZ, np.float32).reshape(3, 3) * scale).astype(np.float32)
    pre, rgb_cam = gls.cam_xyz_coeff(cam_xyz)
    rpre, rrgb = (ctypes.c_float * 3)(), F9()
    REF.ref_cam_xyz_coeff(F9(*[float(v) for v in cam_xyz.ravel()]), rpre, rrgb)
    np.testing.assert_array_equal(pre.view(np.uint32), np.array(rpre[:], np.float32).view(np.uint32))
    np.testing.assert_array_equal(rgb_cam.ravel().view(np.uint32), np.array(rrgb[:], np.float32).view(np.uint32))
    cy = gls.cam_ycbcr(rgb_cam)
    np.testing.assert_array_equal(cy.ravel().view(np.uint32), ref_m9(REF.ref_cam_ycbcr, rgb_cam).view(np.uint32))
    inv = gls.inverse3x3(cy)
    np.testing.assert_array_equal(inv.ravel().view(np.uint32), ref_m9(REF.ref_inverse3x3, cy).view(np.uint32))
