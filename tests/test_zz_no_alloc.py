"""gls_guided_filter_noalloc: GuidedFilter::filter over the library's static scratch array.

It is checked through the C ABI against gls_guided_filter (the entry point with cudaMalloc'd
scratch, itself parity-tested against the oracle): bit for bit, on calls in a row, at the
size limit, and for the rejection of larger images.  The file is collected last, so its
first call on the device comes either in a fresh process or after every other test; both
must pass.
"""
import os
import re

import numpy as np
import pytest

from climage_gb300 import gls

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EPS_A = [4e-4, 1e-4, 1.2e-4]
EPS_B = [2e-3, 5e-4, 6e-4]


def _header_define(name):
    text = open(os.path.join(ROOT, "include", "gls_cuda.h")).read()
    m = re.search(r"#define\s+%s\s+\(?(\d+)u?(?:\s*<<\s*(\d+))?\)?" % name, text)
    assert m, name
    return int(m.group(1)) << int(m.group(2) or 0)


def test_size_limit_matches_scratch_layout():
    """The limit is the largest image whose ten scratch buffers (144 bytes a pixel, each
    buffer padded to 256 bytes) fit the static array."""
    nbytes = _header_define("GLS_GUIDED_FILTER_NOALLOC_SCRATCH_BYTES")
    max_px = _header_define("GLS_GUIDED_FILTER_NOALLOC_MAX_PIXELS")
    assert nbytes == 16 << 20
    assert max_px == gls.GUIDED_FILTER_NOALLOC_MAX_PIXELS

    def need(n):
        return n * 144 + 10 * 256

    assert need(max_px) <= nbytes < need(max_px + 1)


def _image(rng, w, h, half):
    import torch
    a = rng.uniform(0.0, 1.0, (h, w, 4)).astype(np.float32)
    a[..., 3] = 0.0
    return torch.from_numpy(a).to(torch.float16 if half else torch.float32).cuda()


def _like(t, fill):
    import torch
    return torch.full_like(t, fill)


def _bits(t):
    import torch
    return t.view(torch.int16 if t.dtype == torch.float16 else torch.int32)


def _same(a, b):
    import torch
    return torch.equal(_bits(a), _bits(b))


@pytest.fixture(scope="module")
def nctx(cuda):
    c = gls.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_two_calls_in_a_row_match_existing_entry_point(nctx, half):
    import torch
    rng = np.random.default_rng(31 + half)
    a = _image(rng, 200, 150, half)
    b = _image(rng, 97, 61, half)
    ref_a, ref_b = _like(a, 0.0), _like(b, 0.0)
    nctx.guidedFilter(a, 5, EPS_A, ref_a)
    nctx.guidedFilter(b, 3, EPS_B, ref_b)
    out_a1, out_b, out_a2 = _like(a, float("nan")), _like(b, float("nan")), _like(a, float("nan"))
    # back to back on one stream, no synchronisation between them
    nctx.guidedFilterNoAlloc(a, 5, EPS_A, out_a1)
    nctx.guidedFilterNoAlloc(b, 3, EPS_B, out_b)
    nctx.guidedFilterNoAlloc(a, 5, EPS_A, out_a2)
    torch.cuda.synchronize()
    assert _same(out_a1, ref_a)
    assert _same(out_b, ref_b)
    assert _same(out_a2, ref_a)


@pytest.mark.gpu
def test_matches_oracle():
    import torch

    from oracle import oracle as orc
    c = gls.Context(0)
    try:
        rng = np.random.default_rng(7)
        img = _image(rng, 67, 45, False)
        out = _like(img, float("nan"))
        c.guidedFilterNoAlloc(img, 5, EPS_A, out)
        torch.cuda.synchronize()
        want = orc.guided_filter(img.cpu().numpy(), 5, EPS_A)
        assert np.array_equal(out.cpu().numpy().view(np.int32), want.view(np.int32))
    finally:
        c.close()


@pytest.mark.gpu
def test_largest_image_is_accepted(nctx):
    import torch
    w, h = 330, 353
    assert w * h == gls.GUIDED_FILTER_NOALLOC_MAX_PIXELS
    img = _image(np.random.default_rng(3), w, h, False)
    ref, out = _like(img, 0.0), _like(img, float("nan"))
    nctx.guidedFilter(img, 7, EPS_A, ref)
    nctx.guidedFilterNoAlloc(img, 7, EPS_A, out)
    torch.cuda.synchronize()
    assert _same(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", [(331, 353), (4032, 3024)])
def test_larger_image_is_rejected(nctx, w, h):
    import torch
    img = _image(np.random.default_rng(5), w, h, True)
    out = _like(img, 0.25)
    launches = nctx.kernel_launches()
    with pytest.raises(gls.GlsError) as err:
        nctx.guidedFilterNoAlloc(img, 5, EPS_A, out)
    assert err.value.status == gls.GLS_ERR_INVALID_SIZE
    assert "static scratch" in str(err.value) and str(gls.GUIDED_FILTER_NOALLOC_MAX_PIXELS) in str(err.value)
    assert nctx.kernel_launches() == launches
    torch.cuda.synchronize()
    assert bool((out == 0.25).all())
    # the context stays usable
    small = _image(np.random.default_rng(6), 40, 30, True)
    ref, res = _like(small, 0.0), _like(small, float("nan"))
    nctx.guidedFilter(small, 3, EPS_B, ref)
    nctx.guidedFilterNoAlloc(small, 3, EPS_B, res)
    torch.cuda.synchronize()
    assert _same(res, ref)
