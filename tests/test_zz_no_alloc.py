"""gls_guided_filter_noalloc: GuidedFilter::filter over the library's static scratch array.

It is checked through the C ABI against gls_guided_filter (the entry point with cudaMalloc'd
scratch, itself parity-tested against the oracle): bit for bit, on calls in a row, at the
size limit, and for the rejection of larger images.  The file is collected last, so its
first call on the device comes either in a fresh process or after every other test; both
must pass.
"""
import os
import re
import subprocess

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
def test_matches_oracle(nctx):
    import torch

    from oracle import oracle as orc
    rng = np.random.default_rng(7)
    img = _image(rng, 67, 45, False)
    out = _like(img, float("nan"))
    nctx.guidedFilterNoAlloc(img, 5, EPS_A, out)
    torch.cuda.synchronize()
    want = orc.guided_filter(img.cpu().numpy(), 5, EPS_A)
    assert np.array_equal(out.cpu().numpy().view(np.int32), want.view(np.int32))


@pytest.mark.gpu
@pytest.mark.parametrize("half", [False, True], ids=["f32", "f16"])
def test_pitched_images_match_existing_entry_point(nctx, half):
    """Input and output rows padded (column slices of wider images: the row pitch is larger
    than the width), which the first box-blur pass and the final write must honour."""
    import torch
    rng = np.random.default_rng(41 + half)
    wide = _image(rng, 160, 90, half)
    img = wide[:, 7:7 + 121]  # pitch 160 pixels, width 121
    assert img.stride(0) == 160 * 4
    ref_wide, out_wide = _like(wide, 0.5), _like(wide, float("nan"))
    ref, out = ref_wide[:, 13:13 + 121], out_wide[:, 13:13 + 121]
    nctx.guidedFilter(img, 5, EPS_A, ref)
    nctx.guidedFilterNoAlloc(img, 5, EPS_A, out)
    nctx.guidedFilterNoAlloc(img, 5, EPS_A, out)
    torch.cuda.synchronize()
    assert _same(out, ref)
    # the padding columns of the output stay as they were
    assert bool(torch.isnan(out_wide[:, :13]).all()) and bool(torch.isnan(out_wide[:, 13 + 121:]).all())


@pytest.mark.gpu
def test_other_current_device_is_rejected(nctx):
    """Every call needs the context's device current; with another device current the call is
    rejected before it launches anything (needs two GPUs)."""
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    img = _image(np.random.default_rng(8), 40, 30, False)
    out = _like(img, 0.25)
    launches = nctx.kernel_launches()
    with torch.cuda.device(1):
        with pytest.raises(gls.GlsError) as err:
            nctx.guidedFilterNoAlloc(img, 3, EPS_A, out)
    assert err.value.status == gls.GLS_ERR_INVALID_ARGUMENT
    assert nctx.kernel_launches() == launches


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



SLOT_TEST = r"""
#include <cstdio>
#include "gls_scratch_slot.h"
static int lookups = 0;
static unsigned long long live = 0;  // the context a lookup finds current
static char mem[3];
int main() {
    gls::ScratchSlot s;
    auto lookup = [](unsigned long long* id) -> void* { ++lookups; *id = live; return live ? &mem[live - 1] : nullptr; };
    int bad = 0;
    live = 1;
    bad += gls::scratch_slot_get(s, 0, lookup) != &mem[0] || lookups != 1;   // nothing current yet: set-up
    bad += gls::scratch_slot_get(s, 1, lookup) != &mem[0] || lookups != 1;   // same context: cached
    bad += gls::scratch_slot_get(s, 1, lookup) != &mem[0] || lookups != 1;
    live = 2;                                                                // a device reset: new context id
    bad += gls::scratch_slot_get(s, 2, lookup) != &mem[1] || lookups != 2;   // looked up again
    bad += gls::scratch_slot_get(s, 2, lookup) != &mem[1] || lookups != 2;
    live = 0;                                                                // a failed lookup
    bad += gls::scratch_slot_get(s, 3, lookup) != nullptr || lookups != 3;
    bad += s.ctx_id != 2 || s.ptr != &mem[1];                                // cache unchanged
    live = 3;
    bad += gls::scratch_slot_get(s, 3, lookup) != &mem[2] || lookups != 4;
    std::printf("%d\n", bad);
    return bad;
}
"""


def test_address_is_looked_up_again_in_a_new_context(tmp_path):
    """The cache of the array's address is keyed on the CUDA context: the same context reuses
    it, a new one (after a device reset) repeats the lookup, a failed lookup caches nothing.
    Host logic, compiled with the host compiler against the header the library uses."""
    src = tmp_path / "slot.cpp"
    src.write_text(SLOT_TEST)
    exe = tmp_path / "slot"
    cc = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "climage_gb300", "csrc"), str(src), "-o",
                         str(exe)], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "0", r.stdout + r.stderr
