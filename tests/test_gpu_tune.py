"""Launch-shape tuner: every compiled tile shape of the fused demosaic and final kernels
gives the oracle's frame bit for bit (a tile only decides which block computes a pixel), on
frames whose sizes are not multiples of any tile, in both storage precisions and both output
formats; and a converted frame leaves one timed choice per kernel for its size.
"""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic
from tests.test_gpu_pipeline import check, run_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture
def unforced():
    yield
    gls.tune_force(gls.TUNE_DEMOSAIC, -1)
    gls.tune_force(gls.TUNE_FINAL, -1)


CASES = [
    dict(w=338, h=246, bayer=1, bits=12, levels=4, storage=gls.STORAGE_F32, out_float=False, seed=61),
    dict(w=402, h=298, bayer=3, bits=14, levels=5, storage=gls.STORAGE_F16, out_float=False, seed=62),
    dict(w=290, h=214, bayer=0, bits=10, levels=4, storage=gls.STORAGE_F32, out_float=True, seed=63),
    # rows a multiple of 4 pixels: interior tiles of the split green kernel read 8-byte words
    dict(w=416, h=256, bayer=2, bits=12, levels=4, storage=gls.STORAGE_F32, out_float=False, seed=66),
]


@pytest.mark.parametrize("kernel", [gls.TUNE_DEMOSAIC, gls.TUNE_FINAL], ids=["demosaic", "final"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_every_tile_shape_equals_the_oracle(ctx, unforced, kernel, case):
    c = CASES[case]
    raw, _, meta = synthetic.make_frame(c["w"], c["h"], bayer=c["bayer"], bits=c["bits"], seed=c["seed"])
    spec = configs.make_spec(meta, levels=c["levels"], storage=c["storage"])
    for shape in range(len(gls.TUNE_SHAPES[kernel])):
        gls.tune_force(kernel, shape)
        check(ctx, raw, spec, out_float=c["out_float"])


@pytest.mark.parametrize("w,h,storage", [(258, 194, gls.STORAGE_F32), (416, 256, gls.STORAGE_F16)],
                         ids=["258x194-fp32", "416x256-fp16"])
def test_high_noise_branch_every_demosaic_shape(ctx, unforced, w, h, storage):
    # the high-noise branch feeds the demosaic pre-scaled, denoised raw (the other input form);
    # rows a multiple of 4 pixels let interior tiles read it in words of 4 pixels
    raw, _, meta = synthetic.make_frame(w, h, bayer=2, gain=16.0, read_sigma=12.0, seed=64)
    spec = configs.make_spec(meta, levels=4, noise_level=0.7, storage=storage)
    for shape in range(len(gls.TUNE_SHAPES[gls.TUNE_DEMOSAIC])):
        gls.tune_force(gls.TUNE_DEMOSAIC, shape)
        check(ctx, raw, spec)


def test_a_frame_records_one_choice_per_kernel(ctx, unforced):
    gls.tune_reset()
    raw, _, meta = synthetic.make_frame(640, 480, bayer=2, seed=65)
    spec = configs.make_spec(meta, levels=4)
    first = run_gpu(ctx, raw, spec, taps=False)["out"]
    entries = gls.tune_entries()
    kernels = sorted(e["kernel"] for e in entries if (e["width"], e["height"]) == (640, 480))
    assert kernels == [gls.TUNE_DEMOSAIC, gls.TUNE_FINAL], entries
    for e in entries:
        assert 0 <= e["shape"] < len(gls.TUNE_SHAPES[e["kernel"]])
        assert all(t > 0 for t in e["ms"])
        # the default shape unless another one beats it by 3 %, then the fastest
        if e["shape"] == 0:
            assert all(t >= 0.97 * e["ms"][0] for t in e["ms"])
        else:
            assert e["ms"][e["shape"]] == min(e["ms"]) and e["ms"][e["shape"]] < 0.97 * e["ms"][0]
    # the second frame of the size launches the chosen shapes and gives the same output
    again = run_gpu(ctx, raw, spec, taps=False)["out"]
    np.testing.assert_array_equal(first, again)
    assert len(gls.tune_entries()) == len(entries)


def test_force_rejects_unknown_shapes(ctx):
    for kernel, shape in ((gls.TUNE_DEMOSAIC, len(gls.TUNE_SHAPES[gls.TUNE_DEMOSAIC])), (gls.TUNE_FINAL, -2), (2, 0)):
        with pytest.raises(gls.GlsError):
            gls.tune_force(kernel, shape)
