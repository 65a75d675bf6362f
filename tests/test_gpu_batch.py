"""gls_raw_batch on the GPU: a burst of uneven frames (sizes, CFA phases, 10/12/14-bit, the
high-noise branch, storage precisions, output formats) gives, frame for frame, exactly the
output of a single converter; the batch can be reused with other sizes, captured in a CUDA
graph and replayed, and run from host buffers."""
import numpy as np
import pytest

from climage_gb300 import configs, gls, synthetic

pytestmark = pytest.mark.gpu

# (width, height, bayer, bits, gain, read sigma, noise_level, levels, storage, float output)
BURST = [
    (136, 104, 2, 12, 2.0, 3.0, 0.2, 4, gls.STORAGE_F32, False),
    (200, 152, 0, 14, 1.0, 2.0, 0.2, 5, gls.STORAGE_F32, True),
    (96, 64, 3, 10, 16.0, 12.0, 0.7, 4, gls.STORAGE_F32, False),
    (128, 96, 1, 12, 4.0, 6.0, 0.45, 4, gls.STORAGE_F32, False),
    (64, 48, 2, 12, 2.0, 3.0, 0.2, 4, gls.STORAGE_F32, True),
]


def frames(burst, seed0=0):
    import torch
    out = []
    for k, (w, h, bayer, bits, gain, sigma, nl, levels, storage, fout) in enumerate(burst):
        raw, _, meta = synthetic.make_frame(w, h, bayer=bayer, bits=bits, gain=gain, read_sigma=sigma,
                                            seed=seed0 + 17 * k + 3)
        spec = configs.make_spec(meta, levels=levels, storage=storage, noise_level=nl)
        out.append(dict(raw=torch.from_numpy(raw).cuda(), raw_np=raw, params=configs.to_gls_params(spec),
                        out_dtype=torch.float32 if fout else torch.uint8, w=w, h=h))
    return out


def empty_outs(fr):
    import torch
    return [torch.full((f["h"], f["w"], 4), 7, dtype=f["out_dtype"], device="cuda") for f in fr]


def single(ctx, fr):
    import torch
    res = []
    for f in fr:
        conv = gls.RawConverter(ctx)
        out = torch.empty((f["h"], f["w"], 4), dtype=f["out_dtype"], device="cuda")
        conv.demosaicImage(f["raw"], f["params"], out, defer_noise_model=True)
        torch.cuda.synchronize()
        conv.close()
        res.append(out)
    return res


def same(a, b):
    import torch
    if a.dtype == torch.float32:
        return torch.equal(a.view(torch.int32), b.view(torch.int32))
    return torch.equal(a, b)


@pytest.mark.parametrize("lanes", [1, 3])
def test_burst_matches_single_converter(ctx, lanes):
    import torch
    fr = frames(BURST)
    want = single(ctx, fr)
    batch = gls.RawBatch(ctx, lanes)
    outs = empty_outs(fr)
    batch.demosaic([f["raw"] for f in fr], [f["params"] for f in fr], outs)
    torch.cuda.synchronize()
    for k, (o, w) in enumerate(zip(outs, want)):
        assert same(o, w), "frame %d" % k
    # reuse: another burst, frames in another order and a half-precision frame (a lane whose
    # capacity or precision does not fit reallocates)
    burst2 = list(reversed(BURST)) + [(136, 104, 2, 12, 2.0, 3.0, 0.2, 4, gls.STORAGE_F16, False)]
    fr2 = frames(burst2, seed0=1000)
    want2 = single(ctx, fr2)
    outs2 = empty_outs(fr2)
    batch.demosaic([f["raw"] for f in fr2], [f["params"] for f in fr2], outs2)
    torch.cuda.synchronize()
    for k, (o, w) in enumerate(zip(outs2, want2)):
        assert same(o, w), "second burst, frame %d" % k
    batch.close()


def test_graph_capture_and_replay():
    import torch
    stream = torch.cuda.Stream()
    cctx = gls.Context(0, stream=stream)
    fr = frames(BURST, seed0=2000)
    want = single(cctx, fr)
    batch = gls.RawBatch(cctx, 3)
    batch.reserve(max(f["w"] for f in fr), max(f["h"] for f in fr), 5, gls.STORAGE_F32)
    outs = empty_outs(fr)
    raws, params = [f["raw"] for f in fr], [f["params"] for f in fr]
    with torch.cuda.stream(stream):
        batch.demosaic(raws, params, outs)  # eager run on the capture stream
    torch.cuda.synchronize()
    for o, w in zip(outs, want):
        assert same(o, w)
    for o in outs:
        o.fill_(3)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        batch.demosaic(raws, params, outs)
    for _ in range(2):
        for o in outs:
            o.fill_(5)
        g.replay()
        torch.cuda.synchronize()
        for k, (o, w) in enumerate(zip(outs, want)):
            assert same(o, w), "replay, frame %d" % k
    batch.close()
    cctx.close()


def test_one_lane_graph_replays_the_pyramid_launch():
    """A one-lane burst runs the pyramid statistics as one launch, whose work queue and tile
    marks live on the device and are reset by the launch itself: captured once into a CUDA
    graph, it replays correctly again and again (the burst holds frames of three sizes)."""
    import torch
    stream = torch.cuda.Stream()
    cctx = gls.Context(0, stream=stream)
    fr = frames(BURST[:3], seed0=2500)
    want = single(cctx, fr)
    batch = gls.RawBatch(cctx, 1)
    batch.reserve(max(f["w"] for f in fr), max(f["h"] for f in fr), 5, gls.STORAGE_F32)
    outs = empty_outs(fr)
    raws, params = [f["raw"] for f in fr], [f["params"] for f in fr]
    with torch.cuda.stream(stream):
        batch.demosaic(raws, params, outs)
    torch.cuda.synchronize()
    for o, w in zip(outs, want):
        assert same(o, w)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        batch.demosaic(raws, params, outs)
    for _ in range(3):
        for o in outs:
            o.fill_(7)
        g.replay()
        torch.cuda.synchronize()
        for k, (o, w) in enumerate(zip(outs, want)):
            assert same(o, w), "replay, frame %d" % k
    batch.close()
    cctx.close()


def test_host_buffers(ctx):
    import torch
    fr = frames(BURST[:4], seed0=3000)
    want = []
    for f in fr:
        conv = gls.RawConverter(ctx)
        o = np.zeros((f["h"], f["w"], 4), np.uint8)
        # this entry point writes the fitted noise model back into its parameters: give it a copy
        p = gls.DemosaicParams.from_buffer_copy(f["params"])
        conv.demosaicImageHost(np.ascontiguousarray(f["raw_np"]), p, o)
        conv.close()
        want.append(o)
    hr = [torch.from_numpy(f["raw_np"]).pin_memory() for f in fr]
    ho = [torch.zeros((f["h"], f["w"], 4), dtype=torch.uint8).pin_memory() for f in fr]
    batch = gls.RawBatch(ctx, 2)
    batch.demosaic_host_ptr([t.data_ptr() for t in hr], [(f["w"], f["h"]) for f in fr], [f["params"] for f in fr],
                            [t.data_ptr() for t in ho], 4)
    for k, (o, w) in enumerate(zip(ho, want)):
        assert np.array_equal(o.numpy(), w), "frame %d" % k
    batch.close()


def test_packed_host_frames(ctx):
    """Packed 10/12/14-bit host frames (one MSB-first bit stream, as an uncompressed DNG strip)
    give exactly the unpacked frames' output, through a converter and through a batch."""
    import torch
    fr = frames(BURST[:4], seed0=4000)
    bits = [12, 14, 10, 12]  # the bit depths of BURST[:4]
    want, packed = [], []
    for f, b in zip(fr, bits):
        conv = gls.RawConverter(ctx)
        o = np.zeros((f["h"], f["w"], 4), np.uint8)
        conv.demosaicImageHost(np.ascontiguousarray(f["raw_np"]), gls.DemosaicParams.from_buffer_copy(f["params"]), o)
        want.append(o)
        pk = np.frombuffer(synthetic.pack_bits(f["raw_np"], b), np.uint8).copy()
        packed.append(pk)
        o2 = np.zeros_like(o)
        conv.demosaicImagePackedHost(pk, b, f["w"], f["h"], gls.DemosaicParams.from_buffer_copy(f["params"]), o2)
        assert np.array_equal(o2, o)
        conv.close()
    pinned = [torch.from_numpy(pk).pin_memory() for pk in packed]
    ho = [torch.zeros((f["h"], f["w"], 4), dtype=torch.uint8).pin_memory() for f in fr]
    batch = gls.RawBatch(ctx, 2)
    batch.demosaic_packed_host_ptr([t.data_ptr() for t in pinned], [pk.size for pk in packed], bits,
                                   [(f["w"], f["h"]) for f in fr], [f["params"] for f in fr],
                                   [t.data_ptr() for t in ho], 4)
    for k, (o, w) in enumerate(zip(ho, want)):
        assert np.array_equal(o.numpy(), w), "frame %d" % k
    batch.close()
    conv = gls.RawConverter(ctx)
    with pytest.raises(gls.GlsError):  # too few bytes for the frame
        conv.demosaicImagePackedHost(packed[0][:-2], 12, fr[0]["w"], fr[0]["h"], fr[0]["params"],
                                     np.zeros((fr[0]["h"], fr[0]["w"], 4), np.uint8))
    conv.close()


def test_rejects_bad_frame(ctx):
    import torch
    fr = frames(BURST[:2])
    p = [f["params"] for f in fr]
    p[1].pyramid_levels = 2
    batch = gls.RawBatch(ctx, 2)
    with pytest.raises(gls.GlsError):
        batch.demosaic([f["raw"] for f in fr], p, empty_outs(fr))
    with pytest.raises(gls.GlsError):
        gls.RawBatch(ctx, 0)
    torch.cuda.synchronize()
    batch.close()
