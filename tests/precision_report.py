"""Per-stage error of the GPU pipeline against the FP64 run of the pipeline.

The FP64 run is the oracle's (oracle/: every stage restated in double precision, no fp16
rounding) on the same frame.  For each intermediate image the converter can tap (scaled
raw, green, level 0 after the despeckle, denoised level 0, LTM mask) and for the float
output, the report gives the largest absolute difference and the PSNR over the reference
image's value range.  With fp16 storage (the precision form: 8064x6048 GRBG 14-bit, six
levels) this measures what binary16 intermediates cost.

    python -m tests.precision_report [--width 8064 --height 6048 --bayer 0 --bits 14
                                      --levels 6 --storage f16]

Test infrastructure (it runs the oracle); tests/test_gpu_precision.py runs it on small frames.
"""
import argparse
import json

import numpy as np

from climage_gb300 import configs, gls, synthetic

TAPS = {0: "scaled_raw", 1: "green", 2: "level0", 3: "denoised0", 4: "ltm_mask"}


def _stats(got, ref):
    """Errors over the pixels finite in both; NaN positions must agree (the LTM mask is NaN
    where the camera-space luma is negative, in every precision)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    both = np.isfinite(got) & np.isfinite(ref)
    err = np.abs(got[both] - ref[both])
    peak = float(ref[both].max() - ref[both].min()) or 1.0
    mse = float(np.mean(err ** 2))
    return {"max_abs": float(err.max()), "psnr_db": round(10 * np.log10(peak * peak / mse), 2) if mse > 0 else None,
            "peak": round(peak, 6), "nonfinite_mismatch": int(np.sum(np.isfinite(got) != np.isfinite(ref)))}


def stage_errors(ctx, raw, spec):
    """GPU run (taps + float output) and the oracle's FP64 run of one frame; per-stage stats."""
    import torch

    from oracle import oracle as orc
    from tests.helpers import oracle_params
    h, w = raw.shape
    conv = gls.RawConverter(ctx)
    bufs = {}
    for k, name in TAPS.items():
        shape = (h, w) if name in ("scaled_raw", "green", "ltm_mask") else (h, w, 4)
        bufs[name] = torch.zeros(shape, dtype=torch.float32, device="cuda")
        conv.setTap(k, bufs[name])
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    conv.demosaicImage(torch.from_numpy(raw).cuda(), configs.to_gls_params(spec), out, defer_noise_model=True)
    torch.cuda.synchronize()
    conv.close()
    ref = orc.demosaic(raw, oracle_params(spec), orc.F64, want=("rgbaf",), taps=tuple(TAPS.values()))
    report = {}
    for name in TAPS.values():
        g = bufs[name].cpu().numpy()
        r = ref[name]
        if g.ndim == 3:
            g, r = g[..., :3], r[..., :3]
        report[name] = _stats(g, r)
    report["output_rgb"] = _stats(out.cpu().numpy()[..., :3], ref["rgbaf"][..., :3])
    return report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=8064)
    ap.add_argument("--height", type=int, default=6048)
    ap.add_argument("--bayer", type=int, default=0)
    ap.add_argument("--bits", type=int, default=14)
    ap.add_argument("--levels", type=int, default=6)
    ap.add_argument("--storage", choices=["f16", "f32"], default="f16")
    ap.add_argument("--seed", type=int, default=3)
    args = ap.parse_args()
    raw, _, meta = synthetic.make_frame(args.width, args.height, bayer=args.bayer, bits=args.bits, seed=args.seed)
    storage = gls.STORAGE_F16 if args.storage == "f16" else gls.STORAGE_F32
    spec = configs.make_spec(meta, levels=args.levels, storage=storage)
    ctx = gls.Context(0)
    rep = stage_errors(ctx, raw, spec)
    print(json.dumps({"frame": "%dx%d bayer %d %d-bit" % (args.width, args.height, args.bayer, args.bits),
                      "levels": args.levels, "storage": args.storage, "stages": rep}))
    ctx.close()


if __name__ == "__main__":
    main()
