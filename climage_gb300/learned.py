"""The learned stage's data, training and judging (the network itself is gls_cnn; its kernels
are in csrc/k_cnn.cu).

Training pairs are rendered by the plain pipeline from seeded synthetic scenes: the input is
the pipeline's own image after interpolateRedBlue plus the noise sigma map
(gls_raw_converter_cnn_input), the target is the clean linear scene, which the white balance
and black/white scaling map onto the same scale.  Crops of 256 x 256 from 1024 x 768 frames
at noise levels spread over the bench's range (read sigma 2..12 DN, gain 1..16 e-/DN).

The judge is the plain pipeline: on held-out frames, the learned and the plain pipeline's
float RGB outputs are compared with the plain pipeline's output of the same scene without
noise (PSNR and CIE76 Delta E); the learned stage is only worth running when it wins.

    python -m climage_gb300.learned --crops 20000 --epochs 3 --out climage_gb300/cnn_params.npy
"""
import argparse
import json
import multiprocessing as mp
import os
import time

import numpy as np

from climage_gb300 import configs, gls, synthetic

HERE = os.path.dirname(os.path.abspath(__file__))
PARAMS_PATH = os.path.join(HERE, "cnn_params.npy")
FRAME = (1024, 768)
CROP = 256


def noise_for(seed):
    rng = np.random.default_rng(seed ^ 0x5EED)
    sigma = float(rng.uniform(2.0, 12.0))
    gain = float(np.exp(rng.uniform(np.log(1.0), np.log(16.0))))
    return sigma, gain


def _render(seed):
    sigma, gain = noise_for(seed)
    raw, scene, meta = synthetic.make_frame(FRAME[0], FRAME[1], bayer=2, gain=gain, read_sigma=sigma, seed=seed)
    return seed, raw, scene, meta


def frames(seeds, workers=None):
    """Synthetic frames rendered in a process pool (spawned: safe next to a CUDA context)."""
    workers = workers or min(16, os.cpu_count() or 1)
    if workers <= 1:
        for s in seeds:
            yield _render(s)
        return
    with mp.get_context("spawn").Pool(workers) as pool:
        for item in pool.imap(_render, seeds, chunksize=4):
            yield item


def render_crops(ctx, n_crops, seed0=0, workers=None):
    """(inputs (n, 256, 256, 4), targets (n, 256, 256, 3)) as float16 CUDA tensors."""
    import torch
    per = (FRAME[0] // CROP) * (FRAME[1] // CROP)
    n_frames = (n_crops + per - 1) // per
    conv = gls.RawConverter(ctx)
    inp = torch.empty((n_frames * per, CROP, CROP, 4), dtype=torch.float16, device="cuda")
    gt = torch.empty((n_frames * per, CROP, CROP, 3), dtype=torch.float16, device="cuda")
    buf = torch.empty((FRAME[1], FRAME[0], 4), dtype=torch.float32, device="cuda")
    k = 0
    for seed, raw, scene, meta in frames(range(seed0, seed0 + n_frames), workers):
        params = configs.to_gls_params(configs.make_spec(meta, levels=5))
        conv.cnnInput(torch.from_numpy(raw).cuda(), params, buf)
        sc = torch.from_numpy(scene).cuda()
        for y in range(0, FRAME[1] - CROP + 1, CROP):
            for x in range(0, FRAME[0] - CROP + 1, CROP):
                inp[k] = buf[y:y + CROP, x:x + CROP].half()
                gt[k] = sc[y:y + CROP, x:x + CROP].half()
                k += 1
    torch.cuda.synchronize()
    conv.close()
    return inp[:n_crops], gt[:n_crops]


def train(cnn, inp, gt, epochs=3, batch=16, lr=2e-3, seed=0, log=None):
    """Adam over shuffled crops, the learning rate halved in each later epoch; returns the
    mean losses per epoch."""
    import torch
    n = inp.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for ep in range(epochs):
        order = torch.randperm(n, generator=g)
        rate = lr * (0.5 ** ep)
        tot = np.zeros(2)
        steps = 0
        for i in range(0, n - batch + 1, batch):
            idx = order[i:i + batch].cuda()
            x = inp.index_select(0, idx).float().contiguous()
            y = gt.index_select(0, idx).float().contiguous()
            tot += cnn.train_step(x, y, rate)
            steps += 1
        hist.append((tot / max(steps, 1)).tolist())
        if log:
            log("epoch %d: residual mse %.3e, strength loss %.3e" % (ep, hist[-1][0], hist[-1][1]))
    return hist


def _lab(rgb):
    """sRGB-encoded RGB in [0, 1] -> CIE L*a*b* (D65)."""
    c = np.clip(rgb, 0.0, 1.0).astype(np.float64)
    lin = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)
    m = np.array([[0.4124, 0.3576, 0.1805], [0.2126, 0.7152, 0.0722], [0.0193, 0.1192, 0.9505]])
    xyz = lin @ m.T / np.array([0.95047, 1.0, 1.08883])
    f = np.where(xyz > (6 / 29) ** 3, np.cbrt(xyz), xyz / (3 * (6 / 29) ** 2) + 4 / 29)
    return np.stack([116 * f[..., 1] - 16, 500 * (f[..., 0] - f[..., 1]), 200 * (f[..., 1] - f[..., 2])], -1)


def judge(ctx, cnn, seeds, width=1024, height=768):
    """Learned against plain on held-out scenes: PSNR (dB) and mean CIE76 Delta E of the float
    RGB output against the plain pipeline's output of the noise-free scene."""
    import torch
    plain, learned = gls.RawConverter(ctx), gls.RawConverter(ctx)
    learned.setCnn(cnn)
    out = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    res = {"plain": [], "learned": []}
    for seed in seeds:
        sigma, gain = noise_for(seed)
        raw, _, meta = synthetic.make_frame(width, height, bayer=2, gain=gain, read_sigma=sigma, seed=seed)
        clean, _, cmeta = synthetic.make_frame(width, height, bayer=2, gain=1e6, read_sigma=0.0, seed=seed)
        spec = configs.make_spec(meta, levels=5)
        plain.demosaicImage(torch.from_numpy(clean).cuda(), configs.to_gls_params(configs.make_spec(cmeta, levels=5)),
                            out, defer_noise_model=True)
        torch.cuda.synchronize()
        ref = out.cpu().numpy()[8:-8, 8:-8, :3].copy()
        for name, conv in (("plain", plain), ("learned", learned)):
            conv.demosaicImage(torch.from_numpy(raw).cuda(), configs.to_gls_params(spec), out, defer_noise_model=True)
            torch.cuda.synchronize()
            got = out.cpu().numpy()[8:-8, 8:-8, :3]
            mse = float(np.mean((np.clip(got, 0, 1) - np.clip(ref, 0, 1)) ** 2))
            de = float(np.mean(np.linalg.norm(_lab(got) - _lab(ref), axis=-1)))
            res[name].append((10 * np.log10(1.0 / mse), de, sigma, gain))
    plain.close()
    learned.close()
    summary = {k: {"psnr_db": round(float(np.mean([r[0] for r in v])), 3),
                   "delta_e": round(float(np.mean([r[1] for r in v])), 3)} for k, v in res.items()}
    summary["frames"] = [{"read_sigma": round(p[2], 2), "gain": round(p[3], 2), "plain_db": round(p[0], 2),
                          "learned_db": round(l[0], 2)} for p, l in zip(res["plain"], res["learned"])]
    return summary


def load_params(path=PARAMS_PATH):
    return np.load(path).astype(np.float32) if os.path.exists(path) else None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--crops", type=int, default=20000)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=PARAMS_PATH)
    ap.add_argument("--judge-frames", type=int, default=6)
    args = ap.parse_args()
    import torch
    ctx = gls.Context(0)
    t0 = time.time()
    inp, gt = render_crops(ctx, args.crops, seed0=0)
    t1 = time.time()
    cnn = gls.Cnn(ctx)
    cnn.set_params(gls.cnn_init(0))
    hist = train(cnn, inp, gt, args.epochs, args.batch, args.lr, log=print)
    torch.cuda.synchronize()
    t2 = time.time()
    np.save(args.out, cnn.params())
    verdict = judge(ctx, cnn, range(10**6, 10**6 + args.judge_frames))
    print(json.dumps({"crops": int(inp.shape[0]), "render_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1),
                      "epochs": hist, "judge": verdict}))
    cnn.close()
    ctx.close()


if __name__ == "__main__":
    main()
