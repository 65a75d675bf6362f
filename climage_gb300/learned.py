"""The learned stage's data, training and judging (the network itself is gls_cnn; its kernels
are in csrc/k_cnn.cu).

Training pairs are rendered by the plain pipeline from seeded synthetic scenes: the input is
the pipeline's own image after interpolateRedBlue plus the noise sigma map
(gls_raw_converter_cnn_input) of a noisy raw frame, the target the same image of the same
scene mosaicked without noise -- so the network learns to remove noise as the pipeline
renders the scene (clipping, demosaic) rather than to re-render it.  Crops of 256 x 256 from
1024 x 768 frames at read noise 4..16 DN and gain 0.25..4 e-/DN (at the bench's lower noise
levels the texture of the scenes dominates the error and a network this small learns
nothing over the identity).

The judge is the plain pipeline: on held-out frames, the learned and the plain pipeline's
float RGB outputs are compared with the plain pipeline's output of the noise-free frame
(PSNR and CIE76 Delta E); the learned stage is only worth running when it wins.

    python -m climage_gb300.learned --crops 20000 --epochs 12 --lr 3e-4 --out climage_gb300/cnn_params.npy
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


# noise of the training and judging frames: read sigma (DN) and gain (e-/DN) ranges (the
# shipped parameters were trained on these: 12 epochs over 20000 crops, Adam at 3e-4)
NOISE = {"sigma": (4.0, 16.0), "gain": (0.25, 4.0)}


def noise_for(seed, noise=None):
    noise = noise or NOISE
    rng = np.random.default_rng(seed ^ 0x5EED)
    sigma = float(rng.uniform(*noise["sigma"]))
    gain = float(np.exp(rng.uniform(np.log(noise["gain"][0]), np.log(noise["gain"][1]))))
    return sigma, gain


CLEAN = dict(gain=1e6, read_sigma=0.0)  # noise-free mosaic of the same scene


def pair(width, height, seed, bayer=2, noise=None):
    """(noisy raw, clean raw, noisy meta, clean meta) of one seeded scene."""
    sigma, gain = noise_for(seed, noise)
    scene = synthetic.make_scene(width, height, seed)
    m = dict(bayer=bayer, black=64, white=4095, wb=(2.0, 1.0, 1.6), bits=12)
    noisy = synthetic.mosaic(scene, bayer, m["black"], m["white"], m["wb"], gain, sigma, seed)
    clean = synthetic.mosaic(scene, bayer, m["black"], m["white"], m["wb"], CLEAN["gain"], CLEAN["read_sigma"], seed)
    return noisy, clean, dict(m, gain=gain, read_sigma=sigma), dict(m, **CLEAN)


def _render(job):
    seed, noise = job
    return (seed,) + pair(FRAME[0], FRAME[1], seed, noise=noise)


def frames(seeds, workers=None):
    """Synthetic frames rendered in a process pool (spawned: safe next to a CUDA context; a
    calling script must guard its entry point with `if __name__ == "__main__":`).  The noise
    ranges travel with each job (a spawned worker has its own copy of the module)."""
    workers = workers or min(16, os.cpu_count() or 1)
    jobs = [(s, dict(NOISE)) for s in seeds]
    if workers <= 1:
        for j in jobs:
            yield _render(j)
        return
    with mp.get_context("spawn").Pool(workers) as pool:
        for item in pool.imap(_render, jobs, chunksize=4):
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
    cbuf = torch.empty((FRAME[1], FRAME[0], 4), dtype=torch.float32, device="cuda")
    k = 0
    for seed, noisy, clean, meta, cmeta in frames(range(seed0, seed0 + n_frames), workers):
        conv.cnnInput(torch.from_numpy(noisy).cuda(), configs.to_gls_params(configs.make_spec(meta, levels=5)), buf)
        conv.cnnInput(torch.from_numpy(clean).cuda(), configs.to_gls_params(configs.make_spec(cmeta, levels=5)), cbuf)
        for y in range(0, FRAME[1] - CROP + 1, CROP):
            for x in range(0, FRAME[0] - CROP + 1, CROP):
                inp[k] = buf[y:y + CROP, x:x + CROP].half()
                gt[k] = cbuf[y:y + CROP, x:x + CROP, :3].half()
                k += 1
    torch.cuda.synchronize()
    conv.close()
    return inp[:n_crops], gt[:n_crops]


def train(cnn, inp, gt, epochs=6, batch=32, lr=1e-3, seed=0, log=None):
    """Adam over shuffled crops: the learning rate held for the first 60 % of the epochs
    (the zero-initialised head needs a few hundred steps before the loss moves), then halved
    every epoch; returns the mean losses per epoch."""
    import torch
    n = inp.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    hist = []
    for ep in range(epochs):
        order = torch.randperm(n, generator=g)
        hold = max(1, int(round(0.6 * epochs)))
        rate = lr * (0.5 ** max(0, ep + 1 - hold))
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


def residual_only(params):
    """The same network with its strength head zeroed: logit 0, noise-model multiplier 1."""
    p = np.array(params, np.float32, copy=True)
    o = sum(cout * 9 * cin + cout for cin, cout in gls.CNN_LAYERS[:-1])
    cin, cout = gls.CNN_LAYERS[-1]
    w = p[o:o + cout * 9 * cin].reshape(cout, 3, 3, cin)
    w[0] = 0.0
    p[o + cout * 9 * cin] = 0.0
    return p


def judge(ctx, cnn, seeds, width=1024, height=768):
    """Learned against plain on held-out scenes.  Pipeline: PSNR (dB) and mean CIE76 Delta E
    of the float RGB output against the plain pipeline's output of the noise-free frame, for
    the plain pipeline, the learned one and the learned one with the strength head zeroed.
    Linear: PSNR of the network's input and of input + residual against the noise-free
    frame's image after interpolateRedBlue."""
    import torch
    alt = gls.Cnn(ctx)
    alt.set_params(residual_only(cnn.params()))
    convs = {"plain": gls.RawConverter(ctx), "learned": gls.RawConverter(ctx), "residual_only": gls.RawConverter(ctx)}
    convs["learned"].setCnn(cnn)
    convs["residual_only"].setCnn(alt)
    out = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    lin = torch.empty((1, height, width, 4), dtype=torch.float32, device="cuda")
    clin = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
    head = torch.empty((1, height, width, 4), dtype=torch.float32, device="cuda")
    res = {k: [] for k in convs}
    res["linear_input"], res["linear_corrected"] = [], []
    c = (slice(8, -8), slice(8, -8))
    for seed in seeds:
        noisy, clean, meta, cmeta = pair(width, height, seed)
        spec = configs.to_gls_params(configs.make_spec(meta, levels=5))
        cspec = configs.to_gls_params(configs.make_spec(cmeta, levels=5))
        convs["plain"].demosaicImage(torch.from_numpy(clean).cuda(), cspec, out, defer_noise_model=True)
        convs["plain"].cnnInput(torch.from_numpy(clean).cuda(), cspec, clin)
        torch.cuda.synchronize()
        ref = out.cpu().numpy()[c][..., :3].copy()
        cref = clin.cpu().numpy()[c][..., :3].copy()
        for name, conv in convs.items():
            conv.demosaicImage(torch.from_numpy(noisy).cuda(), spec, out, defer_noise_model=True)
            torch.cuda.synchronize()
            got = out.cpu().numpy()[c][..., :3]
            mse = float(np.mean((np.clip(got, 0, 1) - np.clip(ref, 0, 1)) ** 2))
            de = float(np.mean(np.linalg.norm(_lab(got) - _lab(ref), axis=-1)))
            res[name].append((10 * np.log10(1.0 / mse), de))
        convs["plain"].cnnInput(torch.from_numpy(noisy).cuda(), spec, lin[0])
        cnn.forward(lin, head)
        torch.cuda.synchronize()
        xs = lin[0].cpu().numpy()[c]
        x = xs[..., :3]
        r = xs[..., 3:4] * head[0].cpu().numpy()[c][..., 1:4]  # residual = sigma * output
        for name, v in (("linear_input", x), ("linear_corrected", x + r)):
            res[name].append((10 * np.log10(1.0 / float(np.mean((v - cref) ** 2))), 0.0))
    for conv in convs.values():
        conv.close()
    alt.close()
    summary = {k: {"psnr_db": round(float(np.mean([r[0] for r in v])), 3),
                   "delta_e": round(float(np.mean([r[1] for r in v])), 3)} for k, v in res.items()}
    summary["linear_input"].pop("delta_e")
    summary["linear_corrected"].pop("delta_e")
    return summary


def load_params(path=PARAMS_PATH):
    return np.load(path).astype(np.float32) if os.path.exists(path) else None


def time_forward(w, h, warmup=3, reps=5, backend=None):
    """CUDA-event time of one forward pass of the shipped network over a w x h frame
    (hidden layers on `backend`: 0 warp-level MMA, 1 tcgen05; None keeps the default)."""
    import torch
    ctx = gls.Context(0)
    cnn = gls.Cnn(ctx)
    cnn.set_params(load_params())
    if backend is not None:
        cnn.set_backend(backend)
    x = torch.rand((1, h, w, 4), device="cuda")
    out = torch.empty_like(x)
    for _ in range(warmup):
        cnn.forward(x, out)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        cnn.forward(x, out)
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / reps
    flop = 2 * 9 * sum(cin * cout for cin, cout in gls.CNN_LAYERS) * w * h
    cnn.status()
    print(json.dumps({"backend": backend, "forward_ms": round(ms, 4), "pixels": w * h, "tflops": round(flop / ms / 1e9, 1)}))
    cnn.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--crops", type=int, default=20000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--out", default=PARAMS_PATH)
    ap.add_argument("--judge-frames", type=int, default=6)
    ap.add_argument("--judge-only", default=None, help="judge these saved parameters, no training")
    ap.add_argument("--gain", type=float, nargs=2, default=None, help="gain range (e-/DN) of the frames")
    ap.add_argument("--sigma", type=float, nargs=2, default=None, help="read noise range (DN) of the frames")
    ap.add_argument("--backend", type=int, default=None, choices=(0, 1, 2),
                    help="forward backend for --time-forward (0 mma.sync, 1 tcgen05 layers, 2 fused tcgen05)")
    ap.add_argument("--time-forward", type=int, nargs=2, default=None, metavar=("W", "H"),
                    help="only time the network's forward pass over a W x H frame (shipped parameters)")
    args = ap.parse_args()
    if args.time_forward:
        time_forward(*args.time_forward, backend=args.backend)
        return
    if args.gain:
        NOISE["gain"] = tuple(args.gain)
    if args.sigma:
        NOISE["sigma"] = tuple(args.sigma)
    import torch
    ctx = gls.Context(0)
    if args.judge_only:
        cnn = gls.Cnn(ctx)
        cnn.set_params(np.load(args.judge_only))
        print(json.dumps({"judge": judge(ctx, cnn, range(10**6, 10**6 + args.judge_frames))}))
        return
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
