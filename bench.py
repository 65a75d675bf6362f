"""Benchmark: RAW->RGB MPix/s on one GB300, with the CPU oracle beside it.

Workload (default): the phone-resolution plain pipeline -- three 4032x3024 RGGB 12-bit
synthetic frames at read-noise/gain {2/1, 6/4, 12/16} (the last one takes the high-noise
raw branch), 5-level pyramid, fp32 intermediates, local tone mapping on, RGBA8 output.
One step = those three frames as one burst (gls_raw_batch: demosaicImage per frame, each
frame on its own stream).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value: MPix/s with the raw frames already in HBM, CUDA-event timed per step with an L2
flush (a 256 MB write) between steps, max over ranks.  e2e: the same frames through the
host-buffer burst entry point (pinned uint16 in, RGB8 out, copies inside the timed region).
--impl reference times the CPU restatement of the reference pipeline (the oracle; the
reference's OpenCL kernels cannot run on this machine) with every host thread, three frames
per step as above; that arm imports no module of the product package and maps none of its
libraries (the workload tables and the scene generator, plain numpy, are loaded from their
files; the camera matrices come from the oracle's host math).
--gpus N without a launcher's environment (WORLD_SIZE unset) starts N replicas itself under
torch.distributed.run on 127.0.0.1.
"""
import argparse
import importlib.util
import json
import os
import socket
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RAW→RGB MPix/s on 1 GB300 (plain vs batched/learned) at PSNR vs FP64 oracle"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gls", choices=["gls", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-psnr", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-awb", action="store_true")
    ap.add_argument("--no-dng", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the config-1 and precision-form lines")
    ap.add_argument("--profile-only", action="store_true", help="a short run for ncu: no clocks, no cpu leg")
    ap.add_argument("--shapes", default="",
                    help="force launch shapes instead of timing them, e.g. 'demosaic=split,final=32x24' "
                         "(under ncu the tuner would time serialised cold launches)")
    ap.add_argument("--cpu-replicas", action="store_true",
                    help="check the replica plumbing on the CPU (gloo): each rank runs the oracle on a tiny "
                         "workload of its own frames; prints one check line, not a bench line")
    return ap.parse_args(argv)


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def launch_replicas(args, argv):
    """--gpus N > 1 outside a launcher: start N processes of this script under
    torch.distributed.run (one per GPU, rendezvous on 127.0.0.1) and return their exit code;
    None when this process is already a rank (WORLD_SIZE set) or N == 1."""
    if args.gpus <= 1 or "WORLD_SIZE" in os.environ:
        return None
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=%d" % args.gpus,
           "--master-addr=127.0.0.1", "--master-port=%d" % free_port(), os.path.abspath(__file__)] + list(argv)
    return subprocess.call(cmd, cwd=ROOT)


def load_file(name, rel):
    """A module loaded from its file alone (no package import, so nothing else of the package
    and none of its native libraries comes with it)."""
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, rel))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload_modules(reference=False):
    """(configs, synthetic, cam_xyz_coeff): the workload tables, the scene generator and the
    camera-matrix conversion.  The reference arm takes the tables and the generator from their
    files and the conversion from the oracle; the GPU arm from the product package."""
    if reference:
        from oracle import oracle as orc
        return (load_file("gls_workload_configs", "climage_gb300/configs.py"),
                load_file("gls_workload_synthetic", "climage_gb300/synthetic.py"), orc.cam_xyz_coeff)
    from climage_gb300 import configs, synthetic
    return configs, synthetic, None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_replicas(backend):
    """One process per GPU, each an independent replica of the whole step (the pipeline has
    no exchange step, so frames are never split across ranks): the process group carries only
    the barriers around the timed region and the max-over-ranks reduction of its duration."""
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend, init_method="env://", rank=rank, world_size=world)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(total_ms, world, dev):
    """The slowest replica's timed-region duration (every rank returns the same number)."""
    if world == 1:
        return float(total_ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, mpix_per_step, steps, total_ms):
    """Whole-job throughput: every rank processed steps x mpix_per_step in at most total_ms."""
    return world * mpix_per_step * steps / (total_ms / 1e3)


def make_frames(cfg, rank, reference=False):
    configs, synthetic, cam_xyz_coeff = workload_modules(reference)
    frames = []
    for i, (sigma, gain, nl) in enumerate(cfg["noise"]):
        raw, scene, meta = synthetic.make_frame(cfg["width"], cfg["height"], bayer=cfg["bayer"], bits=cfg["bits"],
                                                black=cfg["black"], white=cfg["white"], wb=cfg["wb"], gain=gain,
                                                read_sigma=sigma, seed=1000 * rank + i)
        spec = configs.make_spec(meta, levels=cfg["levels"], storage=cfg["storage"], noise_level=nl,
                                 cam_xyz_coeff=cam_xyz_coeff)
        frames.append((raw, scene, spec))
    return frames


def tuner_summary():
    """The launch-shape tuner's choices made in this process: per kernel and frame size, the
    chosen tile shape and the best time of every shape (ms, timed on the frame on first use)."""
    from climage_gb300 import gls
    names = {gls.TUNE_DEMOSAIC: "demosaic", gls.TUNE_FINAL: "final"}
    out = []
    for e in gls.tune_entries():
        shapes = gls.TUNE_SHAPES[e["kernel"]]
        out.append({"kernel": names[e["kernel"]], "size": "%dx%d" % (e["width"], e["height"]), "flags": e["flags"],
                    "shape": shapes[e["shape"]], "ms": dict(zip(shapes, e["ms"]))})
    return out


def workload_config(cfg, world):
    """The line's config: the same dict on both arms (GPU and reference)."""
    return {"workload": cfg["name"], "frames_per_step": len(cfg["noise"]), "width": cfg["width"],
            "height": cfg["height"], "levels": cfg["levels"], "storage": "fp16" if cfg["storage"] else "fp32",
            "output": "rgba8", "local_tone_mapping": True, "noise": [list(n) for n in cfg["noise"]],
            "l2": "GPU arm: flushed between steps (256 MB write); CPU arm: 3 x 24 MB raw in, well above its caches",
            "parallelism": "replicas" if world > 1 else "single"}


def make_burst(bases, dev, n=64, seed=4):
    """The batched form's burst: n frames of sizes drawn uniformly from 1920x1080, 2016x1512,
    4032x3024 and 8064x6048, CFA phase from the four, 10/12/14-bit, white-balance gains in
    [1, 3].  Assembled on the device from the 4032x3024 RGGB 12-bit frames already rendered
    (crops, 2x2 tilings, one-pixel shifts for the CFA phase, bit shifts for the depth), so
    that building it costs no scene rendering.  Returns [(raw uint16 device tensor, spec)]."""
    import torch
    from climage_gb300 import configs
    rng = np.random.default_rng(seed)
    sizes = [(1920, 1080), (2016, 1512), (4032, 3024), (8064, 6048)]
    phase = {(0, 0): 2, (1, 0): 0, (0, 1): 1, (1, 1): 3}  # shift of an RGGB mosaic -> CFA
    base = [torch.from_numpy(b.astype(np.int32)).to(dev) for b in bases]
    out = []
    for _ in range(n):
        w, h = sizes[rng.integers(4)]
        dx, dy = int(rng.integers(2)), int(rng.integers(2))
        bits = int(rng.choice([10, 12, 14]))
        picks = [int(rng.integers(len(bases))) for _ in range(4)]
        sh = [torch.roll(base[i], (-dy, -dx), dims=(0, 1)) for i in picks[:4 if w == 8064 else 1]]
        if (w, h) == (8064, 6048):
            raw = torch.cat([torch.cat([sh[0], sh[1]], 1), torch.cat([sh[2], sh[3]], 1)], 0)
        else:
            raw = sh[0][:h, :w]
        if bits == 10:
            raw, black, white = raw >> 2, 16, 1023
        elif bits == 14:
            raw, black, white = raw << 2, 256, 16383
        else:
            black, white = 64, 4095
        wb = (float(rng.uniform(1, 3)), 1.0, float(rng.uniform(1, 3)))
        meta = dict(bayer=phase[(dx, dy)], black=black, white=white, wb=wb)
        out.append((raw.contiguous().to(torch.uint16), configs.make_spec(meta, levels=4, noise_level=0.2)))
    return out


def algorithmic_bytes_per_px(S, O, L):
    """Compulsory bytes per pixel of the reference dataflow, every global sync point
    materialised once: raw noise fit 3 passes x 2 B; demosaic 2 B in + level 0 S out;
    level-0 fit 3 passes x S; final pass level 0 S in + output O; each coarser level 7 S-byte
    accesses per pixel of its own (write, 3 fit passes, denoise read and write, parent read),
    G = sum of 4^-l over the coarser levels.  Total 8 + 5S + O + 7S*G."""
    G = sum(4.0 ** -l for l in range(1, L))
    return 8 + 5 * S + O + 7 * S * G


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) and issue-slot use
# of the two largest stages, from one ncu capture of this workload (4032x3024, fp32
# storage, RGBA8 out; the demosaic in its split shape, the green kernel and the red/blue +
# despeckle kernel together, issue use weighted by time); the roofline fraction is computed
# live, these explain it.
NCU_TRAFFIC = {"denoise L0+LTM+sRGB": (235657984, 76.4), "demosaic": (151781632, 80.1)}


# Compulsory bytes per full-resolution pixel of each full-resolution kernel (what it must
# read and write at least once; fp32 storage: s1 = 4 B single channel, s4 = 16 B RGBA).
# Fused kernels: level 0 is stored in binary16 (8 B/px) because the despeckle that
# produces it already rounds every value to binary16.
def stage_bytes(name, s1, s4):
    table = {
        # fused schedule
        "rawNoiseStatistics+fit": 2,                      # uint16 raw in
        "demosaic": 2 + 8,                                # raw in, level 0 out
        "noiseStatistics+downsample L0": 8 + s4 / 4,      # level 0 in, level 1 out
        "denoise L0+LTM+sRGB": 8 + 2 * s4 / 4 + s4 / 64 + 4,  # level 0, level 1 (both), level 3 guide, RGBA8 out
        # single-stage schedule
        "scaleRawData": 2 + s1, "interpolateGreen": 2 * s1, "interpolateRedBlue": 2 * s1 + s4,
        "blendHighlights": 2 * s4, "transformImage": 2 * s4, "despeckleImage": 2 * s4,
        "denoise L0": 2 * s4, "reassemble L0": 2 * s4, "localToneMappingMask": s4 + s1,
        "convertTosRGB": s4 + s1 + 4, "noiseStatistics+fit L0": s4,
    }
    return table.get(name)


class ClockSampler:
    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is running: samples from here on are
            # the region's (the first, taken before, is kept only when the region ends first)
            t0 = time.time()
            while not self.samples and time.time() - t0 < 5.0:
                time.sleep(0.005)
        except Exception:
            self.proc = None
        self.first = len(self.samples)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        during = self.samples[self.first:]
        where = "during the timed region (20 ms interval)"
        if not during:
            during, where = self.samples[-1:], "just before the timed region (it was shorter than one interval)"
        self.samples = during
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples), "sampled": where}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_leg(frames, max_seconds=30.0, gpu_rgb=None):
    """The oracle on the host cores over a bounded sample: the first frame, full size.  With
    gpu_rgb (the GPU's float RGB output of that frame) it also runs the oracle's FP64
    pipeline once, untimed, as the error checker: PSNR and error tail of the GPU output."""
    from oracle import oracle as orc
    from tests.helpers import oracle_params
    raw, _, spec = frames[0]
    psnr = None
    if gpu_rgb is not None:
        ref = orc.demosaic(raw, oracle_params(spec), orc.F64, want=("rgbaf",))["rgbaf"][..., :3].astype(np.float64)
        err = np.abs(gpu_rgb.astype(np.float64) - ref)
        mse = float(np.mean(err ** 2))
        psnr = {"db": round(10 * np.log10(1.0 / mse), 2) if mse > 0 else None, "max_abs": round(float(err.max()), 6),
                "p99_99_abs": round(float(np.quantile(err, 0.9999)), 6),
                "frac_over_half_lsb": float(np.mean(err > 0.5 / 255)),
                "frame": "%dx%d, read sigma 2 DN, gain 1" % (raw.shape[1], raw.shape[0]),
                "output": "RGB float (before UNORM8)"}
    threads = orc.threads()
    t0 = time.perf_counter()
    n = 0
    while True:
        orc.demosaic(raw, oracle_params(spec), orc.F32, want=("rgba8",))
        n += 1
        if time.perf_counter() - t0 > max_seconds * 0.3 or n >= 3:
            break
    dt = (time.perf_counter() - t0) / n
    mpix = raw.size / 1e6
    return {"value": round(mpix / dt, 3), "unit": "MPix/s", "cores": threads, "kind": "port",
            "sample": "%d frame(s) of %dx%d (read sigma %.0f DN, gain %.0f), oracle fp32, %d threads, %.2f s/frame"
                      % (n, raw.shape[1], raw.shape[0], 2.0, 1.0, threads, dt)}, psnr


def run_reference(args, cfg=None):
    """The reference arm: the oracle (the CPU restatement of the reference's pipeline) on the
    host cores, every thread, on the GPU arm's workload -- each step converts the same three
    frames (RGBA8 out).  Rank 0 alone runs and prints; other ranks return at once."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc
    from tests.helpers import oracle_params
    if cfg is None:
        cfg = load_file("gls_workload_configs", "climage_gb300/configs.py").CONFIG2
    frames = make_frames(cfg, 0, reference=True)
    params = [oracle_params(f[2]) for f in frames]
    threads = orc.threads()
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for (raw, _, _), p in zip(frames, params):
            orc.demosaic(raw, p, orc.F32, want=("rgba8",))
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    mpix_per_step = len(frames) * cfg["width"] * cfg["height"] / 1e6
    value = mpix_per_step * len(times) / sum(times)
    line = {"metric": METRIC, "value": round(value, 3), "unit": "MPix/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * sum(times) / len(times), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(cfg, world),
            "cpu_baseline": {"value": round(value, 3), "unit": "MPix/s", "cores": threads, "kind": "port",
                             "sample": "each step the workload's %d full frames (one per noise level), oracle fp32, "
                                       "%d threads" % (len(frames), threads)},
            "e2e": {"value": round(value, 3), "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_cpu_replicas(args, cfg):
    """--cpu-replicas: the replica plumbing of the GPU arm on the CPU (gloo) -- process group,
    barriers, each rank converting frames of its own (the oracle stands in for the GPU),
    max-over-ranks timing -- and one check line from rank 0."""
    import hashlib

    import torch
    import torch.distributed as dist
    from oracle import oracle as orc
    from tests.helpers import oracle_params

    rank, world, _ = init_replicas("gloo")
    frames = make_frames(cfg, rank, reference=True)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        outs = [orc.demosaic(f[0], oracle_params(f[2]), orc.F32, want=("rgba8",))["rgba8"] for f in frames]
    total_ms = max_over_ranks(1e3 * (time.perf_counter() - t0), world, torch.device("cpu"))
    barrier(world)
    digest = hashlib.sha256(b"".join(o.tobytes() for o in outs)).hexdigest()
    digests = [None] * world
    if world > 1:
        dist.all_gather_object(digests, digest)
    else:
        digests = [digest]
    if rank == 0:
        mpix = len(frames) * cfg["width"] * cfg["height"] / 1e6
        print(json.dumps({"check": "cpu-replicas", "n_ranks": world, "steps": args.steps,
                          "value": round(replica_value(world, mpix, args.steps, total_ms), 3), "unit": "MPix/s",
                          "slowest_ms": round(total_ms, 3), "digests": digests,
                          "config": workload_config(cfg, world)}), flush=True)
    if world > 1:
        dist.destroy_process_group()


def single_frame_line(ctx, cfg, dev, args, flush):
    """One configuration's own line: its frame alone per step through RawConverter::demosaicImage
    (device-resident, CUDA events, L2 flushed between steps), the same through host buffers
    (pinned raw in and output back, copies inside the timed region), and the whole-pipeline
    algorithmic bandwidth with the configuration's storage and output bytes."""
    import torch
    from climage_gb300 import configs, gls
    raw, _, spec = make_frames(cfg, 0)[0]
    h, w = raw.shape
    out_f32 = cfg["out"] == "rgba_f32"
    half = cfg["storage"] == gls.STORAGE_F16
    p = configs.to_gls_params(spec)
    conv = gls.RawConverter(ctx)
    raw_d = torch.from_numpy(raw).to(dev)
    out_d = torch.empty((h, w, 4), dtype=torch.float32 if out_f32 else torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        conv.demosaicImage(raw_d, p, out_d)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in ev:
        flush.fill_(1)
        a.record(stream)
        conv.demosaicImage(raw_d, p, out_d)
        b.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    # end to end: pinned host raw -> device, convert, output -> pinned host; an 8-bit output
    # goes through the host-buffer entry point (the converter's own overlapped copies), a float
    # output (which that entry point does not produce) through copies around demosaicImage
    raw_h = torch.from_numpy(raw).pin_memory()
    out_h = torch.empty(out_d.shape, dtype=out_d.dtype).pin_memory()

    def e2e_step():
        if out_f32:
            raw_d.copy_(raw_h, non_blocking=True)
            conv.demosaicImage(raw_d, p, out_d)
            out_h.copy_(out_d, non_blocking=True)
            torch.cuda.synchronize()
        else:
            conv.demosaicImageHostPtr(raw_h.data_ptr(), w, h, p, out_h.data_ptr(), 4)

    for _ in range(args.warmup):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    conv.close()
    peak, _ = measured_peak_hbm()
    S, O = (8 if half else 16), (16 if out_f32 else 4)
    bpp = algorithmic_bytes_per_px(S, O, cfg["levels"])
    achieved = bpp * w * h / (ms / 1e3) / 1e9
    return {"workload": cfg["name"], "value": round(w * h / 1e3 / ms, 3), "unit": "MPix/s", "ms_per_frame": round(ms, 4),
            "e2e": {"value": round(w * h / 1e3 / e2e_ms, 3), "unit": "MPix/s", "h2d_bytes_per_step": int(raw.nbytes),
                    "d2h_bytes_per_step": int(out_d.numel() * out_d.element_size()),
                    "path": "torch copies around demosaicImage" if out_f32 else
                            "host-buffer entry point (gls_raw_converter_demosaic_host), RGBA8"},
            "storage": "fp16" if half else "fp32", "output": "rgba_f32" if out_f32 else "rgba8", "levels": cfg["levels"],
            "pipeline_roofline": {"algorithmic_bytes_per_px": round(bpp, 2), "achieved": round(achieved, 1),
                                  "unit": "GB/s", "frac": round(achieved / peak, 4)},
            "timing": "one frame per step, CUDA events, L2 flushed between steps; e2e by the host clock"}


def burst_vs_oracle(burst, bouts):
    """Four frames of the batched burst against the oracle, outside any timed region: the first
    8064x6048 frame, the first 10-bit and the first 14-bit frames, and frames of the CFA phases
    still missing, until every phase is covered or four frames are chosen."""
    from oracle import oracle as orc
    from tests.helpers import oracle_params
    picks, phases = [], set()

    def take(i):
        if i is not None and i not in picks and len(picks) < 4:
            picks.append(i)
            phases.add(burst[i][1]["bayer_pattern"])

    take(next((i for i, (r, _) in enumerate(burst) if r.shape[1] == 8064), None))
    take(next((i for i, (_, sp) in enumerate(burst) if sp["white_level"] == 1023), None))
    take(next((i for i, (_, sp) in enumerate(burst) if sp["white_level"] == 16383), None))
    for i, (_, sp) in enumerate(burst):
        if sp["bayer_pattern"] not in phases:
            take(i)
    res = []
    for i in picks:
        raw, sp = burst[i]
        ref = orc.demosaic(raw.cpu().numpy(), oracle_params(sp), orc.F32, want=("rgba8",))["rgba8"]
        got = bouts[i].cpu().numpy()
        res.append({"frame": i, "size": "%dx%d" % (raw.shape[1], raw.shape[0]), "cfa": int(sp["bayer_pattern"]),
                    "bits": {1023: 10, 4095: 12, 16383: 14}.get(int(sp["white_level"]), 0),
                    "codes_differing": int((got[..., :3] != ref[..., :3]).sum())})
    return {"bit_exact": all(r["codes_differing"] == 0 for r in res), "frames": res}


def force_shapes(gls, spec):
    """Apply --shapes: 'kernel=shape' pairs, names from gls.TUNE_SHAPES."""
    kernels = {"demosaic": gls.TUNE_DEMOSAIC, "final": gls.TUNE_FINAL}
    for item in filter(None, spec.split(",")):
        name, _, shape = item.partition("=")
        k = kernels[name.strip()]
        gls.tune_force(k, gls.TUNE_SHAPES[k].index(shape.strip()))


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    args = parse(argv)
    rc = launch_replicas(args, argv)
    if rc is not None:
        sys.exit(rc)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.cpu_replicas:
        run_cpu_replicas(args, load_file("gls_workload_configs", "climage_gb300/configs.py").CPU_REPLICA_CHECK)
        return
    from climage_gb300 import configs
    cfg = configs.CONFIG2
    import torch
    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
    init_replicas("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    from climage_gb300 import gls

    force_shapes(gls, args.shapes)
    frames = make_frames(cfg, rank)
    ctx = gls.Context(dev.index)
    conv = gls.RawConverter(ctx)
    h, w = cfg["height"], cfg["width"]
    raws = [torch.from_numpy(f[0]).to(dev) for f in frames]
    params = [configs.to_gls_params(f[2]) for f in frames]
    outs = [torch.empty((h, w, 4), dtype=torch.uint8, device=dev) for _ in frames]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    # the frames of a step are a burst: one lane (converter on its own stream) per frame
    lanes = len(frames)
    batch = gls.RawBatch(ctx, lanes)
    batch.reserve(w, h, cfg["levels"], cfg["storage"])

    def step():
        batch.demosaic(raws, params, outs)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    launches0 = ctx.kernel_launches()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(dev.index)
    with sampler:
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
            step()
            ends[k].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    launches = ctx.kernel_launches() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(sum(step_ms), world, dev)
    mpix_per_step = len(frames) * w * h / 1e6
    value = replica_value(world, mpix_per_step, args.steps, total_ms)

    # ---- per-stage profile (separate pass) and roofline of the dominant kernel ----
    conv.profile(True)
    for _ in range(2):
        for r, p, o in zip(raws, params, outs):
            conv.demosaicImage(r, p, o, defer_noise_model=True)
    torch.cuda.synchronize()
    prof = conv.profileReport()
    conv.profile(False)
    peak, peak_kind = measured_peak_hbm()
    S1, S4 = 4, 16
    dom = max((k for k in prof if stage_bytes(k, S1, S4)), key=lambda k: prof[k][0])
    dom_ms = prof[dom][0] / prof[dom][1]
    dom_bytes = stage_bytes(dom, S1, S4) * w * h
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    bpp = algorithmic_bytes_per_px(16, 4, cfg["levels"])
    frame_ms = total_ms / args.steps / len(frames)
    pipe_achieved = bpp * w * h / (frame_ms / 1e3) / 1e9

    # ---- end to end through the host-buffer entry point ----
    e2e = None
    if not args.no_e2e and not args.profile_only:
        # the host product is RGB8, as the reference's demosaicImage + convertToRGBImage give it
        # (raw_converter.cpp:226-237): the alpha byte never crosses to the host
        hosts = [torch.from_numpy(f[0]).pin_memory() for f in frames]
        houts = [torch.empty((h, w, 3), dtype=torch.uint8).pin_memory() for _ in frames]

        def host_step():
            batch.demosaic_host_ptr([t.data_ptr() for t in hosts], [(w, h)] * len(frames), params,
                                    [t.data_ptr() for t in houts], 3)

        for _ in range(args.warmup):
            host_step()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            host_step()
        e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
        e2e = {"value": round(replica_value(world, mpix_per_step, args.steps, 1e3 * e2e_s), 3), "unit": "MPix/s",
               "h2d_bytes_per_step": int(sum(f[0].nbytes for f in frames)),
               "d2h_bytes_per_step": int(len(frames) * w * h * 3), "output": "rgb8 host buffers",
               "overlap": "uploads one frame at a time; the final stage in 8 row bands, each copied back "
                          "while the next band runs"}
        # the same burst from packed 12-bit host frames (an uncompressed DNG strip's layout):
        # the packed bytes cross to the device and are unpacked there
        from climage_gb300 import synthetic
        packed = [torch.from_numpy(np.frombuffer(synthetic.pack_bits(f[0], cfg["bits"]), np.uint8).copy()).pin_memory()
                  for f in frames]

        def packed_step():
            batch.demosaic_packed_host_ptr([t.data_ptr() for t in packed], [t.numel() for t in packed],
                                           [cfg["bits"]] * len(frames), [(w, h)] * len(frames), params,
                                           [t.data_ptr() for t in houts], 3)

        for _ in range(args.warmup):
            packed_step()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            packed_step()
        pk_s = max_over_ranks(time.perf_counter() - t0, world, dev)
        e2e["packed_input"] = {"value": round(replica_value(world, mpix_per_step, args.steps, 1e3 * pk_s), 3), "unit": "MPix/s",
                               "h2d_bytes_per_step": int(sum(t.numel() for t in packed)), "bits": cfg["bits"]}

    # ---- the learned form: the same burst with the learned stage (shipped parameters) ----
    learned_line = None
    if not args.no_learned and not args.profile_only:
        from climage_gb300 import learned
        prm = learned.load_params()
        if prm is not None:
            cnn = gls.Cnn(ctx)
            cnn.set_params(prm)
            lb = gls.RawBatch(ctx, lanes)
            lb.reserve(w, h, cfg["levels"], cfg["storage"])
            lb.set_cnn(cnn)
            for _ in range(args.warmup):
                lb.demosaic(raws, params, outs)
            torch.cuda.synchronize()
            barrier(world)
            ls = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
            le = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
            for k in range(args.steps):
                flush.fill_(k & 0xFF)
                ls[k].record(stream)
                lb.demosaic(raws, params, outs)
                le[k].record(stream)
            torch.cuda.synchronize()
            lms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(ls, le)), world, dev)
            verdict = learned.judge(ctx, cnn, range(10**6, 10**6 + 2))
            learned_line = {"value": round(replica_value(world, mpix_per_step, args.steps, lms), 3), "unit": "MPix/s",
                            "ms_per_step": round(lms / args.steps, 4),
                            "judge": {k: verdict[k] for k in ("plain", "learned", "linear_input", "linear_corrected")},
                            "judge_frames": "2 held-out 1024x768 scenes, read sigma 4-16 DN, gain 0.25-4"}
            lb.close()
            cnn.close()

    # ---- autoWhiteBalance of the first frame (its own entry point, bit-exact) ----
    awb_line = None
    if rank == 0 and not args.no_awb and not args.profile_only:
        sp = frames[0][2]
        awb_args = (gls.cam_ycbcr(np.array(sp["rgb_cam"], np.float32).reshape(3, 3)), sp["scale_mul"],
                    sp["white_level"], sp["black_level"], cfg["bayer"])
        for _ in range(3):
            wb, hl = ctx.autoWhiteBalance(raws[0], *awb_args)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(5):
            wb, hl = ctx.autoWhiteBalance(raws[0], *awb_args)
        a1.record(stream)
        torch.cuda.synchronize()
        awb_ms = a0.elapsed_time(a1) / 5
        awb_line = {"ms_per_frame": round(awb_ms, 4), "mpix_s": round(w * h / 1e3 / awb_ms, 1),
                    "gains": [float(v) for v in wb], "highlights": float(hl),
                    "note": "one call per frame, synchronous (16-byte result read back); the reference's fp32 "
                            "sums are kept in quad order, one block per tile"}
        if world == 1 and not args.no_cpu:
            from oracle import oracle as orc
            t0 = time.perf_counter()
            owb, ohl = orc.auto_white_balance(frames[0][0], *awb_args)
            awb_line["cpu_baseline"] = {"ms_per_frame": round((time.perf_counter() - t0) * 1e3, 1), "cores": 1,
                                        "kind": "port"}
            awb_line["bit_exact_vs_oracle"] = bool(np.array_equal(owb.view(np.uint32), wb.view(np.uint32))
                                                   and np.float32(ohl).view(np.uint32) == np.float32(hl).view(np.uint32))

    # ---- the batched form: a 64-frame uneven burst captured once in a CUDA graph ----
    batched_line = None
    if rank == 0 and not args.no_batched and not args.profile_only:
        from climage_gb300 import configs
        burst = make_burst([f[0] for f in frames], dev)
        bstream = torch.cuda.Stream(dev)
        bctx = gls.Context(dev.index, stream=bstream)
        blanes = 4
        bb = gls.RawBatch(bctx, blanes)
        bb.reserve(max(r.shape[1] for r, _ in burst), max(r.shape[0] for r, _ in burst), 4, gls.STORAGE_F32)
        braws = [r for r, _ in burst]
        bparams = [configs.to_gls_params(sp) for _, sp in burst]
        bouts = [torch.empty((r.shape[0], r.shape[1], 4), dtype=torch.uint8, device=dev) for r, _ in burst]
        with torch.cuda.stream(bstream):
            bb.demosaic(braws, bparams, bouts)  # eager: buffers settle before capture
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        l0 = bctx.kernel_launches()
        with torch.cuda.graph(graph, stream=bstream):
            bb.demosaic(braws, bparams, bouts)
        kernels_per_replay = bctx.kernel_launches() - l0
        for _ in range(args.warmup):
            graph.replay()
        torch.cuda.synchronize()
        bs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        be = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for k in range(args.steps):
            with torch.cuda.stream(bstream):
                flush.fill_(k & 0xFF)
                bs[k].record(bstream)
                graph.replay()
                be[k].record(bstream)
        torch.cuda.synchronize()
        bms = float(sum(a.elapsed_time(b) for a, b in zip(bs, be))) / args.steps
        bpx = sum(r.numel() for r, _ in burst)
        batched_line = {"value": round(bpx / 1e3 / bms, 3), "unit": "MPix/s", "ms_per_burst": round(bms, 3),
                        "frames": len(burst), "mpix_per_burst": round(bpx / 1e6, 2), "lanes": blanes,
                        "kernels_per_replay": int(kernels_per_replay), "levels": 4, "output": "rgba8",
                        "launch": "one CUDA graph replay per burst (captured once)",
                        "sizes": "uniform over 1920x1080, 2016x1512, 4032x3024, 8064x6048",
                        "frame_data": "crops, 2x2 tilings and one-pixel shifts of the rendered 4032x3024 frames; "
                                      "10/14-bit by bit shifts; per-frame WB gains in [1, 3]"}
        del graph
        if world == 1 and not args.no_cpu:
            batched_line["bit_exact_vs_oracle"] = burst_vs_oracle(burst, bouts)
        # the same burst with the learned stage (shipped parameters): batched + learned
        if not args.no_learned:
            from climage_gb300 import learned
            prm = learned.load_params()
            if prm is not None:
                bcnn = gls.Cnn(bctx)
                bcnn.set_params(prm)
                bb.set_cnn(bcnn)
                with torch.cuda.stream(bstream):
                    bb.demosaic(braws, bparams, bouts)
                torch.cuda.synchronize()
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph, stream=bstream):
                    bb.demosaic(braws, bparams, bouts)
                for _ in range(args.warmup):
                    graph.replay()
                torch.cuda.synchronize()
                for k in range(args.steps):
                    with torch.cuda.stream(bstream):
                        flush.fill_(k & 0xFF)
                        bs[k].record(bstream)
                        graph.replay()
                        be[k].record(bstream)
                torch.cuda.synchronize()
                lms = float(sum(a.elapsed_time(b) for a, b in zip(bs, be))) / args.steps
                bcnn.status()
                batched_line["learned"] = {"value": round(bpx / 1e3 / lms, 3), "unit": "MPix/s",
                                           "ms_per_burst": round(lms, 3),
                                           "vs_plain_value": round(bpx / 1e3 / lms / value, 3),
                                           "launch": "one CUDA graph replay per burst, learned stage on every frame"}
                del graph
                bb.set_cnn(None)
                bcnn.close()
        bb.close()
        bctx.close()
        del braws, bouts, burst

    # ---- configurations 1 and 3 on their own lines ----
    config_lines = None
    if rank == 0 and not args.no_configs and not args.profile_only:
        config_lines = {"config1": single_frame_line(ctx, configs.CONFIG1, dev, args, flush),
                        "precision_form": single_frame_line(ctx, configs.CONFIG3, dev, args, flush)}

    # ---- DNG ingest: the first frame as one lossless-JPEG strip (the layout the reference's
    # DNG writer uses), decoded from pinned host memory into the device frame ----
    dng_line = None
    if rank == 0 and world == 1 and not args.no_cpu and not args.no_dng and not args.profile_only:
        from oracle import oracle as orc
        raw0 = frames[0][0]
        stream = orc.lj92_encode(raw0, 1, cfg["bits"], 1, 0)  # the input (test encoder)
        pinned = torch.from_numpy(np.frombuffer(stream, np.uint8).copy()).pin_memory()
        dec = torch.empty((h, w), dtype=torch.int32, device=dev).to(torch.uint16)
        for _ in range(3):
            ctx.decodeLosslessJPEG(pinned.numpy(), [0], [len(stream)], w, h, dec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            ctx.decodeLosslessJPEG(pinned.numpy(), [0], [len(stream)], w, h, dec)
        torch.cuda.synchronize()
        dms = (time.perf_counter() - t0) / 5 * 1e3
        exact = bool(np.array_equal(dec.cpu().numpy(), raw0))
        t0 = time.perf_counter()
        orc.lj92_decode(stream)
        cms = (time.perf_counter() - t0) * 1e3
        dng_line = {"ms_per_frame": round(dms, 3), "mpix_s": round(w * h / 1e3 / dms, 1),
                    "stream_bytes": len(stream), "bit_exact": exact,
                    "layout": "one strip, one component, predictor 1, %d-bit" % cfg["bits"],
                    "timed": "host pinned stream in, decoded frame in HBM, synchronous call",
                    "cpu_baseline": {"ms_per_frame": round(cms, 1), "cores": 1, "kind": "port"}}

    cpu = psnr = None
    if rank == 0 and world == 1 and not args.no_cpu and not args.profile_only:
        gpu_rgb = None
        if not args.no_psnr:
            fo = torch.empty((h, w, 4), dtype=torch.float32, device=dev)
            conv.demosaicImage(raws[0], configs.to_gls_params(frames[0][2]), fo, defer_noise_model=True)
            torch.cuda.synchronize()
            gpu_rgb = fo.cpu().numpy()[..., :3]
        cpu, psnr = cpu_leg(frames, gpu_rgb=gpu_rgb)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "MPix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(cfg, world),
            "schedule": "the step's frames as one burst over %d streams (gls_raw_batch)" % lanes,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": NCU_TRAFFIC[dom][0] if dom in NCU_TRAFFIC else None, "traffic_unit": "B/launch",
                         "algorithmic_bytes_per_launch": int(dom_bytes),
                         "issue_active_pct": NCU_TRAFFIC[dom][1] if dom in NCU_TRAFFIC else None,
                         "algorithmic_bytes_per_px": stage_bytes(dom, S1, S4)},
            "pipeline_roofline": {"algorithmic_bytes_per_px": round(bpp, 2), "achieved": round(pipe_achieved, 1),
                                  "unit": "GB/s", "frac": round(pipe_achieved / peak, 4), "ms_per_frame": round(frame_ms, 4)},
            "stages_ms_per_frame": {k: round(v[0] / (2 * len(frames)), 4) for k, v in prof.items()},
            # per full-resolution stage: its compulsory bytes over its time, as a fraction of the
            # measured HBM peak (the stages are issue-bound; issue_active_pct says by how much)
            "stages_roofline_frac": {k: round(stage_bytes(k, S1, S4) * w * h / (v[0] / (2 * len(frames)) / 1e3) / 1e9 / peak, 4)
                                     for k, v in prof.items() if stage_bytes(k, S1, S4) and v[0] > 0},
            "gpu_launches": int(launches),
            "clocks": sampler.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
            "psnr_vs_fp64": psnr,
            "learned_form": learned_line,
            "auto_white_balance": awb_line,
            "dng_decode": dng_line,
            "batched_form": batched_line,
            "config1": config_lines["config1"] if config_lines else None,
            "precision_form": config_lines["precision_form"] if config_lines else None,
            "tuner": tuner_summary(),
        }
        print(json.dumps(line), flush=True)
    conv.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
