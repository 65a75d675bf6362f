"""Pipeline parameter sets and the benchmark workloads.

A *spec* is a plain dict with every DemosaicParameters field (demosaic.hpp:61-81); the
product turns it into gls_demosaic_params (to_gls_params), and the tests turn the same
dict into the oracle's parameter block, so both sides always run on identical floats.

Parameter sources in the reference:
  * cam_xyz: the Adobe-style colour matrix of transcodeAdobeDNG (raw_pipeline.cpp:77),
    converted by cam_xyz_coeff (demosaic_utils.cpp:25-52);
  * scale_mul: unpackDNGMetadata's white balance (demosaic_utils.cpp:366-371);
  * initial noise model and the "plain" denoise parameters: demosaicPlainFile
    (raw_pipeline.cpp:89-146);
  * the "strong" denoise parameters: Sonya6400DenoiseParameters (Sonya6400Calibration.cpp:182-233);
  * tone mapping with LTM: demosaicIMX571DNG (IMX571Calibration.cpp:287-304).

This module loads no native library by itself: the camera-matrix conversion is the
product's (gls.cam_xyz_coeff) unless the caller passes another implementation of it, and
only to_gls_params needs the product's parameter block.  bench.py's reference arm loads
this file on its own and passes the oracle's cam_xyz_coeff, so that arm never maps the
product's library.
"""
import math

import numpy as np

# image storage precision (gls_cuda.h GLS_STORAGE_F32 / _F16 / _F16_STATS)
STORAGE_F32, STORAGE_F16, STORAGE_F16_STATS = 0, 1, 2

CAM_XYZ = [1.4955, -0.6760, -0.1453, -0.1341, 1.0072, 0.1269, -0.0647, 0.1987, 0.4304]

RAW_NLF0 = [2.8482e-04, 3.6848e-04, 3.3079e-04, 3.2821e-04]
PYRAMID_NLF0 = [
    [2.1e-04, 1.0e-08, 8.2e-06, 2.6e-04, 3.9e-05, 9.0e-06],
    [1.6e-04, 1.0e-08, 1.6e-06, 6.1e-04, 1.8e-04, 6.1e-05],
    [2.5e-04, 1.0e-08, 1.0e-08, 6.0e-04, 3.6e-04, 1.3e-04],
    [4.2e-04, 1.0e-08, 1.0e-08, 4.2e-04, 8.8e-04, 3.4e-04],
    [3.0e-04, 1.0e-08, 1.0e-08, 1.0e-03, 1.8e-03, 4.2e-04],
]

RGB_DEFAULT = dict(contrast=1.05, saturation=1.0, toneCurveSlope=3.5, exposureBias=0.0, blacks=0.0, localToneMapping=0)
RGB_LTM = dict(contrast=1.0, saturation=0.9, toneCurveSlope=3.5, exposureBias=-0.8, blacks=0.12, localToneMapping=1)
LTM_DEFAULT = dict(guidedFilterEps=0.01, shadows=1.25, highlights=1.0, detail=1.1)


def scale_mul_from(pre_mul, black, white, exposure_multiplier=1.0):
    """unpackDNGMetadata (demosaic_utils.cpp:366-371), with its float/double promotions."""
    pre = np.asarray(pre_mul, np.float32)
    mn = pre.min()
    em = np.float32(max(exposure_multiplier, 1.0))
    out = []
    for c in range(4):
        idx = 1 if c == 3 else c
        ratio = np.float32(pre[idx] / mn)
        v = float(np.float32(em * ratio)) * 65535.0 / float(np.float32(white) - np.float32(black))
        out.append(float(np.float32(v)))
    return out


def denoise_plain(levels):
    return [dict(luma=0.125, chroma=0.125, chromaBoost=1.0, gradientBoost=1.0, sharpening=1.0) for _ in range(levels)]


def denoise_strong(levels, iso=1600):
    a = min(max((math.log2(iso) - math.log2(100)) / (math.log2(102400) - math.log2(100)), 0.0), 1.0)
    lerp = float(np.float32(0.125 + (1.2 - 0.125) * a))
    lerp_c = float(np.float32(0.5 + (2.0 - 0.5) * a))
    lmult = [0.25, 2, 0.5, 0.25, 0.125]
    out = []
    for i in range(levels):
        lm = lmult[min(i, 4)]
        sharp = float(np.float32(1.5 + (1.0 - 1.5) * a)) if i == 0 else (1.1 if i == 1 else 1.0)
        out.append(dict(luma=float(np.float32(lm * lerp)), chroma=float(np.float32(1 * lerp_c)), chromaBoost=4.0,
                        gradientBoost=2.0, sharpening=sharp))
    return out


def make_spec(meta, levels=5, storage=STORAGE_F32, ltm=True, noise_level=0.2, denoise="plain", algorithm=0,
              exposure_multiplier=1.0, cam_xyz_coeff=None):
    if cam_xyz_coeff is None:
        from . import gls
        cam_xyz_coeff = gls.cam_xyz_coeff
    pre_mul, rgb_cam = cam_xyz_coeff(CAM_XYZ)
    wb = meta["wb"]
    pyr = [PYRAMID_NLF0[min(i, 4)] for i in range(levels)]
    return dict(
        bayer_pattern=meta["bayer"],
        black_level=float(meta["black"]),
        white_level=float(meta["white"]),
        exposure_multiplier=float(exposure_multiplier),
        scale_mul=scale_mul_from(wb, meta["black"], meta["white"], exposure_multiplier),
        rgb_cam=[float(v) for v in np.ravel(rgb_cam)],
        raw_nlf=list(RAW_NLF0),
        pyramid_nlf=[list(r) for r in pyr],
        denoise=denoise_plain(levels) if denoise == "plain" else denoise_strong(levels),
        noise_level=float(noise_level),
        rgb=dict(RGB_LTM if ltm else RGB_DEFAULT),
        ltm=dict(LTM_DEFAULT),
        pyramid_levels=int(levels),
        denoise_algorithm=int(algorithm),
        storage=int(storage),
    )


def to_gls_params(spec):
    from . import gls
    p = gls.DemosaicParams()
    p.bayer_pattern = spec["bayer_pattern"]
    p.black_level = spec["black_level"]
    p.white_level = spec["white_level"]
    p.exposure_multiplier = spec["exposure_multiplier"]
    for i in range(4):
        p.scale_mul[i] = spec["scale_mul"][i]
        p.raw_nlf[i] = spec["raw_nlf"][i]
    for i in range(9):
        p.rgb_cam[i] = spec["rgb_cam"][i]
    for i, row in enumerate(spec["pyramid_nlf"]):
        for k in range(6):
            p.pyramid_nlf[i][k] = row[k]
    for i, d in enumerate(spec["denoise"]):
        for k, v in d.items():
            setattr(p.denoise[i], k, v)
    p.noise_level = spec["noise_level"]
    for k, v in spec["rgb"].items():
        setattr(p.rgb_conversion, k, v)
    for k, v in spec["ltm"].items():
        setattr(p.ltm, k, v)
    p.pyramid_levels = spec["pyramid_levels"]
    p.denoise_algorithm = spec["denoise_algorithm"]
    p.storage = spec["storage"]
    p.rotate_180 = int(spec.get("rotate_180", 0))
    return p


# ---- benchmark workloads (synthetic frames stand in for DNG captures) ----

CONFIG1 = dict(name="plain-1024x768-rggb12-4lvl", width=1024, height=768, bayer=2, bits=12, black=64, white=4095,
               wb=(2.0, 1.0, 1.6), noise=[(3.0, 2.0, 0.2)], levels=4, storage=STORAGE_F32, out="rgba_f32")
CONFIG2 = dict(name="plain-4032x3024-rggb12-5lvl", width=4032, height=3024, bayer=2, bits=12, black=64, white=4095,
               wb=(2.0, 1.0, 1.6), noise=[(2.0, 1.0, 0.2), (6.0, 4.0, 0.45), (12.0, 16.0, 0.7)], levels=5,
               storage=STORAGE_F32, out="rgba8")
CONFIG3 = dict(name="fp16-8064x6048-grbg14-6lvl", width=8064, height=6048, bayer=0, bits=14, black=256, white=16383,
               wb=(2.0, 1.0, 1.6), noise=[(3.0, 2.0, 0.2)], levels=6, storage=STORAGE_F16, out="rgba8")
# the replica plumbing check on the CPU (bench.py --cpu-replicas): frames small enough for
# the oracle to convert in well under a second
CPU_REPLICA_CHECK = dict(name="plain-64x48-rggb12-5lvl", width=64, height=48, bayer=2, bits=12, black=64, white=4095,
                         wb=(2.0, 1.0, 1.6), noise=[(2.0, 1.0, 0.2), (6.0, 4.0, 0.45), (12.0, 16.0, 0.7)], levels=5,
                         storage=STORAGE_F32, out="rgba8")
