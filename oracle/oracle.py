"""ctypes wrapper of the CPU oracle (liboracle.so) and of the reference-host shim.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg as the checker of the CUDA pipeline; the product never imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_host.so")

F32, F16, F64 = 0, 1, 2
F16_STATS = 3  # F16 storage with the noise-statistics images in fp16 too (the shipped build)
MAX_LEVELS = 8


class DenoiseParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("luma", "chroma", "chromaBoost", "gradientBoost", "sharpening")]


class RGBParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("contrast", "saturation", "toneCurveSlope", "exposureBias", "blacks")] + [
        ("localToneMapping", ctypes.c_int)
    ]


class LTMParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("guidedFilterEps", "shadows", "highlights", "detail")]


class Params(ctypes.Structure):
    _fields_ = [
        ("bayer_pattern", ctypes.c_int),
        ("black_level", ctypes.c_float),
        ("white_level", ctypes.c_float),
        ("exposure_multiplier", ctypes.c_float),
        ("scale_mul", ctypes.c_float * 4),
        ("rgb_cam", ctypes.c_float * 9),
        ("noise_level", ctypes.c_float),
        ("pyramid_levels", ctypes.c_int),
        ("denoise_algorithm", ctypes.c_int),
        ("rotate_180", ctypes.c_int),
        ("raw_nlf", ctypes.c_float * 4),
        ("pyramid_nlf", (ctypes.c_float * 6) * MAX_LEVELS),
        ("denoise", DenoiseParams * MAX_LEVELS),
        ("rgb", RGBParams),
        ("ltm", LTMParams),
    ]


class Taps(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("scaled_raw", "green", "linear_rgb", "ycbcr", "level0", "denoised0", "ltm_mask", "camera_rgb")]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle/liboracle.so is not built: run __graft_entry__.build() or make -C oracle")
        _lib = ctypes.CDLL(LIB_PATH)
        f = ctypes.c_float
        for name, res, args in [
            ("oracle_atan2pi", f, [f, f]),
            ("oracle_tanh", f, [f]),
            ("oracle_exp2", f, [f]),
            ("oracle_log2", f, [f]),
            ("oracle_pow", f, [f, f]),
            ("oracle_f32_to_f16", ctypes.c_uint16, [f]),
            ("oracle_f16_to_f32", f, [ctypes.c_uint16]),
            ("oracle_unpack_bits", ctypes.c_long, [ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_void_p, ctypes.c_long]),
            ("oracle_regress", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
        ]:
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def ref_lib():
    """The reference's own host code compiled from its sources, or None when absent."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        _ref = ctypes.CDLL(REF_PATH, mode=os.RTLD_LAZY)
    return _ref


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _arr(vals, n):
    return (ctypes.c_float * n)(*[float(v) for v in vals])


def set_threads(n):
    lib().oracle_set_threads(int(n))


def threads():
    return lib().oracle_threads()


# ---- whole pipeline ----

def demosaic(raw, params, prec=F32, want=("rgba8",), taps=()):
    """Runs the pipeline; returns a dict with 'rgba8'/'rgbaf', the taps asked for and the
    updated params (raw_nlf, pyramid_nlf)."""
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    h, w = raw.shape
    out = {}
    o8 = np.zeros((h, w, 4), np.uint8) if "rgba8" in want else None
    of = np.zeros((h, w, 4), np.float32) if "rgbaf" in want else None
    t = Taps()
    shapes = {"scaled_raw": (h, w), "green": (h, w), "linear_rgb": (h, w, 4), "ycbcr": (h, w, 4),
              "level0": (h, w, 4), "denoised0": (h, w, 4), "ltm_mask": (h, w), "camera_rgb": (h, w, 4)}
    bufs = {}
    for name in taps:
        bufs[name] = np.zeros(shapes[name], np.float32)
        setattr(t, name, bufs[name].ctypes.data)
    rc = lib().oracle_demosaic(_p(raw), w, h, w, ctypes.byref(params), prec, _p(o8), _p(of), ctypes.byref(t))
    if rc != 0:
        raise ValueError("oracle_demosaic failed: %d" % rc)
    if o8 is not None:
        out["rgba8"] = o8
    if of is not None:
        out["rgbaf"] = of
    out.update(bufs)
    out["raw_nlf"] = np.array(params.raw_nlf[:], np.float32)
    out["pyramid_nlf"] = np.array([params.pyramid_nlf[i][:] for i in range(params.pyramid_levels)], np.float32)
    return out


def fast_demosaic(raw, params, prec=F32):
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    h, w = raw.shape
    o8 = np.zeros((h // 2, w // 2, 4), np.uint8)
    of = np.zeros((h // 2, w // 2, 4), np.float32)
    rc = lib().oracle_fast_demosaic(_p(raw), w, h, w, ctypes.byref(params), prec, _p(o8), _p(of))
    if rc != 0:
        raise ValueError("oracle_fast_demosaic failed: %d" % rc)
    return o8, of


# ---- single stages ----

def scale_raw(raw, bayer, scale_mul, black_norm, prec=F32):
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    h, w = raw.shape
    out = np.zeros((h, w), np.float32)
    lib().oracle_scale_raw(_p(raw), w, h, w, bayer, _arr(scale_mul, 4), ctypes.c_float(black_norm), prec, _p(out))
    return out


def raw_noise_statistics(scaled, bayer):
    s = _f32(scaled)
    h, w = s.shape
    mean = np.zeros((h // 2, w // 2, 4), np.float32)
    var = np.zeros((h // 2, w // 2, 4), np.float32)
    lib().oracle_raw_noise_statistics(_p(s), w, h, bayer, _p(mean), _p(var))
    return mean, var


def compute_raw_nlf(scaled, bayer):
    s = _f32(scaled)
    h, w = s.shape
    out = (ctypes.c_float * 8)()
    lib().oracle_compute_raw_nlf(_p(s), w, h, bayer, out)
    return np.array(out[:], np.float32)


def interpolate_green(scaled, bayer, luma_variance, prec=F32):
    s = _f32(scaled)
    h, w = s.shape
    out = np.zeros((h, w), np.float32)
    lib().oracle_interpolate_green(_p(s), w, h, bayer, ctypes.c_float(luma_variance), prec, _p(out))
    return out


def interpolate_red_blue(scaled, green, bayer, chroma_variance, prec=F32, rotate_180=False):
    s, g = _f32(scaled), _f32(green)
    h, w = s.shape
    out = np.zeros((h, w, 4), np.float32)
    lib().oracle_interpolate_red_blue(_p(s), _p(g), w, h, bayer, ctypes.c_float(chroma_variance), prec,
                                      int(bool(rotate_180)), _p(out))
    return out


def blend_highlights(img, clip=1.0, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_blend_highlights(_p(a), w, h, ctypes.c_float(clip), prec, _p(out))
    return out


def transform(img, m, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_transform(_p(a), w, h, _arr(np.ravel(m), 9), prec, _p(out))
    return out


def despeckle(img, var_a, var_b, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_despeckle(_p(a), w, h, _arr(var_a, 3), _arr(var_b, 3), prec, _p(out))
    return out


def downsample(img, ow, oh, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros((oh, ow, 4), np.float32)
    lib().oracle_downsample(_p(a), w, h, ow, oh, prec, _p(out))
    return out


def noise_statistics(img):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_noise_statistics(_p(a), w, h, _p(out))
    return out


def compute_nlf(img):
    a = _f32(img)
    h, w, _ = a.shape
    out = (ctypes.c_float * 6)()
    lib().oracle_compute_nlf(_p(a), w, h, out)
    return np.array(out[:], np.float32)


def denoise_bilateral(img, var_a, var_b, chroma_boost, gradient_boost, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_denoise_bilateral(_p(a), w, h, _arr(var_a, 3), _arr(var_b, 3), ctypes.c_float(chroma_boost),
                                   ctypes.c_float(gradient_boost), prec, _p(out))
    return out


def denoise_guided(img, var_a, var_b, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_denoise_guided(_p(a), w, h, _arr(var_a, 3), _arr(var_b, 3), prec, _p(out))
    return out


def guided_filter(img, filter_size, eps, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_guided_filter(_p(a), w, h, filter_size, _arr(eps, 3), prec, _p(out))
    return out


def reassemble(den0, img1, den1, sharpening, nlf, prec=F32):
    d0, i1, d1 = _f32(den0), _f32(img1), _f32(den1)
    h, w, _ = d0.shape
    h1, w1, _ = i1.shape
    out = np.zeros_like(d0)
    lib().oracle_reassemble(_p(d0), w, h, _p(i1), _p(d1), w1, h1, ctypes.c_float(sharpening), _arr(nlf, 2), prec, _p(out))
    return out


def ltm_mask(img, guide, ltm, m, prec=F32):
    a, g = _f32(img), _f32(guide)
    h, w, _ = a.shape
    gh, gw, _ = g.shape
    out = np.zeros((h, w), np.float32)
    lib().oracle_ltm_mask(_p(a), w, h, _p(g), gw, gh, ctypes.byref(ltm), _arr(np.ravel(m), 9), prec, _p(out))
    return out


def convert_to_srgb(img, mask, m, rgb):
    a = _f32(img)
    h, w, _ = a.shape
    o8 = np.zeros((h, w, 4), np.uint8)
    of = np.zeros((h, w, 4), np.float32)
    mk = None if mask is None else _f32(mask)
    lib().oracle_convert_to_srgb(_p(a), _p(mk), w, h, _arr(np.ravel(m), 9), ctypes.byref(rgb), _p(o8), _p(of))
    return o8, of


def bayer_to_rgba(scaled, bayer, prec=F32):
    s = _f32(scaled)
    h, w = s.shape
    out = np.zeros((h // 2, w // 2, 4), np.float32)
    lib().oracle_bayer_to_rgba(_p(s), w, h, bayer, prec, _p(out))
    return out


def rgba_to_bayer(rgba, bayer, prec=F32):
    a = _f32(rgba)
    qh, qw, _ = a.shape
    out = np.zeros((2 * qh, 2 * qw), np.float32)
    lib().oracle_rgba_to_bayer(_p(a), 2 * qw, 2 * qh, bayer, prec, _p(out))
    return out


def despeckle_rgba(img, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_despeckle_rgba(_p(a), w, h, prec, _p(out))
    return out


def denoise_rgba(img, raw_variance, prec=F32):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    lib().oracle_denoise_rgba(_p(a), w, h, _arr(raw_variance, 4), prec, _p(out))
    return out


def fast_debayer(scaled, bayer, prec=F32):
    s = _f32(scaled)
    h, w = s.shape
    out = np.zeros((h // 2, w // 2, 4), np.float32)
    lib().oracle_fast_debayer(_p(s), w, h, bayer, prec, _p(out))
    return out


def regress(m, v):
    m = _f32(m)
    v = _f32(v)
    n = v.shape[0]
    mc = 1 if m.ndim == 1 else m.shape[1]
    nc = v.shape[1]
    out = np.zeros(2 * nc, np.float32)
    lib().oracle_regress(_p(m), _p(v), n, mc, nc, _p(out))
    return out


def unpack_bits(packed, bits):
    b = np.ascontiguousarray(np.frombuffer(bytes(packed), np.uint8))
    n = (b.size * 8) // bits
    out = np.zeros(n, np.uint16)
    k = lib().oracle_unpack_bits(_p(b), b.size, bits, _p(out), n)
    if k < 0:
        raise ValueError("unsupported bit depth %d" % bits)
    return out[:k]


def auto_white_balance(raw, rgb_ycbcr, scale_mul, white, black, bayer, reference=False):
    """autoWhiteBalance (demosaic_utils.cpp:976-1026) over a uint16 raw frame: (wb gains
    (3,) with green 1, highlight fraction).  reference=True runs the reference's own code
    (oracle/_ref/libref_host.so) instead of the restatement."""
    raw = np.ascontiguousarray(raw, np.uint16)
    h, w = raw.shape
    wb = (ctypes.c_float * 3)()
    hl = ctypes.c_float()
    args = (_p(raw), w, h, w, _arr(np.ravel(rgb_ycbcr), 9), _arr(scale_mul, 4), ctypes.c_float(white),
            ctypes.c_float(black), int(bayer), wb, ctypes.byref(hl))
    if reference:
        if ref_lib() is None:
            raise FileNotFoundError(REF_PATH)
        ref_lib().ref_auto_white_balance(*args)
    elif lib().oracle_auto_white_balance(*args) != 0:
        raise ValueError("autoWhiteBalance: invalid arguments")
    return np.array(wb[:], np.float32), np.float32(hl.value)


def lj92_decode(stream, reference=False):
    """A lossless-JPEG stream (bytes) -> (samples uint16 (height, width * components), info
    dict); reference=True runs the reference's DecodeLosslessJPEG (oracle/_ref)."""
    b = np.frombuffer(bytes(stream), np.uint8)
    info = (ctypes.c_int * 8)()
    if reference:
        if ref_lib() is None:
            raise FileNotFoundError(REF_PATH)
        fn = ref_lib().ref_lj92_decode
        fn.restype = ctypes.c_long
        probe = lib().oracle_lj92_decode
        probe.restype = ctypes.c_long
        probe(_p(b), b.size, None, 0, info)  # header only: the geometry
        cap = max(info[0] * info[1] * info[2], 1)
        out = np.zeros(cap, np.uint16)
        n = fn(_p(b), ctypes.c_long(b.size), _p(out), ctypes.c_long(cap))
    else:
        fn = lib().oracle_lj92_decode
        fn.restype = ctypes.c_long
        fn(_p(b), b.size, None, 0, info)
        cap = max(info[0] * info[1] * info[2], 1)
        out = np.zeros(cap, np.uint16)
        n = fn(_p(b), ctypes.c_long(b.size), _p(out), ctypes.c_long(cap), info)
    if n < 0:
        raise ValueError("lossless JPEG stream rejected (%d)" % n)
    keys = ("width", "height", "components", "precision", "predictor", "point_transform", "restart_interval",
            "frame_components")
    meta = dict(zip(keys, info[:8]))
    return out[:n].reshape(meta["height"], meta["width"] * meta["components"]), meta


def lj92_encode(samples, components, precision, predictor=1, restart_rows=0, reference=False):
    """(height, width * components) uint16 samples -> lossless-JPEG bytes.  reference=True
    uses the reference's EncodeLosslessJPEG (predictor 1, no restarts)."""
    s = np.ascontiguousarray(samples, np.uint16)
    rows, n = s.shape
    cols = n // components
    cap = s.size * 4 + 4096
    out = np.zeros(cap, np.uint8)
    if reference:
        if predictor != 1 or restart_rows:
            raise ValueError("the reference encoder writes predictor 1 without restarts")
        fn = ref_lib().ref_lj92_encode
        fn.restype = ctypes.c_long
        k = fn(_p(s), rows, cols, components, precision, _p(out), ctypes.c_long(cap))
    else:
        fn = lib().oracle_lj92_encode
        fn.restype = ctypes.c_long
        k = fn(_p(s), rows, cols, components, precision, predictor, restart_rows, _p(out), ctypes.c_long(cap))
    if k < 0:
        raise ValueError("encoding failed (%d)" % k)
    return out[:k].tobytes()


def color_checker_raw_stats(raw, black, white, bayer, gmb, rotate_180=False):
    """colorCheckerRawStats: (mean (24, 4), var (24, 4)) of the CFA channels per patch."""
    raw = np.ascontiguousarray(raw, np.uint16)
    h, w = raw.shape
    mean = np.zeros(96, np.float32)
    var = np.zeros(96, np.float32)
    g = (ctypes.c_int * 4)(*gmb)
    if lib().oracle_color_checker_raw_stats(_p(raw), w, h, w, ctypes.c_float(black), ctypes.c_float(white),
                                            int(bayer), g, int(rotate_180), _p(mean), _p(var)) != 0:
        raise ValueError("colorCheckerRawStats: invalid arguments")
    return mean.reshape(24, 4), var.reshape(24, 4)


def estimate_raw_parameters(raw, black, white, bayer, gmb, rotate_180=False, reference=False):
    """estimateRawParameters: (cam_xyz (3, 3), pre_mul (3,), raw NLF slopes (4,)); reference=True
    runs the reference's own code (oracle/_ref)."""
    raw = np.ascontiguousarray(raw, np.uint16)
    h, w = raw.shape
    cx, pm, nlf = (ctypes.c_float * 9)(), (ctypes.c_float * 3)(), (ctypes.c_float * 4)()
    g = (ctypes.c_int * 4)(*gmb)
    args = (_p(raw), w, h, w, ctypes.c_float(black), ctypes.c_float(white), int(bayer), g, int(rotate_180), cx, pm, nlf)
    if reference:
        if ref_lib() is None:
            raise FileNotFoundError(REF_PATH)
        rc = ref_lib().ref_estimate_raw_parameters(*args)
    else:
        rc = lib().oracle_estimate_raw_parameters(*args)
    if rc != 0:
        raise ValueError("estimateRawParameters failed (%d)" % rc)
    return np.array(cx[:], np.float32).reshape(3, 3), np.array(pm[:], np.float32), np.array(nlf[:], np.float32)


# ---- host colour math ----

def _m9(fn, *mats):
    args = [_arr(np.ravel(m), 9) for m in mats]
    out = (ctypes.c_float * 9)()
    fn(*args, out)
    return np.array(out[:], np.float32).reshape(3, 3)


def cam_xyz_coeff(cam_xyz):
    pre = (ctypes.c_float * 3)()
    out = (ctypes.c_float * 9)()
    lib().oracle_cam_xyz_coeff(_arr(np.ravel(cam_xyz), 9), pre, out)
    return np.array(pre[:], np.float32), np.array(out[:], np.float32).reshape(3, 3)


def cam_ycbcr(rgb_cam):
    return _m9(lib().oracle_cam_ycbcr, rgb_cam)


def inverse3x3(m):
    return _m9(lib().oracle_inverse3x3, m)


def matmul3x3(a, b):
    return _m9(lib().oracle_matmul3x3, a, b)


def atan2pi(y, x):
    return lib().oracle_atan2pi(y, x)


# ---- the reference's own kernel file (demosaic.cl) run on the CPU through oracle/clref ----
# (built by `make -C oracle clref` where the reference sources are; a checker of this
# oracle's restatement, never of the product directly)
CLREF_PATH = os.path.join(HERE, "_ref", "libclref.so")
_clref = None


def clref_lib():
    """The reference's demosaic.cl compiled as C++ against oracle/clref/cl_shim.h, or None."""
    global _clref
    if _clref is None and os.path.exists(CLREF_PATH):
        _clref = ctypes.CDLL(CLREF_PATH)
    return _clref


def _clref_call(name, *args):
    if clref_lib() is None:
        raise FileNotFoundError(CLREF_PATH)
    rc = getattr(clref_lib(), name)(*args)
    if rc != 0:
        raise ValueError("%s: a vector condition had components that disagree" % name)


def clref_scale_raw(raw, bayer, scale_mul, black_norm):
    raw = np.ascontiguousarray(raw, dtype=np.uint16)
    h, w = raw.shape
    out = np.zeros((h, w), np.float32)
    _clref_call("clref_scale_raw", _p(raw), w, h, bayer, _arr(scale_mul, 4), ctypes.c_float(black_norm), _p(out))
    return out


def clref_interpolate_green(scaled, bayer, luma_variance):
    s = _f32(scaled)
    h, w = s.shape
    out = np.zeros((h, w), np.float32)
    _clref_call("clref_interpolate_green", _p(s), w, h, bayer, ctypes.c_float(luma_variance), _p(out))
    return out


def clref_interpolate_red_blue(scaled, green, bayer, chroma_variance, rotate_180=False):
    s, g = _f32(scaled), _f32(green)
    h, w = s.shape
    out = np.zeros((h, w, 4), np.float32)  # the rotation leaves row 0 and column 0 as they are: zero
    _clref_call("clref_interpolate_red_blue", _p(s), _p(g), w, h, bayer, ctypes.c_float(chroma_variance),
                int(bool(rotate_180)), _p(out))
    return out


def clref_blend_highlights(img, clip=1.0):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_blend_highlights", _p(a), w, h, ctypes.c_float(clip), _p(out))
    return out


def clref_transform(img, m):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_transform", _p(a), w, h, _arr(np.ravel(m), 9), _p(out))
    return out


def clref_noise_statistics(img):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_noise_statistics", _p(a), w, h, _p(out))
    return out


def clref_raw_noise_statistics(scaled, bayer):
    s = _f32(scaled)
    h, w = s.shape
    mean = np.zeros((h // 2, w // 2, 4), np.float32)
    var = np.zeros((h // 2, w // 2, 4), np.float32)
    _clref_call("clref_raw_noise_statistics", _p(s), w, h, bayer, _p(mean), _p(var))
    return mean, var


def clref_denoise_bilateral(img, var_a, var_b, chroma_boost, gradient_boost):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_denoise_bilateral", _p(a), w, h, _arr(var_a, 3), _arr(var_b, 3), ctypes.c_float(chroma_boost),
                ctypes.c_float(gradient_boost), _p(out))
    return out


def clref_downsample(img, ow, oh):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros((oh, ow, 4), np.float32)
    _clref_call("clref_downsample", _p(a), w, h, ow, oh, _p(out))
    return out


def clref_reassemble(den0, img1, den1, sharpening, nlf):
    d0, i1, d1 = _f32(den0), _f32(img1), _f32(den1)
    h, w, _ = d0.shape
    h1, w1, _ = i1.shape
    out = np.zeros_like(d0)
    _clref_call("clref_reassemble", _p(d0), w, h, _p(i1), _p(d1), w1, h1, ctypes.c_float(sharpening), _arr(nlf, 2),
                _p(out))
    return out


def clref_ltm_mask(img, guide, ltm, m):
    """ltm: (guidedFilterEps, shadows, highlights, detail)."""
    a, g = _f32(img), _f32(guide)
    h, w, _ = a.shape
    gh, gw, _ = g.shape
    out = np.zeros((h, w), np.float32)
    _clref_call("clref_ltm_mask", _p(a), w, h, _p(g), gw, gh, _arr(ltm, 4), _arr(np.ravel(m), 9), _p(out))
    return out


def clref_convert_to_srgb(img, mask, m, rgb, local_tone_mapping, out_u8=True):
    """rgb: (contrast, saturation, toneCurveSlope, exposureBias, blacks)."""
    a, mk = _f32(img), _f32(mask)
    h, w, _ = a.shape
    if out_u8:
        out = np.zeros((h, w, 4), np.uint8)
        _clref_call("clref_convert_to_srgb", _p(a), _p(mk), w, h, _arr(np.ravel(m), 9), _arr(rgb, 5),
                    int(local_tone_mapping), _p(out), None)
    else:
        out = np.zeros((h, w, 4), np.float32)
        _clref_call("clref_convert_to_srgb", _p(a), _p(mk), w, h, _arr(np.ravel(m), 9), _arr(rgb, 5),
                    int(local_tone_mapping), None, _p(out))
    return out


def clref_fast_debayer(scaled, bayer):
    s = _f32(scaled)
    h, w = s.shape
    out = np.zeros((h // 2, w // 2, 4), np.float32)
    _clref_call("clref_fast_debayer", _p(s), w, h, bayer, _p(out))
    return out


def clref_bayer_to_rgba(scaled, bayer):
    s = _f32(scaled)
    h, w = s.shape
    out = np.zeros((h // 2, w // 2, 4), np.float32)
    _clref_call("clref_bayer_to_rgba", _p(s), w, h, bayer, _p(out))
    return out


def clref_rgba_to_bayer(rgba, bayer):
    a = _f32(rgba)
    qh, qw, _ = a.shape
    out = np.zeros((2 * qh, 2 * qw), np.float32)
    _clref_call("clref_rgba_to_bayer", _p(a), qw, qh, bayer, _p(out))
    return out


def clref_denoise_rgba(img, raw_variance):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_denoise_rgba", _p(a), w, h, _arr(raw_variance, 4), _p(out))
    return out


def clref_denoise_guided(img, var_a, var_b):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_denoise_guided", _p(a), w, h, _arr(var_a, 3), _arr(var_b, 3), _p(out))
    return out


def clref_despeckle(img, var_a, var_b):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_despeckle", _p(a), w, h, _arr(var_a, 3), _arr(var_b, 3), _p(out))
    return out


def clref_despeckle_rgba(img):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_despeckle_rgba", _p(a), w, h, _p(out))
    return out


def clref_guided_filter(img, filter_size, eps):
    a = _f32(img)
    h, w, _ = a.shape
    out = np.zeros_like(a)
    _clref_call("clref_guided_filter", _p(a), w, h, int(filter_size), _arr(eps, 3), _p(out))
    return out


# ---- the reference's own noise-model regressions (pyramidal_denoise.cpp) on given statistics ----
REGRESS_PATH = os.path.join(HERE, "_ref", "libref_regress.so")
_regress = None


def ref_regress_lib():
    """computeRawNoiseStatistics / computeNoiseStatistics compiled from the reference's source, or None."""
    global _regress
    if _regress is None and os.path.exists(REGRESS_PATH):
        _regress = ctypes.CDLL(REGRESS_PATH, mode=os.RTLD_LAZY)
    return _regress


def ref_regress_raw(mean, var):
    """computeRawNoiseStatistics' fit on quad statistics (h/2, w/2, 4): A0..A3, B0..B3."""
    m, v = _f32(mean), _f32(var)
    qh, qw, _ = m.shape
    out = np.zeros(8, np.float32)
    ref_regress_lib().ref_regress_raw(_p(m), _p(v), 2 * qw, 2 * qh, _p(out))
    return out


def ref_regress_level(stats):
    """computeNoiseStatistics' fit on a noiseStatistics image (h, w, 4): A0..A2, B0..B2."""
    s = _f32(stats)
    h, w, _ = s.shape
    out = np.zeros(6, np.float32)
    ref_regress_lib().ref_regress_level(_p(s), w, h, _p(out))
    return out


# ---- the reference's own RawConverter::demosaicImage, run on the CPU (oracle/clref/ref_pipeline.cpp) ----
PIPELINE_PATHS = {F32: os.path.join(HERE, "_ref", "libref_pipeline.so"),
                  F16: os.path.join(HERE, "_ref", "libref_pipeline16.so")}
_pipelines = {}


def ref_pipeline_lib(prec=F32):
    """The reference's RawConverter built with fp32 image storage (prec F32) or with the fp16
    storage it ships with (F16), or None."""
    if prec not in _pipelines and os.path.exists(PIPELINE_PATHS[prec]):
        _pipelines[prec] = ctypes.CDLL(PIPELINE_PATHS[prec], mode=os.RTLD_LAZY)
    return _pipelines.get(prec)


def ref_raw_converter(raw, spec, prec=F32, rotate_180=False):
    """The reference's RawConverter::demosaicImage (5 pyramid levels, bilateral denoiser) on a
    uint16 frame with a spec dict (climage_gb300.configs.make_spec): (RGBA8, raw NLF (4,),
    pyramid NLF (5, 6)); prec selects the image storage it was built with, rotate_180 its
    last argument (a converter made for the call: its images start at zero)."""
    raw = np.ascontiguousarray(raw, np.uint16)
    h, w = raw.shape
    p = [spec["black_level"], spec["white_level"], spec["exposure_multiplier"], spec["noise_level"]]
    p += list(spec["scale_mul"]) + list(spec["rgb_cam"]) + list(spec["raw_nlf"])
    for row in spec["pyramid_nlf"]:
        p += list(row)
    for d in spec["denoise"]:
        p += [d["luma"], d["chroma"], d["chromaBoost"], d["gradientBoost"], d["sharpening"]]
    r, l = spec["rgb"], spec["ltm"]
    p += [r["contrast"], r["saturation"], r["toneCurveSlope"], r["exposureBias"], r["blacks"]]
    p += [l["guidedFilterEps"], l["shadows"], l["highlights"], l["detail"]]
    params = np.array(p, np.float32)
    out = np.zeros((h, w, 4), np.uint8)
    rn, pn = np.zeros(4, np.float32), np.zeros(30, np.float32)
    rc = ref_pipeline_lib(prec).ref_raw_converter(_p(raw), w, h, int(spec["bayer_pattern"]), _p(params),
                                              int(r["localToneMapping"]), int(bool(rotate_180)), _p(out), _p(rn),
                                              _p(pn))
    if rc != 0:
        raise ValueError("ref_raw_converter: a vector condition had components that disagree")
    return out, rn, pn.reshape(5, 6)
