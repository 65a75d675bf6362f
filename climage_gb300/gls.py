"""ctypes bindings of libgls_cuda.so (include/gls_cuda.h) and a thin Python mirror of the
reference's operator surface (demosaic_cl.hpp free functions, RawConverter).

Device images are torch CUDA tensors: (H, W) for single-channel images, (H, W, 4) for
RGBA, with dtype uint16 (raw), float32/float16 (storage precision) or uint8 (RGBA8).
PyTorch only supplies device memory and the stream; every pixel is computed by the CUDA
kernels of libgls_cuda.  There is no CPU fallback: without the built library every call
raises.
"""
import ctypes
import weakref
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgls_cuda.so")

GLS_OK = 0
GLS_ERR_INVALID_ARGUMENT = 1
GLS_ERR_INVALID_SIZE = 2
GLS_ERR_UNSUPPORTED = 3
GLS_ERR_CUDA = 4
GLS_ERR_OUT_OF_MEMORY = 5
GLS_ERR_TIMEOUT = 6
GLS_ERR_FORMAT = 7
GLS_ERR_BAD_STREAM = 8
# image size limit of Context.guidedFilterNoAlloc (gls_cuda.h)
GUIDED_FILTER_NOALLOC_MAX_PIXELS = 116490
STATUS = {0: "ok", 1: "invalid argument", 2: "invalid size", 3: "unsupported", 4: "CUDA error",
          5: "out of memory", 6: "timeout", 7: "unsupported pixel format", 8: "malformed compressed stream"}

R16_UNORM, R_F32, R_F16, RGBA_F32, RGBA_F16, RGBA8_UNORM, RGB8_UNORM = range(7)
GRBG, GBRG, RGGB, BGGR = range(4)
BILATERAL, GUIDED_FAST, GUIDED_PRECISE = range(3)
STORAGE_F32, STORAGE_F16, STORAGE_F16_STATS = 0, 1, 2
MAX_LEVELS = 8


class GlsError(RuntimeError):
    def __init__(self, status, what, detail=""):
        super().__init__("%s failed: %s%s" % (what, STATUS.get(status, status), (" (%s)" % detail) if detail else ""))
        self.status = status


class LjpegInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("width", "height", "components", "precision", "predictor",
                                            "point_transform", "restart_interval", "tables_alike")]


class ImageDesc(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("stride_bytes", ctypes.c_int), ("format", ctypes.c_int)]


class DenoiseParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("luma", "chroma", "chromaBoost", "gradientBoost", "sharpening")]


class RGBConversionParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("contrast", "saturation", "toneCurveSlope", "exposureBias", "blacks")] + [
        ("localToneMapping", ctypes.c_int)]


class LTMParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("guidedFilterEps", "shadows", "highlights", "detail")]


class DemosaicParams(ctypes.Structure):
    _fields_ = [
        ("bayer_pattern", ctypes.c_int),
        ("black_level", ctypes.c_float),
        ("white_level", ctypes.c_float),
        ("exposure_multiplier", ctypes.c_float),
        ("scale_mul", ctypes.c_float * 4),
        ("rgb_cam", ctypes.c_float * 9),
        ("raw_nlf", ctypes.c_float * 4),
        ("pyramid_nlf", (ctypes.c_float * 6) * MAX_LEVELS),
        ("denoise", DenoiseParams * MAX_LEVELS),
        ("noise_level", ctypes.c_float),
        ("rgb_conversion", RGBConversionParams),
        ("ltm", LTMParams),
        ("pyramid_levels", ctypes.c_int),
        ("denoise_algorithm", ctypes.c_int),
        ("storage", ctypes.c_int),
        ("rotate_180", ctypes.c_int),
    ]


_lib = None

# (name, restype, argtypes) of every entry point declared in include/gls_cuda.h
_P = ctypes.c_void_p
_D = ctypes.POINTER(ImageDesc)
_F = ctypes.c_float
_I = ctypes.c_int
_FP = ctypes.POINTER(ctypes.c_float)
SIGNATURES = [
    ("gls_ctx_create", _I, [_I, ctypes.POINTER(_P)]),
    ("gls_ctx_destroy", _I, [_P]),
    ("gls_ctx_set_stream", _I, [_P, _P]),
    ("gls_ctx_synchronize", _I, [_P]),
    ("gls_status_string", ctypes.c_char_p, [_I]),
    ("gls_ctx_last_error", ctypes.c_char_p, [_P]),
    ("gls_ctx_kernel_launches", ctypes.c_uint64, [_P]),
    ("gls_version", ctypes.c_char_p, []),
    ("gls_scale_raw_data", _I, [_P, _D, _D, _I, _FP, _F]),
    ("gls_raw_noise_statistics", _I, [_P, _D, _I, _D, _D]),
    ("gls_compute_raw_noise_statistics", _I, [_P, _D, _I, _FP]),
    ("gls_interpolate_green", _I, [_P, _D, _D, _I, _F]),
    ("gls_interpolate_red_blue", _I, [_P, _D, _D, _D, _I, _F, _I]),
    ("gls_fast_debayer", _I, [_P, _D, _D, _I]),
    ("gls_blend_highlights", _I, [_P, _D, _F, _D]),
    ("gls_transform_image", _I, [_P, _D, _D, _FP]),
    ("gls_despeckle_image", _I, [_P, _D, _FP, _FP, _D]),
    ("gls_downsample_image", _I, [_P, _D, _D]),
    ("gls_noise_statistics", _I, [_P, _D, _D]),
    ("gls_compute_noise_statistics", _I, [_P, _D, _FP]),
    ("gls_denoise_image", _I, [_P, _D, _FP, _FP, _F, _F, _D]),
    ("gls_denoise_image_guided", _I, [_P, _D, _FP, _FP, _D]),
    ("gls_guided_filter", _I, [_P, _D, _I, _FP, _D]),
    ("gls_guided_filter_noalloc", _I, [_P, _D, _I, _FP, _D]),
    ("gls_reassemble_image", _I, [_P, _D, _D, _D, _F, _FP, _D]),
    ("gls_local_tone_mapping_mask", _I, [_P, _D, _D, ctypes.POINTER(LTMParams), _FP, _D]),
    ("gls_convert_to_srgb", _I, [_P, _D, _D, _D, _FP, ctypes.POINTER(RGBConversionParams)]),
    ("gls_bayer_to_raw_rgba", _I, [_P, _D, _D, _I]),
    ("gls_raw_rgba_to_bayer", _I, [_P, _D, _D, _I]),
    ("gls_despeckle_raw_rgba", _I, [_P, _D, _D]),
    ("gls_denoise_raw_rgba", _I, [_P, _D, _FP, _D]),
    ("gls_unpack_raw_bits", _I, [_P, _P, ctypes.c_size_t, _I, _P, ctypes.c_size_t]),
    ("gls_auto_white_balance", _I, [_P, _D, _FP, _FP, _F, _F, _I, _FP, _FP]),
    ("gls_dng_decode_lossless_jpeg", _I, [_P, _P, ctypes.c_size_t, _I, ctypes.POINTER(ctypes.c_uint64),
                                          ctypes.POINTER(ctypes.c_uint64), _I, _I, _D]),
    ("gls_lossless_jpeg_info", _I, [_P, ctypes.c_size_t, ctypes.POINTER(LjpegInfo)]),
    ("gls_fit_color_checker", _I, [_FP, _FP, _FP, _FP, _FP]),
    ("gls_color_checker_raw_stats", _I, [_P, _D, _F, _F, _I, ctypes.POINTER(ctypes.c_int), _I, _FP, _FP]),
    ("gls_estimate_raw_parameters", _I, [_P, _D, _F, _F, _I, ctypes.POINTER(ctypes.c_int), _I, _FP, _FP, _FP]),
    ("gls_selftest", _I, [_P, ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    ("gls_selftest_reciprocal", _I, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    ("gls_cam_xyz_coeff", _I, [_FP, _FP, _FP]),
    ("gls_cam_ycbcr", _I, [_FP, _FP]),
    ("gls_inverse3x3", _I, [_FP, _FP]),
    ("gls_raw_converter_create", _I, [_P, ctypes.POINTER(_P)]),
    ("gls_raw_converter_destroy", _I, [_P]),
    ("gls_raw_converter_demosaic", _I, [_P, _D, ctypes.POINTER(DemosaicParams), _D, _I]),
    ("gls_raw_converter_noise_model", _I, [_P, ctypes.POINTER(DemosaicParams)]),
    ("gls_raw_converter_status", _I, [_P]),
    ("gls_raw_converter_wait_probe", _I, [_P, ctypes.c_uint]),
    ("gls_raw_converter_demosaic_host", _I, [_P, _P, _I, _I, _I, ctypes.POINTER(DemosaicParams), _P, _I]),
    ("gls_raw_converter_demosaic_packed_host", _I, [_P, _P, ctypes.c_size_t, _I, _I, _I,
                                                    ctypes.POINTER(DemosaicParams), _P, _I]),
    ("gls_raw_batch_demosaic_packed_host", _I, [_P, _I, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_size_t),
                                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(DemosaicParams),
                                                ctypes.POINTER(_P), _I]),
    ("gls_raw_converter_fast_demosaic", _I, [_P, _D, ctypes.POINTER(DemosaicParams), _D]),
    ("gls_raw_converter_set_tap", _I, [_P, _I, _D]),
    ("gls_raw_converter_set_mode", _I, [_P, _I]),
    ("gls_raw_converter_profile", _I, [_P, _I]),
    ("gls_raw_converter_profile_report", _I, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    ("gls_raw_converter_set_cnn", _I, [_P, _P]),
    ("gls_raw_converter_cnn_input", _I, [_P, _D, ctypes.POINTER(DemosaicParams), _D]),
    ("gls_raw_batch_set_cnn", _I, [_P, _P]),
    ("gls_raw_batch_create", _I, [_P, _I, ctypes.POINTER(_P)]),
    ("gls_raw_batch_destroy", _I, [_P]),
    ("gls_raw_batch_reserve", _I, [_P, _I, _I, _I, _I]),
    ("gls_raw_batch_demosaic", _I, [_P, _I, _D, ctypes.POINTER(DemosaicParams), _D]),
    ("gls_raw_batch_demosaic_host", _I, [_P, _I, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(DemosaicParams), ctypes.POINTER(_P), _I]),
    ("gls_cnn_create", _I, [_P, ctypes.POINTER(_P)]),
    ("gls_cnn_destroy", _I, [_P]),
    ("gls_cnn_param_count", _I, []),
    ("gls_cnn_set_params", _I, [_P, _FP, _I]),
    ("gls_cnn_get_params", _I, [_P, _FP, _I]),
    ("gls_cnn_get_grads", _I, [_P, _FP, _I]),
    ("gls_cnn_forward", _I, [_P, _P, _I, _I, _I, _P]),
    ("gls_cnn_set_backend", _I, [_P, _I]),
    ("gls_cnn_get_backend", _I, [_P]),
    ("gls_cnn_status", _I, [_P]),
    ("gls_cnn_wait_probe", _I, [_P, ctypes.c_uint]),
    ("gls_cnn_train_step", _I, [_P, _P, _P, _I, _I, _I, _F, _FP]),
    ("gls_raw_batch_plan", _I, [_I, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _I,
                                ctypes.POINTER(ctypes.c_int)]),
    ("gls_tune_force", _I, [_I, _I]),
    ("gls_tune_reset", _I, []),
    ("gls_tune_count", _I, []),
    ("gls_tune_entry", _I, [_I, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                            ctypes.POINTER(ctypes.c_int), _FP]),
]

# launch-shape tuner: kernels and their compiled tile shapes (gls_tune_force / gls_tune_entry)
TUNE_DEMOSAIC, TUNE_FINAL = 0, 1
TUNE_SHAPES = {TUNE_DEMOSAIC: ("44x28", "32x24", "64x32", "split"), TUNE_FINAL: ("32x24", "32x16", "64x16")}


def lib():
    """Loads libgls_cuda.so; raises when it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgls_cuda.so is not built: run climage_gb300.build.build() (nvcc, sm_103a)")
        l = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def farr(vals, n=None):
    vals = [float(v) for v in np.ravel(vals)]
    n = len(vals) if n is None else n
    return (ctypes.c_float * n)(*vals)


# ---- host colour math (no GPU needed) ----

def cam_xyz_coeff(cam_xyz):
    pre, out = (ctypes.c_float * 3)(), (ctypes.c_float * 9)()
    s = lib().gls_cam_xyz_coeff(farr(cam_xyz, 9), pre, out)
    if s != GLS_OK:
        raise GlsError(s, "cam_xyz_coeff")
    return np.array(pre[:], np.float32), np.array(out[:], np.float32).reshape(3, 3)


def cam_ycbcr(rgb_cam):
    out = (ctypes.c_float * 9)()
    lib().gls_cam_ycbcr(farr(rgb_cam, 9), out)
    return np.array(out[:], np.float32).reshape(3, 3)


def inverse3x3(m):
    out = (ctypes.c_float * 9)()
    s = lib().gls_inverse3x3(farr(m, 9), out)
    if s != GLS_OK:
        raise GlsError(s, "inverse3x3")
    return np.array(out[:], np.float32).reshape(3, 3)


def lossless_jpeg_info(data):
    """The header of one lossless-JPEG stream (bytes or a uint8 array), as the DNG decoder reads
    it: a dict of width, height, components, precision, predictor, point_transform,
    restart_interval and tables_alike.  Host only; raises GlsError for a header the decoder
    rejects."""
    buf = np.frombuffer(bytes(data), np.uint8) if isinstance(data, (bytes, bytearray)) else np.ascontiguousarray(data, np.uint8)
    info = LjpegInfo()
    s = lib().gls_lossless_jpeg_info(ctypes.c_void_p(buf.ctypes.data), buf.size, ctypes.byref(info))
    if s != GLS_OK:
        raise GlsError(s, "lossless_jpeg_info")
    return {n: getattr(info, n) for n, _ in LjpegInfo._fields_}


def fit_color_checker(mean, var):
    """The fit half of estimateRawParameters from colorCheckerRawStats' (mean, var), each (24, 4):
    (cam_xyz (3, 3), pre_mul (3,), raw NLF slopes (4,)).  Host only."""
    cx, pm, nlf = (ctypes.c_float * 9)(), (ctypes.c_float * 3)(), (ctypes.c_float * 4)()
    s = lib().gls_fit_color_checker(farr(np.ravel(mean), 96), farr(np.ravel(var), 96), cx, pm, nlf)
    if s != GLS_OK:
        raise GlsError(s, "fit_color_checker")
    return (np.array(cx[:], np.float32).reshape(3, 3), np.array(pm[:], np.float32), np.array(nlf[:], np.float32))


# ---- device images ----

def _fmt_of(t, channels):
    import torch
    if t.dtype == torch.uint16:
        return R16_UNORM
    if t.dtype == torch.uint8:
        return RGBA8_UNORM if channels == 4 else RGB8_UNORM
    if t.dtype == torch.float32:
        return R_F32 if channels == 1 else RGBA_F32
    if t.dtype == torch.float16:
        return R_F16 if channels == 1 else RGBA_F16
    raise TypeError("unsupported tensor dtype %s" % t.dtype)


def desc(t):
    """gls_image_desc of a contiguous (H, W) or (H, W, C) CUDA tensor."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("device images must be CUDA tensors")
    if t.dim() == 2:
        h, w = t.shape
        c = 1
    elif t.dim() == 3:
        h, w, c = t.shape
    else:
        raise ValueError("images are (H, W) or (H, W, C) tensors")
    if t.stride(-1) != 1 or (t.dim() == 3 and t.stride(1) != c):
        raise ValueError("image rows must be contiguous")
    es = t.element_size()
    return ImageDesc(t.data_ptr(), w, h, t.stride(0) * es, _fmt_of(t, c))


class Context:
    """gls_ctx: one per host thread; launches go to the torch stream current at creation
    unless set_stream is called."""

    def __init__(self, device=0, stream=None):
        import torch
        self._lib = lib()
        self.handle = ctypes.c_void_p()
        s = self._lib.gls_ctx_create(device, ctypes.byref(self.handle))
        if s != GLS_OK:
            raise GlsError(s, "gls_ctx_create")
        # converters and batches made on this context: closed before it, whatever the order
        # in which Python finalises them
        self._children = weakref.WeakSet()
        self.set_stream(stream if stream is not None else torch.cuda.current_stream(device))

    def set_stream(self, stream):
        self.stream = stream
        self._lib.gls_ctx_set_stream(self.handle, ctypes.c_void_p(stream.cuda_stream))

    def check(self, status, what):
        if status != GLS_OK:
            raise GlsError(status, what, self._lib.gls_ctx_last_error(self.handle).decode())

    def synchronize(self):
        self.check(self._lib.gls_ctx_synchronize(self.handle), "synchronize")

    def selftest_reciprocal(self):
        """Divisors of the shared-divisor range whose fast reciprocal differs from __frcp_rn."""
        m = ctypes.c_uint64()
        self.check(lib().gls_selftest_reciprocal(self.handle, ctypes.byref(m)), "selftest_reciprocal")
        return m.value

    def selftest(self, n=1 << 24, seed=1):
        out = (ctypes.c_uint64 * 4)()
        self.check(self._lib.gls_selftest(self.handle, int(n), int(seed), out), "selftest")
        return [int(v) for v in out]

    def kernel_launches(self):
        return int(self._lib.gls_ctx_kernel_launches(self.handle))

    def close(self):
        if self.handle:
            for child in list(getattr(self, "_children", ())):
                child.close()
            self._lib.gls_ctx_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- stages (demosaic_cl.hpp) ----
    def scaleRawData(self, raw, scaled, bayer, scale_mul, black_level):
        self.check(self._lib.gls_scale_raw_data(self.handle, desc(raw), desc(scaled), bayer, farr(scale_mul, 4),
                                                float(black_level)), "scaleRawData")

    def rawNoiseStatistics(self, scaled, bayer, mean, var):
        self.check(self._lib.gls_raw_noise_statistics(self.handle, desc(scaled), bayer, desc(mean), desc(var)),
                   "rawNoiseStatistics")

    def computeRawNoiseStatistics(self, scaled, bayer):
        out = (ctypes.c_float * 8)()
        self.check(self._lib.gls_compute_raw_noise_statistics(self.handle, desc(scaled), bayer, out),
                   "computeRawNoiseStatistics")
        return np.array(out[:], np.float32)

    def autoWhiteBalance(self, raw, rgb_ycbcr, scale_mul, white, black, bayer):
        """autoWhiteBalance over a raw uint16 device tensor: (gains (3,) with green 1,
        highlight fraction)."""
        wb = (ctypes.c_float * 3)()
        hl = ctypes.c_float()
        self.check(self._lib.gls_auto_white_balance(self.handle, desc(raw), farr(rgb_ycbcr, 9),
                                                    farr(scale_mul, 4), float(white), float(black), int(bayer), wb,
                                                    ctypes.byref(hl)), "autoWhiteBalance")
        return np.array(wb[:], np.float32), np.float32(hl.value)

    def decodeLosslessJPEG(self, data, offsets, sizes, tile_width, tile_height, out):
        """Lossless-JPEG tiles (or one strip) of a DNG image: data is a host uint8 array (or
        bytes) holding the streams at offsets/sizes; out is the (H, W) uint16 device image."""
        buf = np.ascontiguousarray(np.frombuffer(data, np.uint8) if isinstance(data, (bytes, bytearray))
                                   else data, np.uint8)
        n = len(offsets)
        offs = (ctypes.c_uint64 * n)(*[int(o) for o in offsets])
        lens = (ctypes.c_uint64 * n)(*[int(v) for v in sizes])
        self.check(self._lib.gls_dng_decode_lossless_jpeg(self.handle, ctypes.c_void_p(buf.ctypes.data), buf.size, n,
                                                          offs, lens, int(tile_width), int(tile_height), desc(out)),
                   "decodeLosslessJPEG")

    def colorCheckerRawStats(self, raw, black, white, bayer, gmb, rotate_180=False):
        """(mean (24, 4), var (24, 4)) of the CFA channels per chart patch; gmb = (x, y, w, h)."""
        mean, var = (ctypes.c_float * 96)(), (ctypes.c_float * 96)()
        self.check(self._lib.gls_color_checker_raw_stats(self.handle, desc(raw), float(black), float(white), int(bayer),
                                                         (ctypes.c_int * 4)(*gmb), int(rotate_180), mean, var),
                   "colorCheckerRawStats")
        return np.array(mean[:], np.float32).reshape(24, 4), np.array(var[:], np.float32).reshape(24, 4)

    def estimateRawParameters(self, raw, black, white, bayer, gmb, rotate_180=False):
        """(cam_xyz (3, 3), pre_mul (3,), raw NLF slopes (4,)) from a ColorChecker chart."""
        cx, pm, nlf = (ctypes.c_float * 9)(), (ctypes.c_float * 3)(), (ctypes.c_float * 4)()
        self.check(self._lib.gls_estimate_raw_parameters(self.handle, desc(raw), float(black), float(white), int(bayer),
                                                         (ctypes.c_int * 4)(*gmb), int(rotate_180), cx, pm, nlf),
                   "estimateRawParameters")
        return np.array(cx[:], np.float32).reshape(3, 3), np.array(pm[:], np.float32), np.array(nlf[:], np.float32)

    def interpolateGreen(self, scaled, green, bayer, luma_variance):
        self.check(self._lib.gls_interpolate_green(self.handle, desc(scaled), desc(green), bayer, float(luma_variance)),
                   "interpolateGreen")

    def interpolateRedBlue(self, scaled, green, rgb, bayer, chroma_variance, rotate_180=False):
        self.check(self._lib.gls_interpolate_red_blue(self.handle, desc(scaled), desc(green), desc(rgb), bayer,
                                                      float(chroma_variance), int(rotate_180)), "interpolateRedBlue")

    def fastDebayer(self, scaled, rgb, bayer):
        self.check(self._lib.gls_fast_debayer(self.handle, desc(scaled), desc(rgb), bayer), "fastDebayer")

    def blendHighlightsImage(self, inp, clip, out):
        self.check(self._lib.gls_blend_highlights(self.handle, desc(inp), float(clip), desc(out)), "blendHighlights")

    def transformImage(self, inp, out, transform):
        self.check(self._lib.gls_transform_image(self.handle, desc(inp), desc(out), farr(transform, 9)),
                   "transformImage")

    def despeckleImage(self, inp, var_a, var_b, out):
        self.check(self._lib.gls_despeckle_image(self.handle, desc(inp), farr(var_a, 3), farr(var_b, 3), desc(out)),
                   "despeckleImage")

    def downsampleImage(self, inp, out):
        self.check(self._lib.gls_downsample_image(self.handle, desc(inp), desc(out)), "downsampleImage")

    def noiseStatistics(self, inp, out):
        self.check(self._lib.gls_noise_statistics(self.handle, desc(inp), desc(out)), "noiseStatistics")

    def computeNoiseStatistics(self, inp):
        out = (ctypes.c_float * 6)()
        self.check(self._lib.gls_compute_noise_statistics(self.handle, desc(inp), out), "computeNoiseStatistics")
        return np.array(out[:], np.float32)

    def denoiseImage(self, inp, var_a, var_b, chroma_boost, gradient_boost, out):
        self.check(self._lib.gls_denoise_image(self.handle, desc(inp), farr(var_a, 3), farr(var_b, 3),
                                               float(chroma_boost), float(gradient_boost), desc(out)), "denoiseImage")

    def denoiseImageGuided(self, inp, var_a, var_b, out):
        self.check(self._lib.gls_denoise_image_guided(self.handle, desc(inp), farr(var_a, 3), farr(var_b, 3),
                                                      desc(out)), "denoiseImageGuided")

    def guidedFilter(self, inp, filter_size, eps, out):
        self.check(self._lib.gls_guided_filter(self.handle, desc(inp), int(filter_size), farr(eps, 3), desc(out)),
                   "GuidedFilter::filter")

    def guidedFilterNoAlloc(self, inp, filter_size, eps, out):
        """guidedFilter over the library's static scratch: allocates nothing, images of at
        most GUIDED_FILTER_NOALLOC_MAX_PIXELS pixels; overlapping calls race."""
        self.check(self._lib.gls_guided_filter_noalloc(self.handle, desc(inp), int(filter_size), farr(eps, 3),
                                                        desc(out)), "GuidedFilter::filter (no allocation)")

    def reassembleImage(self, den0, img1, den1, sharpening, nlf, out):
        self.check(self._lib.gls_reassemble_image(self.handle, desc(den0), desc(img1), desc(den1), float(sharpening),
                                                  farr(nlf, 2), desc(out)), "reassembleImage")

    def localToneMappingMask(self, inp, guide, ltm, transform, out):
        self.check(self._lib.gls_local_tone_mapping_mask(self.handle, desc(inp), desc(guide), ctypes.byref(ltm),
                                                         farr(transform, 9), desc(out)), "localToneMappingMask")

    def convertTosRGB(self, linear, ltm_mask, out, rgb_cam, params):
        self.check(self._lib.gls_convert_to_srgb(self.handle, desc(linear), desc(ltm_mask), desc(out),
                                                 farr(rgb_cam, 9), ctypes.byref(params)), "convertTosRGB")

    def bayerToRawRGBA(self, raw, rgba, bayer):
        self.check(self._lib.gls_bayer_to_raw_rgba(self.handle, desc(raw), desc(rgba), bayer), "bayerToRawRGBA")

    def rawRGBAToBayer(self, rgba, raw, bayer):
        self.check(self._lib.gls_raw_rgba_to_bayer(self.handle, desc(rgba), desc(raw), bayer), "rawRGBAToBayer")

    def despeckleRawRGBAImage(self, inp, out):
        self.check(self._lib.gls_despeckle_raw_rgba(self.handle, desc(inp), desc(out)), "despeckleRawRGBAImage")

    def denoiseRawRGBAImage(self, inp, raw_variance, out):
        self.check(self._lib.gls_denoise_raw_rgba(self.handle, desc(inp), farr(raw_variance, 4), desc(out)),
                   "denoiseRawRGBAImage")

    def unpackRawBits(self, packed, bits, out):
        n = out.numel()
        self.check(self._lib.gls_unpack_raw_bits(self.handle, ctypes.c_void_p(packed.data_ptr()), packed.numel(),
                                                 int(bits), ctypes.c_void_p(out.data_ptr()), n), "unpackRawBits")


class RawConverter:
    """RawConverter (raw_converter.hpp:22-62) over gls_raw_converter."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.handle = ctypes.c_void_p()
        ctx.check(lib().gls_raw_converter_create(ctx.handle, ctypes.byref(self.handle)), "RawConverter")
        ctx._children.add(self)

    def demosaicImage(self, raw, params, out, defer_noise_model=False):
        """raw: (H, W) uint16 CUDA tensor; out: (H, W, 4) uint8 (RGBA8) or float32 CUDA tensor."""
        self.ctx.check(lib().gls_raw_converter_demosaic(self.handle, desc(raw), ctypes.byref(params), desc(out),
                                                        int(defer_noise_model)), "RawConverter::demosaicImage")
        return out

    def noiseModel(self, params):
        self.ctx.check(lib().gls_raw_converter_noise_model(self.handle, ctypes.byref(params)), "noiseModel")

    def status(self):
        """Raises GLS_ERR_TIMEOUT (once) when a bounded wait of the statistics kernels ran out
        since the last call."""
        self.ctx.check(lib().gls_raw_converter_status(self.handle), "RawConverter.status")

    def wait_probe(self, polls):
        """Makes both bounded waits of the statistics kernels run out (after one converted frame)."""
        self.ctx.check(lib().gls_raw_converter_wait_probe(self.handle, int(polls)), "RawConverter.wait_probe")

    def demosaicImageHost(self, raw, params, out):
        """raw: (H, W) uint16 numpy array (ideally pinned); out: (H, W, 3|4) uint8 numpy array."""
        h, w = raw.shape
        ch = out.shape[2]
        self.ctx.check(lib().gls_raw_converter_demosaic_host(
            self.handle, ctypes.c_void_p(raw.ctypes.data), w, h, raw.strides[0] // 2, ctypes.byref(params),
            ctypes.c_void_p(out.ctypes.data), ch), "demosaicImage (host buffers)")
        return out

    def demosaicImagePackedHost(self, packed, bits, w, h, params, out):
        """packed: uint8 numpy array (ideally pinned) holding the w x h samples as one MSB-first
        stream of `bits`-bit samples; out: (H, W, 3|4) uint8 numpy array."""
        packed = np.frombuffer(packed, np.uint8) if isinstance(packed, (bytes, bytearray)) else packed
        ch = out.shape[2]
        self.ctx.check(lib().gls_raw_converter_demosaic_packed_host(
            self.handle, ctypes.c_void_p(packed.ctypes.data), packed.size, int(bits), int(w), int(h),
            ctypes.byref(params), ctypes.c_void_p(out.ctypes.data), ch), "demosaicImage (packed host buffers)")
        return out

    def demosaicImageHostPtr(self, raw_ptr, w, h, params, out_ptr, channels):
        self.ctx.check(lib().gls_raw_converter_demosaic_host(self.handle, ctypes.c_void_p(raw_ptr), w, h, w,
                                                             ctypes.byref(params), ctypes.c_void_p(out_ptr), channels),
                       "demosaicImage (host buffers)")

    def fastDemosaicImage(self, raw, params, out):
        self.ctx.check(lib().gls_raw_converter_fast_demosaic(self.handle, desc(raw), ctypes.byref(params), desc(out)),
                       "RawConverter::fastDemosaicImage")
        return out

    def setMode(self, mode):
        """0: fused tile kernels (default); 1: one kernel per reference stage."""
        self.ctx.check(lib().gls_raw_converter_set_mode(self.handle, int(mode)), "setMode")

    def profile(self, enable=True):
        self.ctx.check(lib().gls_raw_converter_profile(self.handle, int(enable)), "profile")

    def profileReport(self):
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        self.ctx.check(lib().gls_raw_converter_profile_report(self.handle, buf, len(buf)), "profile report")
        return json.loads(buf.value.decode())

    def setCnn(self, cnn):
        """Run the learned stage with (a copy of) this Cnn; None returns to the plain pipeline."""
        self.ctx.check(lib().gls_raw_converter_set_cnn(self.handle, cnn.handle if cnn is not None else None),
                       "RawConverter.setCnn")

    def cnnInput(self, raw, params, out):
        """The learned stage's input (R, G, B, sigma) of a raw frame into out (H, W, 4) float32."""
        self.ctx.check(lib().gls_raw_converter_cnn_input(self.handle, desc(raw), ctypes.byref(params), desc(out)),
                       "RawConverter.cnnInput")
        return out

    def setTap(self, stage, tensor):
        self.ctx.check(lib().gls_raw_converter_set_tap(self.handle, int(stage), desc(tensor)), "setTap")

    def close(self):
        if self.handle:
            lib().gls_raw_converter_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_force(kernel, shape):
    """Pins a kernel's tile shape for every frame size (shape -1: the tuned choice again)."""
    st = lib().gls_tune_force(int(kernel), int(shape))
    if st != 0:
        raise GlsError(st, "gls_tune_force(%d, %d)" % (kernel, shape))


def tune_reset():
    """Forgets every tuned choice and forced shape."""
    lib().gls_tune_reset()


def tune_entries():
    """The tuner's choices: [{kernel, width, height, flags, shape, ms: [best ms per shape]}]."""
    out = []
    for i in range(lib().gls_tune_count()):
        k, w, h, f, sh = (ctypes.c_int() for _ in range(5))
        ms = (ctypes.c_float * 4)()
        if lib().gls_tune_entry(i, ctypes.byref(k), ctypes.byref(w), ctypes.byref(h), ctypes.byref(f),
                                ctypes.byref(sh), ms) != 0:
            break
        n = len(TUNE_SHAPES[k.value])
        out.append(dict(kernel=k.value, width=w.value, height=h.value, flags=f.value, shape=sh.value,
                        ms=[round(float(x), 4) for x in ms[:n]]))
    return out


def batch_plan(sizes, lanes):
    """The lane of each (width, height) frame as gls_raw_batch assigns them."""
    n = len(sizes)
    ws = (ctypes.c_int * max(n, 1))(*[w for w, _ in sizes])
    hs = (ctypes.c_int * max(n, 1))(*[h for _, h in sizes])
    out = (ctypes.c_int * max(n, 1))()
    s = lib().gls_raw_batch_plan(n, ws, hs, int(lanes), out)
    if s != GLS_OK:
        raise GlsError(s, "gls_raw_batch_plan")
    return [int(out[i]) for i in range(n)]


class RawBatch:
    """gls_raw_batch: a burst of frames over `lanes` converters on their own streams, forked
    from and joined back to the context's stream."""

    def __init__(self, ctx, lanes=3):
        self.ctx = ctx
        self.handle = ctypes.c_void_p()
        ctx.check(lib().gls_raw_batch_create(ctx.handle, int(lanes), ctypes.byref(self.handle)), "RawBatch")
        ctx._children.add(self)

    def set_cnn(self, cnn):
        self.ctx.check(lib().gls_raw_batch_set_cnn(self.handle, cnn.handle if cnn is not None else None),
                       "RawBatch.set_cnn")

    def reserve(self, width, height, levels, storage=STORAGE_F32):
        self.ctx.check(lib().gls_raw_batch_reserve(self.handle, int(width), int(height), int(levels), int(storage)),
                       "RawBatch.reserve")

    def demosaic(self, raws, params, outs):
        """raws: (H, W) uint16 CUDA tensors; params: DemosaicParams; outs: (H, W, 4) uint8 or float32."""
        n = len(raws)
        rd = (ImageDesc * max(n, 1))(*[desc(r) for r in raws])
        od = (ImageDesc * max(n, 1))(*[desc(o) for o in outs])
        pa = (DemosaicParams * max(n, 1))(*params)
        self.ctx.check(lib().gls_raw_batch_demosaic(self.handle, n, rd, pa, od), "RawBatch.demosaic")
        return outs

    def demosaic_host_ptr(self, raw_ptrs, sizes, params, out_ptrs, channels=4):
        """Host frames by address (pinned for overlapped copies); sizes: (width, height)."""
        n = len(raw_ptrs)
        rp = (ctypes.c_void_p * max(n, 1))(*raw_ptrs)
        op = (ctypes.c_void_p * max(n, 1))(*out_ptrs)
        ws = (ctypes.c_int * max(n, 1))(*[w for w, _ in sizes])
        hs = (ctypes.c_int * max(n, 1))(*[h for _, h in sizes])
        pa = (DemosaicParams * max(n, 1))(*params)
        self.ctx.check(lib().gls_raw_batch_demosaic_host(self.handle, n, rp, ws, hs, ws, pa, op, int(channels)),
                       "RawBatch.demosaic_host")

    def demosaic_packed_host_ptr(self, packed_ptrs, n_bytes, bits, sizes, params, out_ptrs, channels=4):
        """Packed host frames by address (see RawConverter.demosaicImagePackedHost)."""
        n = len(packed_ptrs)
        pp = (ctypes.c_void_p * max(n, 1))(*packed_ptrs)
        nb = (ctypes.c_size_t * max(n, 1))(*n_bytes)
        bb = (ctypes.c_int * max(n, 1))(*bits)
        op = (ctypes.c_void_p * max(n, 1))(*out_ptrs)
        ws = (ctypes.c_int * max(n, 1))(*[w for w, _ in sizes])
        hs = (ctypes.c_int * max(n, 1))(*[h for _, h in sizes])
        pa = (DemosaicParams * max(n, 1))(*params)
        self.ctx.check(lib().gls_raw_batch_demosaic_packed_host(self.handle, n, pp, nb, bb, ws, hs, pa, op,
                                                                int(channels)), "RawBatch.demosaic_packed_host")

    def close(self):
        if self.handle:
            lib().gls_raw_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# layer shapes of the learned stage: (cin, cout)
CNN_LAYERS = [(4, 32), (32, 32), (32, 32), (32, 32), (32, 4)]


class Cnn:
    """gls_cnn: the learned stage's 5-layer BF16 CNN (forward, training on the GPU)."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.handle = ctypes.c_void_p()
        ctx.check(lib().gls_cnn_create(ctx.handle, ctypes.byref(self.handle)), "Cnn")
        ctx._children.add(self)
        self.nparam = int(lib().gls_cnn_param_count())

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32).ravel()
        self.ctx.check(lib().gls_cnn_set_params(self.handle, p.ctypes.data_as(_FP), p.size), "Cnn.set_params")

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        self.ctx.check(lib().gls_cnn_get_params(self.handle, p.ctypes.data_as(_FP), p.size), "Cnn.params")
        return p

    def grads(self):
        g = np.zeros(self.nparam, np.float32)
        self.ctx.check(lib().gls_cnn_get_grads(self.handle, g.ctypes.data_as(_FP), g.size), "Cnn.grads")
        return g

    def forward(self, inp, out):
        """inp: (n, h, w, 4) float32 CUDA tensor; out: same shape, filled with (strength logit, residual)."""
        n, h, w, _ = inp.shape
        self.ctx.check(lib().gls_cnn_forward(self.handle, ctypes.c_void_p(inp.data_ptr()), w, h, n,
                                             ctypes.c_void_p(out.data_ptr())), "Cnn.forward")
        return out

    def set_backend(self, backend):
        """Forward pass: 1 tcgen05 hidden layers (default), 0 mma.sync, 2 all five layers in one
        fused tcgen05 kernel (inference; training uses the per-layer path)."""
        self.ctx.check(lib().gls_cnn_set_backend(self.handle, int(backend)), "Cnn.set_backend")

    def status(self):
        self.ctx.check(lib().gls_cnn_status(self.handle), "Cnn.status")

    def wait_probe(self, polls):
        """Runs the tensor-core kernels' bounded wait on a barrier that never completes; the
        next status() raises GLS_ERR_TIMEOUT."""
        self.ctx.check(lib().gls_cnn_wait_probe(self.handle, int(polls)), "Cnn.wait_probe")

    def train_step(self, inp, gt, lr):
        n, h, w, _ = inp.shape
        loss = (ctypes.c_float * 2)()
        self.ctx.check(lib().gls_cnn_train_step(self.handle, ctypes.c_void_p(inp.data_ptr()),
                                                ctypes.c_void_p(gt.data_ptr()), w, h, n, float(lr), loss),
                       "Cnn.train_step")
        return float(loss[0]), float(loss[1])

    def close(self):
        if self.handle:
            lib().gls_cnn_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cnn_split(params):
    """Flat parameter array -> [(W (cout, 3, 3, cin), b (cout,)) per layer]."""
    out, o = [], 0
    for cin, cout in CNN_LAYERS:
        W = np.asarray(params[o:o + cout * 9 * cin], np.float32).reshape(cout, 3, 3, cin)
        o += cout * 9 * cin
        out.append((W, np.asarray(params[o:o + cout], np.float32)))
        o += cout
    return out


def cnn_init(seed=0, head_std=0.0):
    """He-initialised hidden layers, zero biases; the head starts at zero (head_std = 0), so
    the untrained network is the plain pipeline exactly (residual 0, multiplier 1)."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (cin, cout) in enumerate(CNN_LAYERS):
        std = head_std if l == len(CNN_LAYERS) - 1 else np.sqrt(2.0 / (9 * cin))
        parts.append(rng.normal(0.0, std, cout * 9 * cin).astype(np.float32) if std > 0
                     else np.zeros(cout * 9 * cin, np.float32))
        parts.append(np.zeros(cout, np.float32))
    return np.concatenate(parts)
