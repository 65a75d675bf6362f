"""gls-cuda: GB300-native (sm_103a) RAW->RGB pipeline with CLImage's operator surface.

    from climage_gb300 import gls, configs, synthetic
    ctx = gls.Context()
    conv = gls.RawConverter(ctx)
    conv.demosaicImage(raw_cuda_u16, configs.to_gls_params(spec), out_cuda_rgba8)

The CUDA kernels live in libgls_cuda.so (built by climage_gb300.build); its C ABI is
include/gls_cuda.h.
"""
__all__ = ["gls", "configs", "synthetic", "build"]
