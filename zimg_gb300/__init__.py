"""zimg_gb300: zimg's separable polyphase resize on one GB300 GPU.

The compute path is the native library built from zimg_gb300/csrc (CUDA for
sm_103a plus C++ host planning) and exposed through the C ABI in
include/zimg_gb300.h. This package is a thin Python mirror of that ABI.
"""
from .capi import ZimgError, load  # noqa: F401
from .resize import (Batch, Colorspace, ColorspaceConversion, Depth, DepthConversion, FilterContext, Graph,  # noqa: F401
                     HostPipeline, Resize,
                     ResizeConversion, Unresize, UnresizeConversion,
                     ResizeImplBuilder, ResizePass, compute_filter, filter_id, graph_params, image_format)

__version__ = "0.1.0"
