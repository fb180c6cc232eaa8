"""ctypes binding of the C ABI in include/zimg_gb300.h.

The shared library is built in-tree (zimg_gb300/build.py). Loading fails
loudly if it is missing: there is no CPU or PyTorch fallback for the resize
path.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libzimg_gb300.so")

# enum values (include/zimg_gb300.h)
PIXEL = {"byte": 0, "word": 1, "half": 2, "float": 3}
FILTER = {"point": 0, "bilinear": 1, "bicubic": 2, "spline16": 3, "spline36": 4, "lanczos": 5, "spline64": 6}
ENGINE = {"auto": 0, "cuda": 1, "tensor": 2}
RESIZE_UNRESIZE = -1  # graph only: unresize instead of resize (zimg.cpp:21)

ERROR_NAMES = {
    -1: "UNKNOWN", 0: "SUCCESS", 1: "OUT_OF_MEMORY", 2: "USER_CALLBACK_FAILED", 1024: "LOGIC",
    1025: "GREYSCALE_SUBSAMPLING", 1026: "COLOR_FAMILY_MISMATCH", 1027: "IMAGE_NOT_DIVISIBLE",
    1028: "BIT_DEPTH_OVERFLOW", 2048: "ILLEGAL_ARGUMENT", 2049: "ENUM_OUT_OF_RANGE", 2050: "INVALID_IMAGE_SIZE",
    3072: "UNSUPPORTED_OPERATION", 3073: "UNSUPPORTED_SUBSAMPLING", 3074: "NO_COLORSPACE_CONVERSION",
    3075: "NO_FIELD_PARITY_CONVERSION", 3076: "RESAMPLING_NOT_AVAILABLE",
}


class ZimgError(RuntimeError):
    """A non-zero zg_error_code, with the library's thread-local message."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)} ({code}): {msg}")
        self.code = code
        self.msg = msg


class PassParams(C.Structure):
    _fields_ = [("src_width", C.c_uint), ("src_height", C.c_uint), ("pixel_type", C.c_int), ("depth", C.c_uint),
                ("horizontal", C.c_int), ("dst_dim", C.c_uint), ("filter", C.c_int), ("filter_param_a", C.c_double),
                ("filter_param_b", C.c_double), ("shift", C.c_double), ("subwidth", C.c_double), ("engine", C.c_int)]


class ResizeParams(C.Structure):
    _fields_ = [("src_width", C.c_uint), ("src_height", C.c_uint), ("pixel_type", C.c_int), ("depth", C.c_uint),
                ("dst_width", C.c_uint), ("dst_height", C.c_uint), ("filter", C.c_int),
                ("filter_param_a", C.c_double), ("filter_param_b", C.c_double), ("shift_w", C.c_double),
                ("shift_h", C.c_double), ("subwidth", C.c_double), ("subheight", C.c_double), ("engine", C.c_int),
                ("allow_fusion", C.c_int)]


class PixelFormat(C.Structure):
    _fields_ = [("type", C.c_int), ("depth", C.c_uint), ("fullrange", C.c_int), ("chroma", C.c_int),
                ("ycgco", C.c_int)]


class DepthParams(C.Structure):
    _fields_ = [("width", C.c_uint), ("height", C.c_uint), ("pixel_in", PixelFormat), ("pixel_out", PixelFormat),
                ("dither_type", C.c_int), ("plane", C.c_uint)]


DITHER = {"none": 0, "ordered": 1, "random": 2, "error_diffusion": 3}


class ColorspaceParams(C.Structure):
    _fields_ = [("width", C.c_uint), ("height", C.c_uint), ("matrix_in", C.c_int), ("transfer_in", C.c_int),
                ("primaries_in", C.c_int), ("matrix_out", C.c_int), ("transfer_out", C.c_int),
                ("primaries_out", C.c_int), ("peak_luminance", C.c_double), ("approximate_gamma", C.c_int),
                ("scene_referred", C.c_int), ("chromatic_adaptation", C.c_int)]


class UnresizeParams(C.Structure):
    _fields_ = [("up_width", C.c_uint), ("up_height", C.c_uint), ("orig_width", C.c_uint),
                ("orig_height", C.c_uint), ("shift_w", C.c_double), ("shift_h", C.c_double)]


class BatchIO(C.Structure):
    _fields_ = [("src", C.c_void_p), ("src_stride", C.c_ssize_t), ("dst", C.c_void_p), ("dst_stride", C.c_ssize_t)]


class ActiveRegion(C.Structure):
    _fields_ = [("left", C.c_double), ("top", C.c_double), ("width", C.c_double), ("height", C.c_double)]


class ImageFormat(C.Structure):
    _fields_ = [("version", C.c_uint), ("width", C.c_uint), ("height", C.c_uint), ("pixel_type", C.c_int),
                ("subsample_w", C.c_uint), ("subsample_h", C.c_uint), ("color_family", C.c_int),
                ("matrix_coefficients", C.c_int), ("transfer_characteristics", C.c_int),
                ("color_primaries", C.c_int), ("depth", C.c_uint), ("pixel_range", C.c_int),
                ("field_parity", C.c_int), ("chroma_location", C.c_int), ("active_region", ActiveRegion),
                ("alpha", C.c_int)]


class GraphBuilderParams(C.Structure):
    _fields_ = [("version", C.c_uint), ("resample_filter", C.c_int), ("filter_param_a", C.c_double),
                ("filter_param_b", C.c_double), ("resample_filter_uv", C.c_int), ("filter_param_a_uv", C.c_double),
                ("filter_param_b_uv", C.c_double), ("dither_type", C.c_int), ("cpu_type", C.c_int),
                ("nominal_peak_luminance", C.c_double), ("allow_approximate_gamma", C.c_char),
                ("scene_referred", C.c_char), ("chromatic_adaptation", C.c_char)]


class _PlaneC(C.Structure):
    _fields_ = [("data", C.c_void_p), ("stride", C.c_ssize_t), ("mask", C.c_uint)]


class ImageBuffer(C.Structure):
    _fields_ = [("version", C.c_uint), ("plane", _PlaneC * 4)]


API_VERSION_2_4 = (2 << 8) | 4

# zg_graph_callback: int (*)(void *user, unsigned i, unsigned left, unsigned right)
GRAPH_CALLBACK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint)
BUFFER_MAX = 0xFFFFFFFF

# (name, restype, argtypes) for every function declared in include/zimg_gb300.h
_P = C.c_void_p
SIGNATURES = [
    ("zg_get_last_error", C.c_int, [C.c_char_p, C.c_size_t]),
    ("zg_pipeline_status", C.c_int, [C.c_int]),
    ("zg_debug_pipeline_fault", C.c_int, [C.c_int, C.c_ulonglong]),
    ("zg_wide_forms_used", C.c_int, [C.c_int]),
    ("zg_unresize_create", C.c_int, [C.POINTER(UnresizeParams), C.POINTER(C.c_void_p)]),
    ("zg_unresize_free", None, [C.c_void_p]),
    ("zg_unresize_get_tmp_size", C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    ("zg_unresize_process", C.c_int, [C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t, C.c_void_p,
                                      C.c_void_p]),
    ("zg_depth_create", C.c_int, [C.POINTER(DepthParams), C.POINTER(C.c_void_p)]),
    ("zg_depth_free", None, [C.c_void_p]),
    ("zg_depth_get_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("zg_depth_process", C.c_int, [C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t, C.c_void_p]),
    ("zg_colorspace_create", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("zg_colorspace_free", None, [C.c_void_p]),
    ("zg_colorspace_get_info", C.c_int, [C.c_void_p, C.POINTER(C.c_uint), C.POINTER(C.c_int)]),
    ("zg_colorspace_process", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_ssize_t),
                                        C.POINTER(C.c_void_p), C.POINTER(C.c_ssize_t), C.c_void_p]),
    ("zg_clear_last_error", None, []),
    ("zg_get_version_info", None, [C.POINTER(C.c_uint)] * 3),
    ("zg_compute_filter", C.c_int, [C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint, C.c_double, C.c_double,
                                    C.POINTER(C.c_uint), C.POINTER(C.c_uint), _P, _P, _P]),
    ("zg_resize_pass_create", C.c_int, [C.POINTER(PassParams), C.POINTER(_P)]),
    ("zg_resize_pass_free", None, [_P]),
    ("zg_resize_pass_get_output", C.c_int, [_P, C.POINTER(C.c_uint), C.POINTER(C.c_uint)]),
    ("zg_resize_pass_process", C.c_int, [_P, _P, C.c_ssize_t, _P, C.c_ssize_t, _P]),
    ("zg_resize_params_default", None, [C.POINTER(ResizeParams)]),
    ("zg_resize_create", C.c_int, [C.POINTER(ResizeParams), C.POINTER(_P)]),
    ("zg_resize_free", None, [_P]),
    ("zg_resize_get_tmp_size", C.c_int, [_P, C.POINTER(C.c_size_t)]),
    ("zg_resize_get_info", C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("zg_resize_process", C.c_int, [_P, _P, C.c_ssize_t, _P, C.c_ssize_t, _P, _P]),
    ("zg_resize_process_no_alloc", C.c_int, [_P, _P, C.c_ssize_t, _P, C.c_ssize_t, _P]),
    ("zg_batch_create", C.c_int, [C.POINTER(ResizeParams), C.c_uint, C.POINTER(_P)]),
    ("zg_batch_free", None, [_P]),
    ("zg_batch_get_tmp_size", C.c_int, [_P, C.POINTER(C.c_size_t)]),
    ("zg_batch_set_io", C.c_int, [_P, C.POINTER(BatchIO), _P]),
    ("zg_batch_process", C.c_int, [_P, _P, _P]),
    ("zg_batch_process_graph", C.c_int, [_P, _P, _P]),
    ("zg_batch_get_launch_count", C.c_int, [_P, C.POINTER(C.c_uint)]),
    ("zg_batch_autotune", C.c_int, [_P, _P, C.POINTER(C.c_uint)]),
    ("zg_image_format_default", None, [C.POINTER(ImageFormat), C.c_uint]),
    ("zg_graph_builder_params_default", None, [C.POINTER(GraphBuilderParams), C.c_uint]),
    ("zg_graph_build", _P, [C.POINTER(ImageFormat), C.POINTER(ImageFormat), C.POINTER(GraphBuilderParams)]),
    ("zg_graph_free", None, [_P]),
    ("zg_graph_get_tmp_size", C.c_int, [_P, C.POINTER(C.c_size_t)]),
    ("zg_graph_process", C.c_int, [_P, C.POINTER(ImageBuffer), C.POINTER(ImageBuffer), _P, _P]),
    ("zg_graph_process_cb", C.c_int, [_P, C.POINTER(ImageBuffer), C.POINTER(ImageBuffer), _P, _P, _P, _P, _P, _P]),
    ("zg_graph_get_input_buffering", C.c_int, [_P, C.POINTER(C.c_uint)]),
    ("zg_graph_get_output_buffering", C.c_int, [_P, C.POINTER(C.c_uint)]),
    ("zg_graph_get_plane_params", C.c_int, [_P, C.c_int, C.POINTER(ResizeParams), C.POINTER(C.c_int)]),
]

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"zimg_gb300 native library not built: {path} (run zimg_gb300/build.py)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> tuple[int, str]:
    buf = C.create_string_buffer(1024)
    code = load().zg_get_last_error(buf, len(buf))
    return code, buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != 0:
        code, msg = last_error()
        raise ZimgError(rc, msg)
