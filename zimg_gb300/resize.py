"""Python mirror of zimg's resize interfaces, over the C ABI.

Names and argument meaning follow the reference:

* ``ResizeImplBuilder`` — src/zimg/resize/resize_impl.h:45-63 (one pass)
* ``ResizeConversion`` — src/zimg/resize/resize.h:22-44 (zero to two passes)
* ``compute_filter``   — src/zimg/resize/filter.h:178 (host-side tap tables)
* ``Batch``            — many conversions in one persistent launch
* ``DepthConversion``  — src/zimg/depth/depth.h:29-53 (pixel type / depth / range)
* ``UnresizeConversion`` — src/zimg/unresize/unresize.h:96-114 (inverse bilinear)
* ``Graph``            — zimg_filter_graph_build/process: resize, with the depth
                         conversions zimg's graph puts around it

Device buffers are PyTorch CUDA tensors (plumbing only: memory and streams);
every computation runs in the native library. WORD planes may be passed as
int16 or uint16 tensors (the bytes are what matters).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import ZimgError, check, load

__all__ = ["ZimgError", "compute_filter", "FilterContext", "ResizeImplBuilder", "ResizePass", "ResizeConversion",
           "Resize", "Batch", "Graph", "DepthConversion", "Depth", "UnresizeConversion", "Unresize", "filter_id"]


def filter_id(kind) -> int:
    if isinstance(kind, str):
        if kind not in capi.FILTER:
            raise ZimgError(2049, f"unrecognized resampling filter {kind!r}")
        return capi.FILTER[kind]
    return int(kind)


def _pixel_id(t) -> int:
    if isinstance(t, str):
        return capi.PIXEL[t]
    return int(t)


def _stream_handle(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _plane(t):
    """(device pointer, byte stride, width, height) of a 2-D CUDA tensor."""
    if t.dim() != 2:
        raise ValueError("planes are 2-D tensors [height, width]")
    if t.stride(1) != 1:
        raise ValueError("plane rows must be contiguous")
    if not t.is_cuda:
        raise ValueError("planes must be CUDA tensors")
    return t.data_ptr(), t.stride(0) * t.element_size(), t.shape[1], t.shape[0]


@dataclass
class FilterContext:
    """zimg's FilterContext (filter.h:133-165) with rows packed densely."""
    filter_width: int
    filter_rows: int
    data: np.ndarray       # float32 [rows, width]
    data_i16: np.ndarray   # int16   [rows, width]
    left: np.ndarray       # uint32  [rows]


def compute_filter(kind, src_dim: int, dst_dim: int, shift: float = 0.0, width: float | None = None,
                   a: float = math.nan, b: float = math.nan) -> FilterContext:
    lib = load()
    w = float(src_dim if width is None else width)
    fw, rows = C.c_uint(), C.c_uint()
    check(lib.zg_compute_filter(filter_id(kind), a, b, src_dim, dst_dim, shift, w, C.byref(fw), C.byref(rows),
                                None, None, None))
    f32 = np.zeros((rows.value, fw.value), np.float32)
    i16 = np.zeros((rows.value, fw.value), np.int16)
    left = np.zeros(rows.value, np.uint32)
    check(lib.zg_compute_filter(filter_id(kind), a, b, src_dim, dst_dim, shift, w, C.byref(fw), C.byref(rows),
                                f32.ctypes.data, i16.ctypes.data, left.ctypes.data))
    return FilterContext(fw.value, rows.value, f32, i16, left)


class _Builder:
    def _set(self, name, value):
        setattr(self, name, value)
        return self


class ResizePass:
    """One ResizeImplH / ResizeImplV equivalent on the GPU."""

    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_resize_pass_free(self._h)
            self._h = None

    @property
    def output_size(self) -> tuple[int, int]:
        w, h = C.c_uint(), C.c_uint()
        check(load().zg_resize_pass_get_output(self._h, C.byref(w), C.byref(h)))
        return w.value, h.value

    def process(self, src, dst, stream=None) -> None:
        sp, ss, _, _ = _plane(src)
        dp, ds, _, _ = _plane(dst)
        check(load().zg_resize_pass_process(self._h, sp, ss, dp, ds, _stream_handle(stream)))


class ResizeImplBuilder(_Builder):
    """ResizeImplBuilder{src_width, src_height, type} (resize_impl.h:45-63)."""

    def __init__(self, src_width: int, src_height: int, pixel_type="float"):
        self.src_width, self.src_height, self.type = src_width, src_height, _pixel_id(pixel_type)
        self.horizontal, self.dst_dim, self.depth = False, 0, 16 if self.type == 1 else 32
        self.filter, self.param_a, self.param_b = 2, math.nan, math.nan
        self.shift, self.subwidth, self.engine = 0.0, math.nan, "auto"

    def set_horizontal(self, v: bool): return self._set("horizontal", bool(v))
    def set_dst_dim(self, v: int): return self._set("dst_dim", int(v))
    def set_depth(self, v: int): return self._set("depth", int(v))
    def set_shift(self, v: float): return self._set("shift", float(v))
    def set_subwidth(self, v: float): return self._set("subwidth", float(v))
    def set_engine(self, v: str): return self._set("engine", v)

    def set_filter(self, kind, a: float = math.nan, b: float = math.nan):
        self.filter, self.param_a, self.param_b = filter_id(kind), float(a), float(b)
        return self

    def create(self) -> ResizePass:
        p = capi.PassParams(self.src_width, self.src_height, self.type, self.depth, int(self.horizontal),
                            self.dst_dim, self.filter, self.param_a, self.param_b, self.shift, self.subwidth,
                            capi.ENGINE[self.engine])
        h = C.c_void_p()
        check(load().zg_resize_pass_create(C.byref(p), C.byref(h)))
        return ResizePass(h.value)


class Resize:
    """The created conversion (what ResizeConversion::create returns)."""

    def __init__(self, handle, params: capi.ResizeParams):
        self._h = handle
        self.params = params

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_resize_free(self._h)
            self._h = None

    @property
    def handle(self) -> int:
        return self._h

    @property
    def tmp_size(self) -> int:
        n = C.c_size_t()
        check(load().zg_resize_get_tmp_size(self._h, C.byref(n)))
        return n.value

    @property
    def info(self) -> dict:
        n, f, fu = C.c_int(), C.c_int(), C.c_int()
        check(load().zg_resize_get_info(self._h, C.byref(n), C.byref(f), C.byref(fu)))
        return {"num_passes": n.value, "first_horizontal": bool(f.value), "fused": bool(fu.value),
                "engine": {0: "passes", 1: "cuda", 2: "tensor", 3: "tensor-passes"}[fu.value]}

    def alloc_tmp(self, device=None):
        import torch
        n = self.tmp_size
        return torch.empty(max(n, 1), dtype=torch.uint8, device=device or "cuda") if n else None

    def process(self, src, dst, tmp=None, stream=None) -> None:
        sp, ss, _, _ = _plane(src)
        dp, ds, _, _ = _plane(dst)
        if tmp is None and self.tmp_size:
            tmp = self.alloc_tmp(src.device)
        tp = tmp.data_ptr() if tmp is not None else None
        check(load().zg_resize_process(self._h, sp, ss, dp, ds, tp, _stream_handle(stream)))


def _resize_params(src_width, src_height, pixel_type, depth, dst_width, dst_height, kind, a, b, shift_w, shift_h,
                   subwidth, subheight, engine="auto", allow_fusion=True) -> capi.ResizeParams:
    p = capi.ResizeParams()
    load().zg_resize_params_default(C.byref(p))
    p.src_width, p.src_height, p.pixel_type = src_width, src_height, _pixel_id(pixel_type)
    p.depth = depth if depth is not None else (16 if p.pixel_type == 1 else 32)
    p.dst_width, p.dst_height = dst_width, dst_height
    p.filter, p.filter_param_a, p.filter_param_b = filter_id(kind), a, b
    p.shift_w, p.shift_h = shift_w, shift_h
    p.subwidth = math.nan if subwidth is None else subwidth
    p.subheight = math.nan if subheight is None else subheight
    p.engine = capi.ENGINE[engine]
    p.allow_fusion = int(bool(allow_fusion))
    return p


class ResizeConversion(_Builder):
    """ResizeConversion{src_width, src_height, type} (resize.h:22-44)."""

    def __init__(self, src_width: int, src_height: int, pixel_type="float"):
        self.src_width, self.src_height, self.type = src_width, src_height, _pixel_id(pixel_type)
        self.depth = 16 if self.type == 1 else 32
        self.filter, self.param_a, self.param_b = 2, math.nan, math.nan
        self.dst_width, self.dst_height = src_width, src_height
        self.shift_w = self.shift_h = 0.0
        self.subwidth = self.subheight = None
        self.engine, self.fusion = "auto", True

    def set_depth(self, v: int): return self._set("depth", int(v))
    def set_dst_width(self, v: int): return self._set("dst_width", int(v))
    def set_dst_height(self, v: int): return self._set("dst_height", int(v))
    def set_shift_w(self, v: float): return self._set("shift_w", float(v))
    def set_shift_h(self, v: float): return self._set("shift_h", float(v))
    def set_subwidth(self, v: float): return self._set("subwidth", float(v))
    def set_subheight(self, v: float): return self._set("subheight", float(v))
    def set_engine(self, v: str): return self._set("engine", v)
    def set_fusion(self, v: bool): return self._set("fusion", bool(v))

    def set_filter(self, kind, a: float = math.nan, b: float = math.nan):
        self.filter, self.param_a, self.param_b = filter_id(kind), float(a), float(b)
        return self

    def params(self) -> capi.ResizeParams:
        return _resize_params(self.src_width, self.src_height, self.type, self.depth, self.dst_width,
                              self.dst_height, self.filter, self.param_a, self.param_b, self.shift_w, self.shift_h,
                              self.subwidth, self.subheight, self.engine, self.fusion)

    def create(self) -> Resize:
        p = self.params()
        h = C.c_void_p()
        check(load().zg_resize_create(C.byref(p), C.byref(h)))
        return Resize(h.value, p)


class Depth:
    """The created depth conversion (zimg's DepthConversion::create result for
    one plane): process(src, dst) converts a whole device plane."""

    MODES = {0: "copy", 1: "left_shift", 2: "to_float", 3: "dither"}

    def __init__(self, handle, params: capi.DepthParams):
        self._h = handle
        self.params = params

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_depth_free(self._h)
            self._h = None

    @property
    def mode(self) -> str:
        m = C.c_int()
        check(load().zg_depth_get_info(self._h, C.byref(m)))
        return self.MODES[m.value]

    def process(self, src, dst, stream=None) -> None:
        sp, ss, _, _ = _plane(src)
        dp, ds, _, _ = _plane(dst)
        check(load().zg_depth_process(self._h, sp, ss, dp, ds, _stream_handle(stream)))


class DepthConversion(_Builder):
    """DepthConversion{width, height} (src/zimg/depth/depth.h:29-53): pixel
    formats as (type, depth, fullrange, chroma), dither type, plane index."""

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self.pixel_in = ("word", 16, False, False)
        self.pixel_out = ("word", 16, False, False)
        self.dither, self.plane = "none", 0

    def set_pixel_in(self, type, depth=0, fullrange=False, chroma=False):
        return self._set("pixel_in", (type, int(depth), bool(fullrange), bool(chroma)))

    def set_pixel_out(self, type, depth=0, fullrange=False, chroma=False):
        return self._set("pixel_out", (type, int(depth), bool(fullrange), bool(chroma)))

    def set_dither_type(self, v: str): return self._set("dither", v)
    def set_plane(self, v: int): return self._set("plane", int(v))

    def params(self) -> capi.DepthParams:
        def fmt(f):
            t, d, full, chroma = f
            return capi.PixelFormat(_pixel_id(t), d, int(full), int(chroma), 0)
        return capi.DepthParams(self.width, self.height, fmt(self.pixel_in), fmt(self.pixel_out),
                                capi.DITHER[self.dither], self.plane)

    def create(self) -> Depth:
        p = self.params()
        h = C.c_void_p()
        check(load().zg_depth_create(C.byref(p), C.byref(h)))
        return Depth(h.value, p)


class Colorspace:
    """The created colorspace conversion (zimg's ColorspaceConversion::create
    result): three FLOAT planes in, three out."""

    OPS = ("matrix", "gamma", "hlg", "hlg_inverse", "cl_to_rgb", "cl_to_yuv")

    def __init__(self, handle, params: capi.ColorspaceParams):
        self._h = handle
        self.params = params

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_colorspace_free(self._h)
            self._h = None

    @property
    def ops(self) -> list:
        n = C.c_uint()
        kinds = (C.c_int * 6)()
        check(load().zg_colorspace_get_info(self._h, C.byref(n), kinds))
        return [self.OPS[kinds[k]] for k in range(n.value)]

    def process(self, src, dst, stream=None) -> None:
        """src, dst: three 2-D float32 CUDA tensors each (dst may be src)."""
        sp = (C.c_void_p * 3)(*[_plane(t)[0] for t in src])
        ss = (C.c_ssize_t * 3)(*[_plane(t)[1] for t in src])
        dp = (C.c_void_p * 3)(*[_plane(t)[0] for t in dst])
        ds = (C.c_ssize_t * 3)(*[_plane(t)[1] for t in dst])
        check(load().zg_colorspace_process(self._h, sp, ss, dp, ds, _stream_handle(stream)))


class ColorspaceConversion(_Builder):
    """ColorspaceConversion{width, height} (src/zimg/colorspace/colorspace.h:
    117-132): colorspaces as (matrix, transfer, primaries) zimg API codes."""

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self.csp_in = (2, 2, 2)
        self.csp_out = (2, 2, 2)
        self.peak_luminance = 100.0
        self.approximate_gamma = self.scene_referred = self.chromatic_adaptation = False

    def set_csp_in(self, matrix, transfer, primaries): return self._set("csp_in", (matrix, transfer, primaries))
    def set_csp_out(self, matrix, transfer, primaries): return self._set("csp_out", (matrix, transfer, primaries))
    def set_peak_luminance(self, v: float): return self._set("peak_luminance", float(v))
    def set_approximate_gamma(self, v: bool): return self._set("approximate_gamma", bool(v))
    def set_scene_referred(self, v: bool): return self._set("scene_referred", bool(v))
    def set_chromatic_adaptation(self, v: bool): return self._set("chromatic_adaptation", bool(v))

    def create(self) -> Colorspace:
        p = capi.ColorspaceParams(self.width, self.height, *self.csp_in, *self.csp_out, self.peak_luminance,
                                  int(self.approximate_gamma), int(self.scene_referred),
                                  int(self.chromatic_adaptation))
        h = C.c_void_p()
        check(load().zg_colorspace_create(C.byref(p), C.byref(h)))
        return Colorspace(h.value, p)


class Unresize:
    """The created unresize (zimg's UnresizeConversion::create result)."""

    def __init__(self, handle, params: capi.UnresizeParams):
        self._h = handle
        self.params = params

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_unresize_free(self._h)
            self._h = None

    @property
    def tmp_size(self) -> int:
        n = C.c_size_t()
        check(load().zg_unresize_get_tmp_size(self._h, C.byref(n)))
        return n.value

    def process(self, src, dst, tmp=None, stream=None) -> None:
        sp, ss, _, _ = _plane(src)
        dp, ds, _, _ = _plane(dst)
        if tmp is None and self.tmp_size:
            import torch
            tmp = torch.empty(self.tmp_size, dtype=torch.uint8, device=src.device)
        tp = tmp.data_ptr() if tmp is not None else None
        check(load().zg_unresize_process(self._h, sp, ss, dp, ds, tp, _stream_handle(stream)))


class UnresizeConversion(_Builder):
    """UnresizeConversion{up_width, up_height, FLOAT} (src/zimg/unresize/unresize.h:96-114)."""

    def __init__(self, up_width: int, up_height: int):
        self.up_width, self.up_height = up_width, up_height
        self.orig_width, self.orig_height = up_width, up_height
        self.shift_w = self.shift_h = 0.0

    def set_orig_width(self, v: int): return self._set("orig_width", int(v))
    def set_orig_height(self, v: int): return self._set("orig_height", int(v))
    def set_shift_w(self, v: float): return self._set("shift_w", float(v))
    def set_shift_h(self, v: float): return self._set("shift_h", float(v))

    def create(self) -> Unresize:
        p = capi.UnresizeParams(self.up_width, self.up_height, self.orig_width, self.orig_height, self.shift_w,
                                self.shift_h)
        h = C.c_void_p()
        check(load().zg_unresize_create(C.byref(p), C.byref(h)))
        return Unresize(h.value, p)


class Batch:
    """Many conversions of uneven sizes, launched together."""

    def __init__(self, conversions: list[ResizeConversion]):
        arr = (capi.ResizeParams * len(conversions))(*[c.params() for c in conversions])
        h = C.c_void_p()
        check(load().zg_batch_create(arr, len(conversions), C.byref(h)))
        self._h = h.value
        self.n = len(conversions)
        self._tmp = None

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_batch_free(self._h)
            self._h = None

    @property
    def tmp_size(self) -> int:
        n = C.c_size_t()
        check(load().zg_batch_get_tmp_size(self._h, C.byref(n)))
        return n.value

    @property
    def launch_count(self) -> int:
        n = C.c_uint()
        check(load().zg_batch_get_launch_count(self._h, C.byref(n)))
        return n.value

    def set_io(self, srcs, dsts, stream=None) -> None:
        if len(srcs) != self.n or len(dsts) != self.n:
            raise ValueError("one src and one dst per job")
        io = (capi.BatchIO * self.n)()
        for i, (s, d) in enumerate(zip(srcs, dsts)):
            sp, ss, _, _ = _plane(s)
            dp, ds, _, _ = _plane(d)
            io[i] = capi.BatchIO(sp, ss, dp, ds)
        check(load().zg_batch_set_io(self._h, io, _stream_handle(stream)))

    def autotune(self, stream=None) -> int:
        """Time the planner's alternatives for every AUTO job on its bound
        planes and keep the fastest (zg_batch_autotune). Returns the number of
        jobs whose plan changed; the tmp size may change with them."""
        n = C.c_uint()
        check(load().zg_batch_autotune(self._h, _stream_handle(stream), C.byref(n)))
        self._tmp = None
        return n.value

    def _tmp_ptr(self, tmp):
        if tmp is None and self.tmp_size:
            if self._tmp is None:
                import torch
                self._tmp = torch.empty(self.tmp_size, dtype=torch.uint8, device="cuda")
            tmp = self._tmp
        return tmp.data_ptr() if tmp is not None else None

    def process(self, tmp=None, stream=None) -> None:
        check(load().zg_batch_process(self._h, self._tmp_ptr(tmp), _stream_handle(stream)))

    def process_graph(self, tmp=None, stream=None) -> None:
        check(load().zg_batch_process_graph(self._h, self._tmp_ptr(tmp), _stream_handle(stream)))


class HostPipeline:
    """Conversions of planes that live in (pinned) host memory.

    The planes are split into `chunks` sub-batches, each with its own device
    staging planes and Batch. Per call, chunk i's host-to-device copies, its
    batch launch and its device-to-host copies go to three streams ordered by
    events, so the copies of one chunk overlap the work of its neighbours.
    `run` returns once the results are in the host planes."""

    def __init__(self, conversions: list[ResizeConversion], chunks: int = 4, autotune: bool = True):
        import torch
        n = len(conversions)
        self.chunks = max(1, min(chunks, n))
        bounds = [round(i * n / self.chunks) for i in range(self.chunks + 1)]
        self.parts = []
        for c in range(self.chunks):
            convs = conversions[bounds[c]:bounds[c + 1]]
            srcs, dsts = [], []
            for conv in convs:
                dt = torch.int16 if conv.type == _pixel_id("word") else torch.float32
                srcs.append(torch.empty((conv.src_height, conv.src_width), dtype=dt, device="cuda"))
                dsts.append(torch.empty((conv.dst_height, conv.dst_width), dtype=dt, device="cuda"))
            b = Batch(convs)
            b.set_io(srcs, dsts)
            if autotune:
                b.autotune()
            tmp = torch.empty(max(b.tmp_size, 1), dtype=torch.uint8, device="cuda")
            self.parts.append((bounds[c], b, srcs, dsts, tmp))
        self.streams = [torch.cuda.Stream() for _ in range(3)]

    def run(self, host_srcs, host_dsts) -> None:
        import torch
        h2d, work, d2h = self.streams
        cur = torch.cuda.current_stream()
        for s in self.streams:
            s.wait_stream(cur)
        for first, b, srcs, dsts, tmp in self.parts:
            with torch.cuda.stream(h2d):
                for k, d in enumerate(srcs):
                    d.copy_(host_srcs[first + k], non_blocking=True)
            work.wait_stream(h2d)
            b.process(tmp, stream=work)
            d2h.wait_stream(work)
            with torch.cuda.stream(d2h):
                for k, d in enumerate(dsts):
                    host_dsts[first + k].copy_(d, non_blocking=True)
        for s in self.streams:
            cur.wait_stream(s)
        cur.synchronize()


def image_format(width, height, pixel_type="float", **kw) -> capi.ImageFormat:
    """zimg_image_format with zimg's defaults (zimg.cpp:595-630), then kw."""
    f = capi.ImageFormat()
    load().zg_image_format_default(C.byref(f), capi.API_VERSION_2_4)
    f.width, f.height, f.pixel_type = width, height, _pixel_id(pixel_type)
    for k, v in kw.items():
        if k == "active_region":
            f.active_region = capi.ActiveRegion(*v)
        else:
            setattr(f, k, v)
    return f


def graph_params(**kw) -> capi.GraphBuilderParams:
    p = capi.GraphBuilderParams()
    load().zg_graph_builder_params_default(C.byref(p), capi.API_VERSION_2_4)
    for k, v in kw.items():
        if k == "resample_filter" and v == "unresize":
            v = capi.RESIZE_UNRESIZE
        elif k in ("resample_filter", "resample_filter_uv"):
            v = filter_id(v)
        setattr(p, k, v)
    return p


class Graph:
    """zimg_filter_graph (zimg.h:507,550-552,679): resize, with the depth
    conversions zimg's graph puts around it when the pixel format changes."""

    def __init__(self, src_format: capi.ImageFormat, dst_format: capi.ImageFormat,
                 params: capi.GraphBuilderParams | None = None):
        lib = load()
        h = lib.zg_graph_build(C.byref(src_format), C.byref(dst_format), C.byref(params) if params else None)
        if not h:
            code, msg = capi.last_error()
            raise ZimgError(code, msg)
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            load().zg_graph_free(self._h)
            self._h = None

    @property
    def tmp_size(self) -> int:
        n = C.c_size_t()
        check(load().zg_graph_get_tmp_size(self._h, C.byref(n)))
        return n.value

    def plane_params(self, plane: int):
        p = capi.ResizeParams()
        present = C.c_int()
        check(load().zg_graph_get_plane_params(self._h, plane, C.byref(p), C.byref(present)))
        return present.value, p

    @property
    def input_buffering(self) -> int:
        n = C.c_uint()
        check(load().zg_graph_get_input_buffering(self._h, C.byref(n)))
        return n.value

    @property
    def output_buffering(self) -> int:
        n = C.c_uint()
        check(load().zg_graph_get_output_buffering(self._h, C.byref(n)))
        return n.value

    def process(self, src_planes, dst_planes, tmp=None, stream=None, src_masks=None, dst_masks=None,
                unpack=None, pack=None) -> None:
        """Planes are 2-D CUDA tensors (or None). A plane given with a mask
        (2^n - 1) is a ring of 2^n lines: line i at row i & mask. unpack /
        pack: Python callables f(i, left, right) -> int, called as zimg's
        zimg_filter_graph_callback (zimg.h:455-484)."""
        def buf(planes, masks):
            b = capi.ImageBuffer()
            b.version = capi.API_VERSION_2_4
            for i, t in enumerate(planes):
                if t is None:
                    continue
                ptr, stride, _, _ = _plane(t)
                mask = capi.BUFFER_MAX if not masks or masks[i] is None else masks[i]
                b.plane[i] = capi._PlaneC(ptr, stride, mask)
            return b
        s, d = buf(src_planes, src_masks), buf(dst_planes, dst_masks)
        if tmp is None and self.tmp_size:
            import torch
            tmp = torch.empty(self.tmp_size, dtype=torch.uint8, device="cuda")
        tp = tmp.data_ptr() if tmp is not None else None
        if unpack is None and pack is None and not src_masks and not dst_masks:
            check(load().zg_graph_process(self._h, C.byref(s), C.byref(d), tp, _stream_handle(stream)))
            return

        def wrap(f):
            return capi.GRAPH_CALLBACK(lambda user, i, left, right: int(f(i, left, right))) if f else None
        ucb, pcb = wrap(unpack), wrap(pack)
        check(load().zg_graph_process_cb(self._h, C.byref(s), C.byref(d), tp,
                                         C.cast(ucb, C.c_void_p) if ucb else None, None,
                                         C.cast(pcb, C.c_void_p) if pcb else None, None, _stream_handle(stream)))
