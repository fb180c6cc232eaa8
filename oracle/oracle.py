"""ORACLE — test infrastructure only; never imported by the product.

ctypes front end for two CPU checkers:

* ``Oracle``  — the plain-C restatement in ``oracle/zimg_oracle.c`` (built to
  ``oracle/_build/liboracle.so``). It exists on every machine that runs the
  tests, because ``__graft_entry__.build()`` compiles it there.
* ``Reference`` — zimg's own resize code compiled from the reference checkout by
  ``oracle/Makefile`` into ``oracle/_ref/libzimgref.so`` (only where that
  checkout exists). It pins the restatement.

Also holds the graph-level parameter mapping (chroma siting, field parity,
active region -> per-plane shift/subwidth), restated from
src/zimg/graph/graphbuilder.cpp:65-188,331-366,769-776 and
src/zimg/api/zimg.cpp:370-400.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libzimgref.so")

# zimg_resample_filter_e (zimg.h:374-382)
FILTERS = {"point": 0, "bilinear": 1, "bicubic": 2, "spline16": 3, "spline36": 4, "lanczos": 5, "spline64": 6}
T_U16, T_F32, T_F64 = 1, 3, 4
# zimg_pixel_type_e (zimg.h:184-189) and zimg_dither_type_e (zimg.h:191-196)
PIXEL_TYPES = {"byte": 0, "word": 1, "half": 2, "float": 3}
DITHERS = {"none": 0, "ordered": 1, "random": 2, "error_diffusion": 3}
NP_TYPES = {0: np.uint8, 1: np.uint16, 2: np.uint16, 3: np.float32}  # HALF planes hold binary16 bits


@dataclass(frozen=True)
class PixelFormat:
    """zimg's PixelFormat (src/zimg/common/pixel.h:135-181)."""
    type: str = "word"
    depth: int | None = None
    fullrange: bool = False
    chroma: bool = False

    @property
    def code(self) -> int:
        return PIXEL_TYPES[self.type]

    @property
    def bits(self) -> int:
        return self.depth if self.depth is not None else {0: 8, 1: 16, 2: 16, 3: 32}[self.code]

    @property
    def dtype(self):
        return NP_TYPES[self.code]


class _PixFmt(C.Structure):
    _fields_ = [("type", C.c_int), ("depth", C.c_uint), ("fullrange", C.c_int), ("chroma", C.c_int),
                ("ycgco", C.c_int)]


def _pixfmt(f: PixelFormat) -> _PixFmt:
    return _PixFmt(f.code, f.bits, int(f.fullrange), int(f.chroma), 0)


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference, where its sources exist)."""
    out = subprocess.run(["make", "-C", HERE, "-j8", "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout[-4000:] + out.stderr[-4000:])
    if not quiet:
        print(out.stdout)


def _f(kind):
    return FILTERS[kind] if isinstance(kind, str) else int(kind)


@dataclass
class FilterContext:
    width: int
    rows: int
    f32: np.ndarray   # [rows, width] float32
    i16: np.ndarray   # [rows, width] int16
    left: np.ndarray  # [rows] uint32
    f64: np.ndarray | None = None  # [rows, width] float64 (unquantised), oracle only


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_compute_filter.argtypes = [C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint, C.c_double, C.c_double,
                                         C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
        L.orc_resize_plane.argtypes = [C.c_int, C.c_uint, C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint,
                                       C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_int, C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t]
        L.orc_plan_create.restype = C.c_void_p
        L.orc_plan_create.argtypes = [C.c_int, C.c_uint, C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_plan_tmp_size.restype = C.c_size_t
        L.orc_plan_tmp_size.argtypes = [C.c_void_p]
        L.orc_plan_run.argtypes = [C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t, C.c_void_p]
        L.orc_plan_free.argtypes = [C.c_void_p]
        L.orc_resize_pass.argtypes = [C.c_int, C.c_uint, C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint,
                                      C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p,
                                      C.c_ssize_t, C.c_void_p, C.c_ssize_t]
        L.orc_plan_order.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.POINTER(C.c_int)]
        L.orc_depth_convert.argtypes = [C.POINTER(_PixFmt), C.POINTER(_PixFmt), C.c_int, C.c_uint, C.c_uint,
                                        C.c_uint, C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t]
        L.orc_depth_mode.argtypes = [C.POINTER(_PixFmt), C.POINTER(_PixFmt), C.c_int]
        L.orc_depth_scale_offset.argtypes = [C.POINTER(_PixFmt), C.POINTER(_PixFmt), C.POINTER(C.c_float),
                                             C.POINTER(C.c_float)]
        L.orc_bayer16.argtypes = [C.c_uint, C.c_uint]
        L.orc_bayer16.restype = C.c_uint
        L.orc_blue_noise.argtypes = [C.c_uint, C.c_uint]
        L.orc_blue_noise.restype = C.c_uint
        L.orc_dither_value.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_uint]
        L.orc_dither_value.restype = C.c_float
        L.orc_unresize_plane.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_double,
                                         C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t]

    def unresize_plane(self, src: np.ndarray, orig_w: int, orig_h: int, shift_w=0.0, shift_h=0.0) -> np.ndarray:
        """zimg's UnresizeConversion of one FLOAT plane (C path)."""
        src = np.ascontiguousarray(src, dtype=np.float32)
        h, w = src.shape
        out = np.zeros((orig_h, orig_w), np.float32)
        rc = self.lib.orc_unresize_plane(w, h, orig_w, orig_h, shift_w, shift_h, src.ctypes.data, src.strides[0],
                                         out.ctypes.data, out.strides[0])
        if rc:
            raise ValueError(f"unresize not available ({rc})")
        return out

    def depth_mode(self, fin: PixelFormat, fout: PixelFormat, dither="none") -> int:
        """0 copy, 1 left shift, 2 to float, 3 dither; negative: not converted."""
        a, b = _pixfmt(fin), _pixfmt(fout)
        return self.lib.orc_depth_mode(C.byref(a), C.byref(b), DITHERS[dither])

    def depth_scale_offset(self, fin: PixelFormat, fout: PixelFormat):
        a, b = _pixfmt(fin), _pixfmt(fout)
        sc, of = C.c_float(), C.c_float()
        self.lib.orc_depth_scale_offset(C.byref(a), C.byref(b), C.byref(sc), C.byref(of))
        return sc.value, of.value

    def depth_convert(self, src: np.ndarray, fin: PixelFormat, fout: PixelFormat, dither="none",
                      plane=0) -> np.ndarray:
        """zimg's depth conversion of one plane (C path)."""
        src = np.ascontiguousarray(src, dtype=fin.dtype)
        h, w = src.shape
        out = np.zeros((h, w), fout.dtype)
        a, b = _pixfmt(fin), _pixfmt(fout)
        rc = self.lib.orc_depth_convert(C.byref(a), C.byref(b), DITHERS[dither], plane, w, h, src.ctypes.data,
                                        src.strides[0], out.ctypes.data, out.strides[0])
        if rc:
            raise ValueError(f"depth conversion not available ({rc})")
        return out

    def compute_filter(self, kind, src_dim, dst_dim, shift=0.0, width=None, a=math.nan, b=math.nan) -> FilterContext:
        width = float(src_dim if width is None else width)
        fw, rows = C.c_uint(), C.c_uint()
        rc = self.lib.orc_compute_filter(_f(kind), a, b, src_dim, dst_dim, shift, width, C.byref(fw), C.byref(rows),
                                         None, None, None, None)
        if rc:
            raise ValueError(f"compute_filter failed ({rc})")
        f32 = np.zeros((rows.value, fw.value), np.float32)
        i16 = np.zeros((rows.value, fw.value), np.int16)
        f64 = np.zeros((rows.value, fw.value), np.float64)
        left = np.zeros(rows.value, np.uint32)
        rc = self.lib.orc_compute_filter(_f(kind), a, b, src_dim, dst_dim, shift, width, C.byref(fw), C.byref(rows),
                                         f32.ctypes.data, i16.ctypes.data, left.ctypes.data, f64.ctypes.data)
        if rc:
            raise ValueError(f"compute_filter failed ({rc})")
        return FilterContext(fw.value, rows.value, f32, i16, left, f64)

    def plan_order(self, src_w, src_h, dst_w, dst_h, shift_w=0.0, shift_h=0.0, subwidth=None, subheight=None):
        order = (C.c_int * 2)()
        n = self.lib.orc_plan_order(src_w, src_h, dst_w, dst_h, shift_w, shift_h,
                                    float(src_w if subwidth is None else subwidth),
                                    float(src_h if subheight is None else subheight), order)
        return ["h" if order[i] else "v" for i in range(n)]

    def resize_plane(self, src: np.ndarray, dst_w: int, dst_h: int, kind, a=math.nan, b=math.nan, depth=None,
                     shift_w=0.0, shift_h=0.0, subwidth=None, subheight=None, mode="c", nthreads=1) -> np.ndarray:
        """mode: 'c' (zimg C path: u16 exact / f32 sequential without FMA),
        'fma' (f32 sequential with fused multiply-add), 'f64' (FP64 oracle)."""
        src = np.ascontiguousarray(src)
        h, w = src.shape
        if mode == "f64":
            t, src = T_F64, src.astype(np.float64)
            out = np.zeros((dst_h, dst_w), np.float64)
        elif src.dtype == np.uint16:
            t, out = T_U16, np.zeros((dst_h, dst_w), np.uint16)
        elif src.dtype == np.float32:
            t, out = T_F32, np.zeros((dst_h, dst_w), np.float32)
        else:
            raise TypeError(src.dtype)
        depth = (16 if t == T_U16 else 32) if depth is None else depth
        rc = self.lib.orc_resize_plane(t, depth, _f(kind), a, b, w, h, dst_w, dst_h, shift_w, shift_h,
                                       float(w if subwidth is None else subwidth),
                                       float(h if subheight is None else subheight),
                                       1 if mode == "fma" else 0, nthreads, src.ctypes.data, w, out.ctypes.data, dst_w)
        if rc:
            raise ValueError(f"resize failed ({rc})")
        return out

    def plan(self, src_w, src_h, dst_w, dst_h, kind, a=math.nan, b=math.nan, dtype=np.uint16, depth=None,
             shift_w=0.0, shift_h=0.0, subwidth=None, subheight=None, mode="c") -> "Plan":
        """A conversion planned once (filter contexts built) and run on many
        planes, each run on the calling thread (zimg_oracle.c orc_plan_*)."""
        t = T_U16 if np.dtype(dtype) == np.uint16 else T_F32
        depth = (16 if t == T_U16 else 32) if depth is None else depth
        h = self.lib.orc_plan_create(t, depth, _f(kind), a, b, src_w, src_h, dst_w, dst_h, shift_w, shift_h,
                                     float(src_w if subwidth is None else subwidth),
                                     float(src_h if subheight is None else subheight), 1 if mode == "fma" else 0)
        if not h:
            raise ValueError("plan failed")
        return Plan(self.lib, h, np.dtype(dtype), (dst_h, dst_w))

    def resize_pass(self, src: np.ndarray, horizontal: bool, dst_dim: int, kind, a=math.nan, b=math.nan, depth=None,
                    shift=0.0, subwidth=None, mode="c", nthreads=1) -> np.ndarray:
        src = np.ascontiguousarray(src)
        h, w = src.shape
        ow, oh = (dst_dim, h) if horizontal else (w, dst_dim)
        if mode == "f64":
            t, src = T_F64, src.astype(np.float64)
            out = np.zeros((oh, ow), np.float64)
        elif src.dtype == np.uint16:
            t, out = T_U16, np.zeros((oh, ow), np.uint16)
        else:
            t, out = T_F32, np.zeros((oh, ow), np.float32)
        depth = (16 if t == T_U16 else 32) if depth is None else depth
        sub = float((w if horizontal else h) if subwidth is None else subwidth)
        rc = self.lib.orc_resize_pass(t, depth, int(horizontal), _f(kind), a, b, w, h, dst_dim, shift, sub,
                                      1 if mode == "fma" else 0, nthreads, src.ctypes.data, w, out.ctypes.data, ow)
        if rc:
            raise ValueError(f"resize failed ({rc})")
        return out


class Plan:
    """One planned conversion of the restatement; run() resizes one plane on
    the calling thread (the foreign call releases the GIL, so Python threads
    run planes in parallel)."""

    def __init__(self, lib, handle, dtype, out_shape):
        self.lib, self.h, self.dtype, self.out_shape = lib, handle, dtype, out_shape
        self.tmp_size = int(lib.orc_plan_tmp_size(handle))

    def run(self, src: np.ndarray, out: np.ndarray, tmp: np.ndarray | None = None):
        it = self.dtype.itemsize
        if tmp is None and self.tmp_size:
            tmp = np.empty(self.tmp_size, np.uint8)
        rc = self.lib.orc_plan_run(self.h, src.ctypes.data, src.strides[0] // it, out.ctypes.data,
                                   out.strides[0] // it, None if tmp is None else tmp.ctypes.data)
        if rc:
            raise ValueError(f"plan run failed ({rc})")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_plan_free(self.h)
            self.h = None


class Reference:
    """zimg's own code, compiled from the reference checkout (oracle/_ref)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        self.err = C.create_string_buffer(512)
        L.ref_filter_eval.argtypes = [C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_size_t,
                                      C.POINTER(C.c_uint), C.c_char_p, C.c_size_t]
        L.ref_compute_filter.argtypes = [C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint, C.c_double,
                                         C.c_double, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
        L.ref_plan_create.restype = C.c_void_p
        L.ref_plan_create.argtypes = [C.c_int, C.c_uint, C.c_int, C.c_double, C.c_double, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                      C.c_char_p, C.c_size_t]
        L.ref_pass_create.restype = C.c_void_p
        L.ref_pass_create.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_int, C.c_uint, C.c_uint, C.c_int, C.c_double,
                                      C.c_double, C.c_double, C.c_double, C.c_int, C.c_char_p, C.c_size_t]
        L.ref_plan_free.argtypes = [C.c_void_p]
        L.ref_unresize_plane.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_int,
                                         C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t, C.c_char_p, C.c_size_t]
        L.ref_depth_convert.argtypes = [C.c_int, C.c_uint, C.c_int, C.c_int, C.c_int, C.c_uint, C.c_int, C.c_int,
                                        C.c_int, C.c_uint, C.c_int, C.c_uint, C.c_uint, C.c_void_p, C.c_ssize_t,
                                        C.c_void_p, C.c_ssize_t, C.c_char_p, C.c_size_t]
        L.ref_plan_num_passes.argtypes = [C.c_void_p]
        L.ref_plan_run.argtypes = [C.c_void_p, C.c_void_p, C.c_ssize_t, C.c_void_p, C.c_ssize_t, C.c_char_p,
                                   C.c_size_t]

    def _raise(self, what):
        raise ValueError(f"{what}: {self.err.value.decode(errors='replace')}")

    def filter_eval(self, kind, x, a=math.nan, b=math.nan):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        sup = C.c_uint()
        if self.lib.ref_filter_eval(_f(kind), a, b, x.ctypes.data, y.ctypes.data, x.size, C.byref(sup), self.err, 512):
            self._raise("filter")
        return y, sup.value

    def compute_filter(self, kind, src_dim, dst_dim, shift=0.0, width=None, a=math.nan, b=math.nan) -> FilterContext:
        width = float(src_dim if width is None else width)
        fw, rows, iw = C.c_uint(), C.c_uint(), C.c_uint()
        args = (_f(kind), a, b, src_dim, dst_dim, shift, width, C.byref(fw), C.byref(rows), C.byref(iw))
        if self.lib.ref_compute_filter(*args, None, None, None, self.err, 512):
            self._raise("compute_filter")
        f32 = np.zeros((rows.value, fw.value), np.float32)
        i16 = np.zeros((rows.value, fw.value), np.int16)
        left = np.zeros(rows.value, np.uint32)
        if self.lib.ref_compute_filter(*args, f32.ctypes.data, i16.ctypes.data, left.ctypes.data, self.err, 512):
            self._raise("compute_filter")
        return FilterContext(fw.value, rows.value, f32, i16, left)

    def plan(self, pixel_type, depth, kind, src_w, src_h, dst_w, dst_h, a=math.nan, b=math.nan, shift_w=0.0,
             shift_h=0.0, subwidth=None, subheight=None, cpu=0):
        p = self.lib.ref_plan_create(pixel_type, depth, _f(kind), a, b, src_w, src_h, dst_w, dst_h, shift_w,
                                     shift_h, float(src_w if subwidth is None else subwidth),
                                     float(src_h if subheight is None else subheight), cpu, self.err, 512)
        if not p:
            self._raise("plan")
        return p

    def run(self, plan, src: np.ndarray, out: np.ndarray):
        """Run on whole planes. The SIMD filters want 64-byte aligned lines
        (align.h:11-20, filtergraph.cpp:188-216), so both planes are staged in
        aligned, padded buffers."""
        s = aligned_plane(*src.shape, src.dtype)
        s[...] = src
        d = aligned_plane(*out.shape, out.dtype)
        if self.lib.ref_plan_run(plan, s.ctypes.data, s.strides[0], d.ctypes.data, d.strides[0], self.err, 512):
            self._raise("run")
        out[...] = d

    def free(self, plan):
        self.lib.ref_plan_free(plan)

    def resize_plane(self, src: np.ndarray, dst_w, dst_h, kind, a=math.nan, b=math.nan, depth=None, shift_w=0.0,
                     shift_h=0.0, subwidth=None, subheight=None, cpu=0) -> np.ndarray:
        src = np.ascontiguousarray(src)
        h, w = src.shape
        t = 1 if src.dtype == np.uint16 else 3
        depth = (16 if t == 1 else 32) if depth is None else depth
        p = self.plan(t, depth, kind, w, h, dst_w, dst_h, a, b, shift_w, shift_h, subwidth, subheight, cpu)
        try:
            out = np.zeros((dst_h, dst_w), src.dtype)
            self.run(p, src, out)
        finally:
            self.free(p)
        return out

    def resize_pass(self, src: np.ndarray, horizontal, dst_dim, kind, a=math.nan, b=math.nan, depth=None,
                    shift=0.0, subwidth=None, cpu=0) -> np.ndarray:
        src = np.ascontiguousarray(src)
        h, w = src.shape
        t = 1 if src.dtype == np.uint16 else 3
        depth = (16 if t == 1 else 32) if depth is None else depth
        sub = float((w if horizontal else h) if subwidth is None else subwidth)
        p = self.lib.ref_pass_create(int(horizontal), w, h, t, depth, dst_dim, _f(kind), a, b, shift, sub, cpu,
                                     self.err, 512)
        if not p:
            self._raise("pass")
        try:
            ow, oh = (dst_dim, h) if horizontal else (w, dst_dim)
            out = np.zeros((oh, ow), src.dtype)
            self.run(p, src, out)
        finally:
            self.free(p)
        return out


def _ref_depth_convert(self, src: np.ndarray, fin: PixelFormat, fout: PixelFormat, dither="none", plane=0,
                       cpu=0) -> np.ndarray:
    """zimg's own DepthConversion (src/zimg/depth/depth.cpp:43-66) on one plane."""
    src = np.ascontiguousarray(src, dtype=fin.dtype)
    h, w = src.shape
    s = aligned_plane(h, w, fin.dtype)
    s[...] = src
    d = aligned_plane(h, w, fout.dtype)
    if self.lib.ref_depth_convert(fin.code, fin.bits, int(fin.fullrange), int(fin.chroma), fout.code, fout.bits,
                                  int(fout.fullrange), int(fout.chroma), DITHERS[dither], plane, cpu, w, h,
                                  s.ctypes.data, s.strides[0], d.ctypes.data, d.strides[0], self.err, 512):
        self._raise("depth_convert")
    return np.array(d)


Reference.depth_convert = _ref_depth_convert


def _ref_unresize_plane(self, src: np.ndarray, orig_w: int, orig_h: int, shift_w=0.0, shift_h=0.0,
                        cpu=0) -> np.ndarray:
    """zimg's own UnresizeConversion (src/zimg/unresize/unresize.cpp:34-91)."""
    src = np.ascontiguousarray(src, dtype=np.float32)
    h, w = src.shape
    s = aligned_plane(h, w, np.float32)
    s[...] = src
    d = aligned_plane(orig_h, orig_w, np.float32)
    if self.lib.ref_unresize_plane(w, h, orig_w, orig_h, shift_w, shift_h, cpu, s.ctypes.data, s.strides[0],
                                   d.ctypes.data, d.strides[0], self.err, 512):
        self._raise("unresize")
    return np.array(d)


Reference.unresize_plane = _ref_unresize_plane


def aligned_plane(h: int, w: int, dtype) -> np.ndarray:
    """[h, w] view with a 64-byte aligned base, 64-byte multiple stride and a
    spare line plus 256 bytes of tail padding."""
    dtype = np.dtype(dtype)
    stride = (w * dtype.itemsize + 63) // 64 * 64
    raw = np.zeros(stride * (h + 1) + 64 + 256, np.uint8)
    off = (-raw.ctypes.data) % 64
    base = raw[off:off + stride * (h + 1)]
    return np.lib.stride_tricks.as_strided(base.view(dtype), shape=(h, w), strides=(stride, dtype.itemsize))


def reference_available() -> bool:
    return os.path.exists(REF_SO)


# ---------------------------------------------------------------------------
# Graph-level parameter mapping (graphbuilder.cpp), restated for the checker.
# ---------------------------------------------------------------------------

def chroma_offset_w(loc_left: bool, subsampling: float) -> float:
    """graphbuilder.cpp:65-88"""
    return -0.5 + 0.5 * subsampling if loc_left else 0.0


def chroma_offset_h(loc: str, subsampling: float) -> float:
    """graphbuilder.cpp:90-110; loc in {'top','center','bottom'}"""
    if loc == "top":
        return -0.5 + 0.5 * subsampling
    if loc == "bottom":
        return 0.5 - 0.5 * subsampling
    return 0.0


def chroma_parity_adjustment(parity: str, offset: float) -> float:
    """graphbuilder.cpp:112-165"""
    if parity == "top":
        return -0.25 + offset / 2
    if parity == "bottom":
        return 0.25 + offset / 2
    return offset


def luma_parity_offset(parity: str) -> float:
    """graphbuilder.cpp:167-188"""
    return -0.25 if parity == "top" else (0.25 if parity == "bottom" else 0.0)


# zimg_chroma_location_e -> (w is LEFT, h location) (zimg.cpp:214-236)
CHROMA_LOC = {0: (True, "center"), 1: (False, "center"), 2: (True, "top"), 3: (False, "top"),
              4: (True, "bottom"), 5: (False, "bottom")}
PARITY = {0: "progressive", 1: "top", 2: "bottom"}


def plane_geometry(fmt: dict) -> list[dict]:
    """Per-plane (width, height, active_left/top/width/height) after siting,
    for a format dict with keys width, height, subsample_w, subsample_h, color
    ('grey'|'yuv'|'rgb'), chroma_location, field_parity, active_region (4 floats
    or NaN). Follows zimg.cpp:388-397 and graphbuilder.cpp:331-366."""
    w, h = fmt["width"], fmt["height"]
    ar = fmt.get("active_region", (math.nan,) * 4)
    al = 0.0 if math.isnan(ar[0]) else ar[0]
    at = 0.0 if math.isnan(ar[1]) else ar[1]
    aw = float(w) if math.isnan(ar[2]) else ar[2]
    ah = float(h) if math.isnan(ar[3]) else ar[3]
    planes = [dict(width=w, height=h, left=al, top=at, aw=aw, ah=ah)]
    color = fmt.get("color", "grey")
    if color != "grey":
        sw, sh = fmt.get("subsample_w", 0), fmt.get("subsample_h", 0)
        ssw, ssh = 1.0 / (1 << sw), 1.0 / (1 << sh)
        u = dict(width=w >> sw, height=h >> sh, left=al * ssw, top=at * ssh, aw=aw * ssw, ah=ah * ssh)
        planes += [dict(u), dict(u)]
    parity = PARITY[fmt.get("field_parity", 0)]
    planes[0]["top"] -= luma_parity_offset(parity)
    if color != "grey":
        loc_left, loc_h = CHROMA_LOC[fmt.get("chroma_location", 0)]
        subscale_w = planes[1]["width"] / planes[0]["width"]
        subscale_h = planes[1]["height"] / planes[0]["height"]
        off_w = chroma_offset_w(loc_left, subscale_w)
        off_h = chroma_parity_adjustment(parity, chroma_offset_h(loc_h, subscale_h))
        for p in (1, 2):
            planes[p]["left"] -= off_w
            planes[p]["top"] -= off_h
    return planes


def resize_params(src_plane: dict, dst_plane: dict) -> dict:
    """graphbuilder.cpp:769-776"""
    scale_w = dst_plane["aw"] / src_plane["aw"]
    scale_h = dst_plane["ah"] / src_plane["ah"]
    return dict(src_w=src_plane["width"], src_h=src_plane["height"], dst_w=dst_plane["width"],
                dst_h=dst_plane["height"],
                shift_w=src_plane["left"] - dst_plane["left"] / scale_w,
                shift_h=src_plane["top"] - dst_plane["top"] / scale_h,
                subwidth=src_plane["aw"] * (dst_plane["width"] / dst_plane["aw"]),
                subheight=src_plane["ah"] * (dst_plane["height"] / dst_plane["ah"]))


def resize_format(fs: PixelFormat, fd: PixelFormat, src_pels: float, dst_pels: float) -> PixelFormat:
    """The format zimg's graph resizes a plane in (choose_resize_format,
    src/zimg/graph/graphbuilder.cpp:720-751), resize supporting WORD and FLOAT."""
    sup = ("word", "float")
    if fs.type in sup and fd.type in sup:
        return fd if src_pels < dst_pels else fs
    if fs.type in sup:
        return fs
    if fd.type in sup:
        return fd
    if fs.type == "byte" and not fs.fullrange:
        return PixelFormat("word", 16, False, fs.chroma)
    return PixelFormat("float")


def graph_plane_chain(o: "Oracle", src: np.ndarray, fs: PixelFormat, fd: PixelFormat, rp: dict | None, kind,
                      a=math.nan, b=math.nan, dither="none", plane=0) -> np.ndarray:
    """One plane through zimg's graph (connect_plane, graphbuilder.cpp:892-953):
    full-range BYTE kept at its depth reinterpreted as limited range, a depth
    conversion into the resize format, the resize (rp: resize_params(); None
    when the geometry is unchanged), a depth conversion to the output format.
    FP32 resizes use the sequential fused multiply-add order (mode "fma") that
    the GPU's CUDA-core kernels follow bit for bit; u16 ones zimg's C path."""
    import dataclasses
    if fs.type == "byte" and fs.fullrange and fd.fullrange and fs.bits == fd.bits:
        fs = dataclasses.replace(fs, fullrange=False)
        fd = dataclasses.replace(fd, fullrange=False)
    if rp is None:
        return o.depth_convert(src, fs, fd, dither, plane)
    h, w = src.shape
    if kind == "unresize":  # FLOAT working format (graphbuilder.cpp:722-723,780-790)
        fr = PixelFormat("float")
        x = src if o.depth_mode(fs, fr, dither) == 0 else o.depth_convert(src, fs, fr, dither, plane)
        y = o.unresize_plane(x, rp["dst_w"], rp["dst_h"], rp["shift_w"], rp["shift_h"])
        return y if o.depth_mode(fr, fd, dither) == 0 else o.depth_convert(y, fr, fd, dither, plane)
    fr = resize_format(fs, fd, float(w * h), float(rp["dst_w"] * rp["dst_h"]))
    x = src if o.depth_mode(fs, fr, dither) == 0 else o.depth_convert(src, fs, fr, dither, plane)
    y = o.resize_plane(x.astype(fr.dtype), rp["dst_w"], rp["dst_h"], kind, a, b,
                       depth=fr.bits if fr.type == "word" else None, shift_w=rp["shift_w"], shift_h=rp["shift_h"],
                       subwidth=rp["subwidth"], subheight=rp["subheight"],
                       mode="c" if fr.type == "word" else "fma", nthreads=16)
    return y if o.depth_mode(fr, fd, dither) == 0 else o.depth_convert(y, fr, fd, dither, plane)


def _same_geometry(a: dict, b: dict) -> bool:
    return all(a[k] == b[k] for k in ("width", "height", "left", "top", "aw", "ah"))


def _float_resize(o: "Oracle", x: np.ndarray, src: dict, dst: dict, kind, a=math.nan, b=math.nan) -> np.ndarray:
    rp = resize_params(src, dst)
    return o.resize_plane(x.astype(np.float32), rp["dst_w"], rp["dst_h"], kind, a, b, shift_w=rp["shift_w"],
                          shift_h=rp["shift_h"], subwidth=rp["subwidth"], subheight=rp["subheight"], mode="fma",
                          nthreads=16)


def graph_straight_alpha(o: "Oracle", srcs: list, fs: list, fd: list, sgeo: list, dgeo: list, color: str,
                         kind, kind_uv, dither="none", a=math.nan, b=math.nan, a_uv=math.nan, b_uv=math.nan) -> list:
    """zimg's graph for straight alpha through an interpolating resize
    (connect_internal, src/zimg/graph/graphbuilder.cpp:1019-1068): srcs / fs /
    fd hold the colour planes then alpha (PixelFormats with alpha full range,
    chroma flags on YUV chroma), sgeo / dgeo plane_geometry() of the two
    formats. Every plane to FLOAT at the source luma geometry (chroma resized
    up with the chroma filter, make_float_444_state :446-457), colour times
    alpha as it is (PremultiplyFilter, simple_filters.cpp:76-89), all planes
    resized to the destination luma geometry (chroma with the chroma filter),
    colour divided by alpha clamped to [0, 1], 0 where that is 0
    (UnpremultiplyFilter :98-110), chroma resized to its own geometry, every
    plane converted to the output format. FP32 resizes in the sequential
    fused multiply-add order, as graph_plane_chain."""
    ncolor = len(srcs) - 1
    gs, gd = sgeo[0], dgeo[0]
    yuv = color == "yuv"

    def chroma(p):
        return yuv and p in (1, 2)

    def fl(p):
        return PixelFormat("float", None, False, chroma(p))

    def to_fmt(x, f_in, f_out, plane):
        return x if o.depth_mode(f_in, f_out, dither) == 0 else o.depth_convert(x, f_in, f_out, dither, plane)

    planes = []
    for k in range(ncolor + 1):
        p = 3 if k == ncolor else k
        g_src = sgeo[p] if chroma(p) else gs
        x = to_fmt(srcs[k], fs[k], fl(p), p).astype(np.float32)
        if chroma(p) and not _same_geometry(g_src, gs):
            x = _float_resize(o, x, g_src, gs, kind_uv, a_uv, b_uv)
        planes.append(x)
    al = planes[ncolor]
    for k in range(ncolor):
        planes[k] = (planes[k] * al).astype(np.float32)
    if not _same_geometry(gs, gd):
        planes = [_float_resize(o, x, gs, gd, kind_uv if chroma(3 if k == ncolor else k) else kind,
                                a_uv if chroma(3 if k == ncolor else k) else a,
                                b_uv if chroma(3 if k == ncolor else k) else b)
                  for k, x in enumerate(planes)]
    al = planes[ncolor]
    c = np.where(al < 0, np.float32(0), np.where(np.float32(1) < al, np.float32(1), al)).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in range(ncolor):
            planes[k] = np.where(c == 0, np.float32(0), planes[k] / c).astype(np.float32)
    out = []
    for k in range(ncolor + 1):
        p = 3 if k == ncolor else k
        x = planes[k]
        if chroma(p) and not _same_geometry(gd, dgeo[p]):
            x = _float_resize(o, x, gd, dgeo[p], kind_uv, a_uv, b_uv)
        out.append(to_fmt(x, fl(p), fd[k], p))
    return out


# ---------------------------------------------------------------- colorspace --
# zimg API codes (zimg.h:283-352) -> zimg's internal enum values
# (colorspace.h:19-60), as translate_matrix / _transfer / _primaries map them
# (zimg.cpp:238-305). Codes absent from the maps raise (NO_COLORSPACE_CONVERSION).
CSP_MATRIX = {0: 1, 1: 3, 2: 0, 4: 4, 5: 2, 6: 2, 7: 5, 8: 6, 9: 7, 10: 8, 12: 9, 13: 10, 14: 12}
CSP_TRANSFER = {1: 4, 2: 0, 7: 7, 6: 4, 4: 5, 5: 6, 11: 8, 12: 9, 13: 10, 14: 4, 15: 4, 8: 1, 9: 2, 10: 3,
                16: 11, 17: 12, 18: 13}
CSP_PRIMARIES = {4: 1, 5: 2, 1: 4, 2: 0, 6: 3, 7: 3, 8: 5, 9: 6, 10: 7, 11: 8, 12: 9, 22: 10}
CSP_OPS = ("matrix", "gamma", "hlg", "hlg_inverse", "cl_to_rgb", "cl_to_yuv")


def csp_internal(matrix: int, transfer: int, primaries: int) -> tuple:
    """API codes -> internal enum values; KeyError when zimg has no mapping."""
    return CSP_MATRIX[matrix], CSP_TRANSFER[transfer], CSP_PRIMARIES[primaries]


def _bind_colorspace(L):
    L.orc_colorspace_create.argtypes = [C.c_int] * 6 + [C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.orc_colorspace_create.restype = C.c_void_p
    L.orc_colorspace_free.argtypes = [C.c_void_p]
    L.orc_colorspace_num_ops.argtypes = [C.c_void_p]
    L.orc_colorspace_op.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
    L.orc_colorspace_run.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.POINTER(C.c_void_p), C.POINTER(C.c_ssize_t),
                                     C.POINTER(C.c_void_p), C.POINTER(C.c_ssize_t)]
    L.orc_colorspace_run_f64.argtypes = L.orc_colorspace_run.argtypes


def _planes_args(planes):
    ptrs = (C.c_void_p * 3)(*[p.ctypes.data for p in planes])
    strides = (C.c_ssize_t * 3)(*[p.strides[0] for p in planes])
    return ptrs, strides


def _orc_colorspace(self, planes, csp_in, csp_out, peak=100.0, approximate=False, scene=False, adapt=False,
                    fp64=False):
    """zimg's ColorspaceConversion (C path) on three FLOAT planes. csp_in /
    csp_out: (matrix, transfer, primaries) API codes. Returns (planes, ops):
    the converted planes and the names of the operations applied. fp64: the
    same operations with the same float parameters evaluated in double, into
    float64 planes (the reference float evaluations are measured against)."""
    L = self.lib
    if not getattr(L, "_csp_bound", False):
        _bind_colorspace(L)
        L._csp_bound = True
    err = C.c_int()
    h = L.orc_colorspace_create(*csp_internal(*csp_in), *csp_internal(*csp_out), float(peak), int(approximate),
                                int(scene), int(adapt), C.byref(err))
    if not h:
        raise ValueError(f"no colorspace conversion ({err.value})")
    try:
        ops = [CSP_OPS[L.orc_colorspace_op(h, k, None)] for k in range(L.orc_colorspace_num_ops(h))]
        src = [np.ascontiguousarray(p, dtype=np.float32) for p in planes]
        out = [np.empty(src[0].shape, np.float64 if fp64 else np.float32) for _ in range(3)]
        hh, ww = src[0].shape
        si, ss = _planes_args(src)
        di, ds = _planes_args(out)
        (L.orc_colorspace_run_f64 if fp64 else L.orc_colorspace_run)(h, ww, hh, si, ss, di, ds)
        if not ops:
            return ([p.astype(np.float64) for p in src] if fp64 else src), ops
        return out, ops
    finally:
        L.orc_colorspace_free(h)


def _ref_colorspace(self, planes, csp_in, csp_out, peak=100.0, approximate=False, scene=False, adapt=False, cpu=0):
    """zimg's own ColorspaceConversion (oracle/_ref) on three FLOAT planes."""
    L = self.lib
    if not getattr(L, "_csp_bound", False):
        L.ref_colorspace.argtypes = [C.c_int] * 6 + [C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint, C.c_uint,
                                                     C.POINTER(C.c_void_p), C.POINTER(C.c_ssize_t),
                                                     C.POINTER(C.c_void_p), C.POINTER(C.c_ssize_t), C.c_char_p,
                                                     C.c_size_t]
        L._csp_bound = True
    src = [np.ascontiguousarray(p, dtype=np.float32) for p in planes]
    out = [np.empty_like(src[0]) for _ in range(3)]
    hh, ww = src[0].shape
    si, ss = _planes_args(src)
    di, ds = _planes_args(out)
    err = C.create_string_buffer(256)
    rc = L.ref_colorspace(*csp_internal(*csp_in), *csp_internal(*csp_out), float(peak), int(approximate), int(scene),
                          int(adapt), cpu, ww, hh, si, ss, di, ds, err, 256)
    if rc == 3:
        return src
    if rc:
        raise ValueError(err.value.decode())
    return out


Oracle.colorspace = _orc_colorspace
Reference.colorspace = _ref_colorspace


def graph_colorspace(o: "Oracle", srcs: list, fs: list, fd: list, sgeo: list, dgeo: list, scolor: str, dcolor: str,
                     csp_in: tuple, csp_out: tuple, kind, kind_uv, dither="none", **kw) -> list:
    """zimg's graph for a colorspace change (connect_color_channels,
    src/zimg/graph/graphbuilder.cpp:975-1014): every colour plane to FLOAT
    4:4:4 at the work geometry (each dimension from the smaller side's luma
    plane, :982-991; chroma with the chroma filter), a GREY source read as
    RGB with equal planes, the colorspace conversion (csp_in / csp_out API
    codes, the GREY source's matrix taken as RGB), then each output plane
    from the work planes to its geometry and format. srcs / fs: the source's
    colour planes and formats; fd: the output planes' formats (one for GREY)."""
    sy, dy = sgeo[0], dgeo[0]
    w_src, h_src = (sy if sy["width"] < dy["width"] else dy), (sy if sy["height"] < dy["height"] else dy)
    gw = dict(width=w_src["width"], left=w_src["left"], aw=w_src["aw"],
              height=h_src["height"], top=h_src["top"], ah=h_src["ah"])

    def chain(x, g_from, g_to, f_from, f_to, k, plane):
        rp = None if _same_geometry(g_from, g_to) else resize_params(g_from, g_to)
        return graph_plane_chain(o, x, f_from, f_to, rp, k, dither=dither, plane=plane)

    work = []
    for p, (x, f) in enumerate(zip(srcs, fs)):
        uv = scolor == "yuv" and p > 0
        g_from = sgeo[p] if scolor == "yuv" else sy
        work.append(chain(x, g_from, gw, f, PixelFormat("float", None, False, uv), kind_uv if uv else kind, p)
                    .astype(np.float32))
    while len(work) < 3:
        work.append(work[0].copy())
    cin = ((csp_out[0] if dcolor == "rgb" else 0),) + tuple(csp_in[1:]) if scolor == "grey" else csp_in
    conv, _ = o.colorspace(work, cin, csp_out, **kw)
    yuv_work = csp_out[0] != 0
    out = []
    for p, f in enumerate(fd):
        uv = dcolor == "yuv" and p > 0
        g_to = dgeo[p] if dcolor == "yuv" else dy
        out.append(chain(conv[p], gw, g_to, PixelFormat("float", None, False, p > 0 and yuv_work), f,
                         kind_uv if uv else kind, p))
    return out
