"""Negative strides (bottom-up planes), which zimg_image_buffer allows
(zimg.h:387-433): line i of a plane is at data + i * stride. Every engine,
the identity copy, a batch and the depth conversion, through the C ABI,
against the oracle on the same logical planes."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class BottomUp:
    """A device plane stored bottom-up: logical line i at base + i * (-pitch)."""

    def __init__(self, h, w, np_dtype, host=None):
        import torch
        tdt = {np.uint8: torch.uint8, np.uint16: torch.int16, np.float32: torch.float32}[np_dtype]
        self.h, self.w, self.dtype = h, w, np_dtype
        self.buf = torch.zeros((h, w), dtype=tdt, device="cuda")
        if host is not None:
            flipped = np.ascontiguousarray(host[::-1])
            self.buf.copy_(torch.from_numpy(flipped.view(np.int16) if np_dtype == np.uint16 else flipped))
        self.pitch = w * np.dtype(np_dtype).itemsize
        self.ptr = self.buf.data_ptr() + (h - 1) * self.pitch
        self.stride = -self.pitch

    def host(self):
        a = self.buf.cpu().numpy()
        if self.dtype == np.uint16:
            a = a.view(np.uint16)
        return np.ascontiguousarray(a[::-1])


class TopDown(BottomUp):
    def __init__(self, h, w, np_dtype, host=None):
        super().__init__(h, w, np_dtype)
        import torch
        if host is not None:
            self.buf.copy_(torch.from_numpy(host.view(np.int16) if np_dtype == np.uint16 else np.ascontiguousarray(host)))
        self.ptr = self.buf.data_ptr()
        self.stride = self.pitch

    def host(self):
        a = self.buf.cpu().numpy()
        return a.view(np.uint16) if self.dtype == np.uint16 else a


def resize(lib, conv, src_plane, dst_plane):
    import torch
    r = conv.create()
    tmp = torch.empty(max(r.tmp_size, 1), dtype=torch.uint8, device="cuda")
    rc = lib.zg_resize_process(r.handle, src_plane.ptr, src_plane.stride, dst_plane.ptr, dst_plane.stride,
                               tmp.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return r


CASES = [
    # (src w, h, dst w, h, type, filter, a, fusion, engine, src bottom-up, dst bottom-up)
    (480, 270, 960, 540, "word", "lanczos", 3, True, "auto", True, True),      # chained tensor-core kernel
    (720, 480, 480, 320, "word", "spline36", math.nan, True, "auto", True, False),
    (480, 270, 960, 540, "word", "lanczos", 3, False, "cuda", True, True),     # separate passes via tmp
    (640, 360, 427, 240, "float", "bicubic", math.nan, True, "cuda", True, False),  # fused CUDA-core kernel
    (1920, 1080, 120, 68, "float", "lanczos", 4, True, "auto", True, True),   # tensor-core passes (64 taps)
    (300, 200, 300, 200, "word", "bicubic", math.nan, True, "auto", True, False),   # identity: a copy
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_resize_bottom_up_planes(cuda, lib, oracle, case):
    import zimg_gb300 as zg
    sw, sh, dw, dh, ptype, kind, a, fusion, engine, s_up, d_up = CASES[case]
    rng = np.random.default_rng(800 + case)
    dt = np.uint16 if ptype == "word" else np.float32
    src = rng.integers(0, 1024, size=(sh, sw)).astype(np.uint16) if ptype == "word" else \
        rng.random((sh, sw), dtype=np.float32)
    sp = (BottomUp if s_up else TopDown)(sh, sw, dt, src)
    dp = (BottomUp if d_up else TopDown)(dh, dw, dt)
    conv = zg.ResizeConversion(sw, sh, ptype).set_filter(kind, a).set_dst_width(dw).set_dst_height(dh) \
        .set_fusion(fusion).set_engine(engine)
    if ptype == "word":
        conv.set_depth(10)
    r = resize(lib, conv, sp, dp)
    got = dp.host()
    if ptype == "word":
        want = oracle.resize_plane(src, dw, dh, kind, a, depth=10, mode="c", nthreads=8)
        np.testing.assert_array_equal(got, want, err_msg=str(CASES[case]))
    elif r.info["engine"] == "cuda":
        want = oracle.resize_plane(src, dw, dh, kind, a, mode="fma", nthreads=8)
        np.testing.assert_array_equal(got, want, err_msg=str(CASES[case]))
    else:
        # tensor-core passes: against FP64 within the FP32 engines' bound
        ref = oracle.resize_plane(src, dw, dh, kind, a, mode="f64", nthreads=8)
        c = oracle.resize_plane(src, dw, dh, kind, a, mode="c", nthreads=8)
        bound = 2 * float(np.max(np.abs(c.astype(np.float64) - ref))) + 1e-6
        assert float(np.max(np.abs(got.astype(np.float64) - ref))) <= bound


def test_batch_bottom_up_planes(cuda, lib, oracle):
    import torch
    import zimg_gb300 as zg
    from zimg_gb300 import capi
    rng = np.random.default_rng(77)
    shapes = [(480, 270, 960, 540), (320, 180, 200, 120), (256, 144, 256, 144)]
    convs, planes, wants = [], [], []
    for k, (sw, sh, dw, dh) in enumerate(shapes):
        src = rng.integers(0, 1024, size=(sh, sw)).astype(np.uint16)
        convs.append(zg.ResizeConversion(sw, sh, "word").set_depth(10).set_filter("spline36")
                     .set_dst_width(dw).set_dst_height(dh))
        planes.append((BottomUp(sh, sw, np.uint16, src), (BottomUp if k % 2 == 0 else TopDown)(dh, dw, np.uint16)))
        wants.append(oracle.resize_plane(src, dw, dh, "spline36", depth=10, mode="c", nthreads=8))
    b = zg.Batch(convs)
    io = (capi.BatchIO * len(shapes))()
    for i, (s, d) in enumerate(planes):
        io[i] = capi.BatchIO(s.ptr, s.stride, d.ptr, d.stride)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.zg_batch_set_io(b._h, io, stream) == 0
    tmp = torch.empty(max(b.tmp_size, 1), dtype=torch.uint8, device="cuda")
    b.process(tmp)
    torch.cuda.synchronize()
    for (s, d), w in zip(planes, wants):
        np.testing.assert_array_equal(d.host(), w)


def test_depth_bottom_up_planes(cuda, lib, oracle):
    import torch
    import zimg_gb300 as zg
    from oracle.oracle import PixelFormat as PF
    rng = np.random.default_rng(78)
    h, w = 97, 203
    src = rng.random((h, w), dtype=np.float32)
    c = zg.DepthConversion(w, h).set_pixel_in("float").set_pixel_out("byte", 8).set_dither_type("ordered").create()
    for s_up, d_up in ((True, True), (True, False), (False, True)):
        sp = (BottomUp if s_up else TopDown)(h, w, np.float32, src)
        dp = (BottomUp if d_up else TopDown)(h, w, np.uint8)
        rc = lib.zg_depth_process(c._h, sp.ptr, sp.stride, dp.ptr, dp.stride, torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        want = oracle.depth_convert(src, PF("float"), PF("byte", 8), "ordered", 0)
        np.testing.assert_array_equal(dp.host(), want, err_msg=str((s_up, d_up)))


def test_stride_below_a_line_still_rejected(cuda, lib):
    import torch
    import zimg_gb300 as zg
    r = zg.ResizeConversion(64, 32, "word").set_depth(10).set_dst_width(128).set_dst_height(64).create()
    buf = torch.zeros(64 * 128 * 2, dtype=torch.uint8, device="cuda")
    rc = lib.zg_resize_process(r.handle, buf.data_ptr() + 31 * 100, -100, buf.data_ptr(), 256, None,
                               torch.cuda.current_stream().cuda_stream)
    assert rc == 2048  # |stride| below 64 samples of 2 bytes: ILLEGAL_ARGUMENT
