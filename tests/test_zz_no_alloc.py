"""zg_resize_process_no_alloc: the conversion entry point for callers that
cannot allocate device memory when they process a frame (for example a
video-filter host that only hands its plugins frame buffers from its own pool,
or a real-time loop that must avoid cudaMalloc/cudaFree and the device-wide
synchronisation they imply).

It runs the same two-pass kernels as zg_resize_process, but keeps the
intermediate plane in the library's built-in scratch array instead of a
caller-provided tmp buffer. These tests call it through the C ABI and compare
it with zg_resize_process on two calls in a row, bit for bit (the tolerance
the other parity tests use for both u16 and the f32 CUDA-core path). This file
is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NO_ALLOC_TMP_BYTES = 32 << 20  # ZG_NO_ALLOC_TMP_BYTES in include/zimg_gb300.h


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a.view(np.int16) if a.dtype == np.uint16 else a)).cuda()


def _plane(t):
    return t.data_ptr(), t.stride(0) * t.element_size()


def _two_pass(zg, w, h, dw, dh, ptype, kind, a, b, depth):
    conv = zg.ResizeConversion(w, h, ptype).set_filter(kind, a, b).set_dst_width(dw).set_dst_height(dh) \
        .set_depth(depth).set_fusion(False).set_engine("cuda")
    r = conv.create()
    assert r.info["num_passes"] == 2
    assert 0 < r.tmp_size <= NO_ALLOC_TMP_BYTES
    return r


@pytest.mark.parametrize("case", [
    ("word", 10, 480, 270, 960, 540, "lanczos", 3.0, float("nan")),
    ("float", 32, 1920, 1080, 1280, 720, "bicubic", 0.0, 0.5),
])
def test_no_alloc_matches_caller_tmp_twice(cuda, case):
    import torch
    import zimg_gb300 as zg
    lib = zg.load()
    ptype, depth, w, h, dw, dh, kind, a, b = case
    r = _two_pass(zg, w, h, dw, dh, ptype, kind, a, b, depth)
    rng = np.random.default_rng(2024)
    tdt = torch.int16 if ptype == "word" else torch.float32
    stream = torch.cuda.current_stream().cuda_stream
    tmp = torch.empty(r.tmp_size, dtype=torch.uint8, device="cuda")

    for call in range(2):  # two calls in a row, different inputs, same static scratch
        if ptype == "word":
            src = _dev(rng.integers(0, 1 << depth, size=(h, w), dtype=np.uint16))
        else:
            src = _dev(rng.random((h, w), dtype=np.float32))
        want = torch.zeros((dh, dw), dtype=tdt, device="cuda")
        got = torch.full((dh, dw), -1, dtype=tdt, device="cuda")
        sp, ss = _plane(src)
        wp, ws = _plane(want)
        gp, gs = _plane(got)
        assert lib.zg_resize_process(r.handle, sp, ss, wp, ws, tmp.data_ptr(), stream) == 0
        assert lib.zg_resize_process_no_alloc(r.handle, sp, ss, gp, gs, stream) == 0
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call}: outputs differ"


def test_no_alloc_rejects_oversized_scratch(cuda):
    import torch
    import zimg_gb300 as zg
    from zimg_gb300 import capi
    lib = zg.load()
    conv = zg.ResizeConversion(4096, 4096, "float").set_filter("bilinear").set_dst_width(8192) \
        .set_dst_height(8192).set_fusion(False).set_engine("cuda")
    r = conv.create()
    assert r.tmp_size > NO_ALLOC_TMP_BYTES
    src = torch.zeros((4, 4), dtype=torch.float32, device="cuda")  # never touched: the call is rejected first
    rc = lib.zg_resize_process_no_alloc(r.handle, src.data_ptr(), 16 * 4096, src.data_ptr(), 16 * 8192,
                                        torch.cuda.current_stream().cuda_stream)
    assert rc == 1  # ZG_ERROR_OUT_OF_MEMORY
    code, msg = capi.last_error()
    assert code == 1 and "static scratch" in msg

