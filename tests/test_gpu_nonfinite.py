"""Non-finite FP32 samples: what the GPU kernels do with NaN and infinities.

zimg's C path (resize_impl.cpp:61-114) multiplies each output's own taps
[left, left + filter_width) with the samples under them, so a NaN or an
infinity reaches exactly the outputs whose taps cover it (an infinity under
taps of both signs, or next to another of opposite sign, becomes NaN).

The GPU kernels compute dense windows: the fused CUDA-core kernel's groups of
output rows, the tensor-core kernels' 16-wide tiles and 8-output blocks. A
window's other outputs multiply the sample by an exact zero tap, and
0 * NaN = 0 * inf = NaN, so a non-finite sample also reaches the other
outputs of its windows. The documented behaviour, pinned here per engine:

  * every output that zimg's C path gives as non-finite is non-finite here;
  * every output that is finite here equals the oracle's (bit for bit on the
    CUDA-core kernels in FMA order; within the FP64 bound on the tensor-core
    passes);
  * the extra non-finite outputs lie within SPREAD[engine] output samples
    (in rows and columns) of one that zimg gives as non-finite: 8 for the
    separate CUDA-core passes (those of fewer than 32 taps use each output's
    own taps and give exactly zimg's non-finite outputs; wider ones compute
    groups of 8 output rows or 4 output columns over a dense window); 4 for
    the fused CUDA-core kernel's row groups; 32 for the tensor-core passes'
    tiles and blocks.
"""
import math

import numpy as np
import pytest

from test_gpu_resize import band_limited, run_conversion

pytestmark = pytest.mark.gpu

SPREAD = {"cuda": 8, "fused": 4, "tensor": 32}


def _inject(rng, src, n=6):
    src = src.copy()
    h, w = src.shape
    vals = [np.nan, np.inf, -np.inf]
    for k in range(n):
        y, x = int(rng.integers(8, h - 8)), int(rng.integers(8, w - 8))
        src[y, x] = vals[k % 3]
    return src


def _dilate(mask, r):
    out = mask.copy()
    ys, xs = np.nonzero(mask)
    for y, x in zip(ys, xs):
        out[max(0, y - r):y + r + 1, max(0, x - r):x + r + 1] = True
    return out


def _check(oracle, src, dw, dh, kind, a, b, engine, fusion, exact):
    got, r = run_conversion(src, dw, dh, kind, a, b, engine=engine, fusion=fusion)
    want = oracle.resize_plane(src, dw, dh, kind, a, b, mode="fma" if exact else "c", nthreads=16)
    A = ~np.isfinite(want)
    B = ~np.isfinite(got)
    spread = SPREAD["tensor" if engine == "tensor" else ("fused" if r.info["engine"] == "cuda" else "cuda")]
    assert A.any(), "the injected samples must reach some outputs"
    assert np.all(B[A]), f"{r.info}: outputs non-finite in zimg's C path are finite here"
    assert np.all(_dilate(A, spread)[B]), f"{r.info}: a non-finite sample spread beyond {spread} outputs"
    fin = ~B
    if exact:
        np.testing.assert_array_equal(got[fin].view(np.uint32), want[fin].view(np.uint32), err_msg=str(r.info))
    else:
        clean = np.where(np.isfinite(src), src, 0).astype(np.float32)
        f64 = oracle.resize_plane(clean, dw, dh, kind, a, b, mode="f64", nthreads=16)
        c = oracle.resize_plane(clean, dw, dh, kind, a, b, mode="c", nthreads=16)
        bound = 2 * float(np.max(np.abs(c.astype(np.float64) - f64))) + 1e-6
        np.testing.assert_allclose(got[fin], want[fin], rtol=0, atol=2 * bound, err_msg=str(r.info))
    return r.info


@pytest.mark.parametrize("engine,fusion,exact", [("cuda", True, True), ("cuda", False, True),
                                                 ("tensor", True, False)])
def test_nonfinite_bicubic_down(cuda, oracle, engine, fusion, exact):
    rng = np.random.default_rng(0x4E4E)
    src = _inject(rng, rng.random((540, 960), dtype=np.float32))
    _check(oracle, src, 640, 360, "bicubic", 0.0, 0.5, engine, fusion, exact)


@pytest.mark.parametrize("engine,fusion,exact", [("cuda", True, True), ("cuda", False, True),
                                                 ("tensor", True, False)])
def test_nonfinite_lanczos_up(cuda, oracle, engine, fusion, exact):
    rng = np.random.default_rng(0x4E4F)
    src = _inject(rng, rng.random((270, 480), dtype=np.float32))
    _check(oracle, src, 960, 540, "lanczos", 3, math.nan, engine, fusion, exact)


@pytest.mark.parametrize("engine,exact", [("cuda", True), ("tensor", False)])
def test_nonfinite_wide_down(cuda, oracle, engine, exact):
    rng = np.random.default_rng(0x4E50)
    src = _inject(rng, band_limited(rng, 1080, 1920))
    _check(oracle, src, 120, 67, "lanczos", 4, math.nan, engine, True, exact)
