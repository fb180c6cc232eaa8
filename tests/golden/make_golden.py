"""Generate tests/golden/resize_golden.npz from zimg's own resize code.

Run in a checkout that has the reference sources (oracle/Makefile compiles them
into oracle/_ref/libzimgref.so):

    make -C oracle && python tests/golden/make_golden.py

Every input is seeded, so the fixture is reproducible. Contents:

* ``kernel/*``  filter kernel values f(x) at fixed points (filter.cpp:132-246)
* ``ctx/*``     FilterContexts (compute_filter, filter.cpp:249-306) for a sweep
                of filters, ratios, shifts and active widths
* ``plane/*``   whole-plane resizes through ResizeConversion with the C path
                (CPUClass::NONE), u16 at several depths and f32, plus a flag
                saying whether zimg's SIMD path gave the same u16 bytes
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402

OUT = os.path.join(HERE, "resize_golden.npz")

KERNELS = [("point", math.nan, math.nan), ("bilinear", math.nan, math.nan), ("bicubic", math.nan, math.nan),
           ("bicubic", 1 / 3, 1 / 3), ("bicubic", 1.0, 0.0), ("spline16", math.nan, math.nan),
           ("spline36", math.nan, math.nan), ("spline64", math.nan, math.nan), ("lanczos", 1, math.nan),
           ("lanczos", 3, math.nan), ("lanczos", 4, math.nan), ("lanczos", 15, math.nan)]

BIG_KERNELS = {("lanczos", 3), ("lanczos", 4), ("spline36", math.nan), ("bicubic", math.nan)}
CTX_CASES = []
for k, a, b in KERNELS:
    for src, dst in [(640, 1344), (640, 305), (1920, 3840), (1920, 1280), (1080, 720), (7680, 480), (6400, 64),
                     (64, 6400), (720, 1920), (480, 1080), (1, 5), (5, 1), (3, 3), (100, 100)]:
        for shift, subf in [(0.0, 1.0), (3.3, 0.75), (-3.3, 1.05), (0.25, 1.0), (-0.25, 1.0)]:
            big = src * dst > 200_000
            if big and ((shift, subf) != (0.0, 1.0) or (k, a) not in BIG_KERNELS):
                continue
            CTX_CASES.append((k, a, b, src, dst, shift, src * subf))

PLANE_CASES = [
    # (name, dtype, depth, kind, a, b, src_w, src_h, dst_w, dst_h, shift_w, shift_h, subw_f, subh_f)
    ("u10_lanczos3_up2", "u16", 10, "lanczos", 3, math.nan, 48, 27, 96, 54, 0.0, 0.0, 1.0, 1.0),
    ("u10_spline36_up", "u16", 10, "spline36", math.nan, math.nan, 40, 30, 61, 47, 0.0, 0.0, 1.0, 1.0),
    ("u16_lanczos4_down", "u16", 16, "lanczos", 4, math.nan, 64, 48, 30, 21, 0.0, 0.0, 1.0, 1.0),
    ("u8_point_up", "u16", 8, "point", math.nan, math.nan, 13, 11, 40, 23, 0.0, 0.0, 1.0, 1.0),
    ("u12_bilinear_shift", "u16", 12, "bilinear", math.nan, math.nan, 37, 29, 50, 20, 3.3, -3.3, 0.75, 1.05),
    ("u7_bicubic_mitchell", "u16", 7, "bicubic", 1 / 3, 1 / 3, 33, 17, 33, 40, -0.25, 0.125, 1.0, 1.0),
    ("u10_spline64_hshift", "u16", 10, "spline64", math.nan, math.nan, 31, 19, 31, 19, 0.25, 0.0, 1.0, 1.0),
    ("u10_chroma_mpeg2", "u16", 10, "spline36", math.nan, math.nan, 24, 16, 48, 27, -0.25, 0.0, 1.0, 1.0),
    ("u16_lanczos3_tiny", "u16", 16, "lanczos", 3, math.nan, 1, 3, 7, 1, 0.0, 0.0, 1.0, 1.0),
    ("f32_bicubic_down", "f32", 32, "bicubic", 0.0, 0.5, 48, 27, 32, 18, 0.0, 0.0, 1.0, 1.0),
    ("f32_lanczos4_down16", "f32", 32, "lanczos", 4, math.nan, 256, 128, 16, 8, 0.0, 0.0, 1.0, 1.0),
    ("f32_lanczos3_up", "f32", 32, "lanczos", 3, math.nan, 8, 8, 64, 64, 0.0, 0.0, 1.0, 1.0),
    ("f32_lanczos3_field", "f32", 32, "lanczos", 3, math.nan, 48, 27, 32, 18, 0.0, -0.125, 1.0, 1.0),
    ("f32_spline16_shift", "f32", 32, "spline16", math.nan, math.nan, 29, 31, 45, 13, 3.3, -3.3, 0.75, 1.05),
]


def make_plane(rng, dtype, depth, w, h):
    if dtype == "u16":
        return rng.integers(0, 1 << depth, size=(h, w), dtype=np.uint16)
    return rng.random((h, w), dtype=np.float32)


def main():
    ref = Reference()
    rng = np.random.default_rng(0x5EED)
    out = {}
    meta = {"kernels": [], "ctx": [], "plane": []}

    xs = np.array([0.0, 0.25, 0.5, 0.75, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 4.0, -0.5, -1.5, -2.5, 1 / 3, 7.9, 14.999],
                  np.float64)
    out["kernel/x"] = xs
    for i, (k, a, b) in enumerate(KERNELS):
        y, sup = ref.filter_eval(k, xs, a, b)
        out[f"kernel/{i}/y"] = y
        meta["kernels"].append({"kind": k, "a": a, "b": b, "support": sup})

    for i, (k, a, b, src, dst, shift, sub) in enumerate(CTX_CASES):
        c = ref.compute_filter(k, src, dst, shift, sub, a, b)
        out[f"ctx/{i}/f32"] = c.f32
        out[f"ctx/{i}/i16"] = c.i16
        out[f"ctx/{i}/left"] = c.left
        meta["ctx"].append({"kind": k, "a": a, "b": b, "src": src, "dst": dst, "shift": shift, "width": sub,
                            "filter_width": c.width})

    for i, (name, dt, depth, k, a, b, sw, sh, dw, dh, shw, shh, fw, fh) in enumerate(PLANE_CASES):
        x = make_plane(rng, dt, depth, sw, sh)
        kw = dict(depth=depth, shift_w=shw, shift_h=shh, subwidth=sw * fw, subheight=sh * fh)
        y = ref.resize_plane(x, dw, dh, k, a, b, cpu=0, **kw)
        simd_same = None
        if dt == "u16":
            ys = ref.resize_plane(x, dw, dh, k, a, b, cpu=1, **kw)
            simd_same = bool(np.array_equal(y, ys))
        out[f"plane/{i}/src"] = x
        out[f"plane/{i}/dst"] = y
        meta["plane"].append({"name": name, "dtype": dt, "depth": depth, "kind": k, "a": a, "b": b,
                              "dst_w": dw, "dst_h": dh, "shift_w": shw, "shift_h": shh, "subwidth": sw * fw,
                              "subheight": sh * fh, "simd_equal_c": simd_same})

    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {len(CTX_CASES)} filter contexts, {len(PLANE_CASES)} planes, "
          f"{os.path.getsize(OUT) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
