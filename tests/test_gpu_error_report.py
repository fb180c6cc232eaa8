"""Per-configuration error of the FP32 engines against the FP64 oracle.

For each FP32 case of the benchmark configurations (at full size where the
oracle finishes in seconds) this measures max-abs and RMS error against the
FP64 oracle for zimg's C path (oracle mode "c"), the CUDA-core kernels and
the tensor-core kernels, and holds every GPU engine to the bound used
throughout: max-abs error <= 2 x the C path's + 1e-6. With ZG_ERROR_REPORT
set to a path, the table is also written there as JSON.
"""
import json
import math
import os

import numpy as np
import pytest

from test_gpu_resize import band_limited, run_conversion

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _errors(got, f64):
    d = got.astype(np.float64) - f64
    return float(np.max(np.abs(d))), float(np.sqrt(np.mean(d * d)))


def _case(oracle, name, src, dw, dh, kind, a=math.nan, b=math.nan, **kw):
    f64 = oracle.resize_plane(src, dw, dh, kind, a, b, mode="f64", nthreads=16, **kw)
    c = oracle.resize_plane(src, dw, dh, kind, a, b, mode="c", nthreads=16, **kw)
    row = {"case": name, "c_path": _errors(c, f64)}
    for engine in ("cuda", "tensor"):
        got, r = run_conversion(src, dw, dh, kind, a, b, engine=engine, **kw)
        row[engine] = _errors(got, f64)
        row[engine + "_plan"] = r.info["engine"]
        assert row[engine][0] <= 2 * row["c_path"][0] + TOL, (name, engine, row)
    return row


def test_fp32_error_per_config(cuda, oracle):
    rng = np.random.default_rng(0x5EED00E0)
    rows = []
    # bicubic b=0 c=0.5, 1920x1080 -> 1280x720, uniform [0,1] plus step edges
    src = rng.random((1080, 1920), dtype=np.float32)
    for _ in range(32):
        x0, y0 = rng.integers(0, 1920), rng.integers(0, 1080)
        src[y0:y0 + rng.integers(8, 300), x0:x0 + rng.integers(8, 300)] += rng.choice([-1, 1]) * rng.uniform(0.2, 0.5)
    rows.append(_case(oracle, "bicubic 1920x1080->1280x720", src, 1280, 720, "bicubic", 0.0, 0.5))
    # Lanczos a=4 16x down, one plane 7680x4320 -> 480x270 (128 taps)
    src = band_limited(rng, 4320, 7680)
    rows.append(_case(oracle, "lanczos4 7680x4320->480x270", src, 480, 270, "lanczos", 4))
    # Lanczos a=3 100x down 6400x6400 -> 64x64 (600 taps)
    src = band_limited(rng, 6400, 6400)
    rows.append(_case(oracle, "lanczos3 6400x6400->64x64", src, 64, 64, "lanczos", 3))
    # Lanczos a=3 100x up 64x64 -> 6400x6400
    src = band_limited(rng, 64, 64)
    rows.append(_case(oracle, "lanczos3 64x64->6400x6400", src, 6400, 6400, "lanczos", 3))
    # interlaced: top field 1920x540 -> 1280x360 (graph shift 0.25 - 0.25 / (360/540))
    frame = band_limited(rng, 1080, 1920)
    field = np.ascontiguousarray(frame[0::2])
    rows.append(_case(oracle, "lanczos3 top field 1920x540->1280x360", field, 1280, 360, "lanczos", 3,
                      shift_h=0.25 - 0.25 / (360 / 540)))
    path = os.environ.get("ZG_ERROR_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(rows, f, indent=1)
