"""zimg's own resize code (oracle/_ref, compiled from the reference checkout)
timed on this host's cores: its C path (CPUClass::NONE) against its best SIMD
path (CPUClass::AUTO: AVX-512 or AVX2 on x86, NEON on aarch64), on the
benchmark's u16 FHD->UHD and f32 bicubic workloads, one thread and all
threads. All threads means frame-parallel workers, each resizing its own
planes, as zimg's test application threads frames (src/testapp/graphapp.cpp
:355-425). Plans are built once; the timed calls run whole planes through
the same whole-plane driver the parity tests use.

This measures the reference, not this library: it reports the SIMD-over-C
factor that the GPU machine's CPU baseline (the C-path restatement, because the
reference checkout is not present there) leaves out.

  python oracle/simd_factor.py [--seconds S] [--json PATH]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository root, not this folder

from oracle.oracle import Reference, aligned_plane, build, reference_available  # noqa: E402

WORKLOADS = [
    # name, pixel type (1 word, 3 float), depth, filter, a, b, src, dst
    ("fhd_uhd_u16 lanczos3 1920x1080->3840x2160", 1, 10, "lanczos", 3.0, float("nan"), (1920, 1080), (3840, 2160)),
    ("bicubic_f32 b=0 c=0.5 1920x1080->1280x720", 3, 32, "bicubic", 0.0, 0.5, (1920, 1080), (1280, 720)),
]


def _planes(ptype, depth, src, dst, rng):
    sw, sh = src
    dw, dh = dst
    s = aligned_plane(sh, sw, np.uint16 if ptype == 1 else np.float32)
    if ptype == 1:
        s[...] = rng.integers(0, 1 << depth, size=(sh, sw), dtype=np.uint16)
    else:
        s[...] = rng.random((sh, sw), dtype=np.float32)
    d = aligned_plane(dh, dw, s.dtype)
    return s, d


def rate(ref: Reference, wl, cpu: int, threads: int, seconds: float) -> float:
    """Output Mpixel/s of `threads` frame-parallel workers for about `seconds`."""
    name, ptype, depth, kind, a, b, src, dst = wl
    plan = ref.plan(ptype, depth, kind, src[0], src[1], dst[0], dst[1], a, b, cpu=cpu)
    err = C.create_string_buffer(512)
    counts = [0] * threads
    stop = threading.Event()

    def worker(t):
        s, d = _planes(ptype, depth, src, dst, np.random.default_rng(t))
        while not stop.is_set():
            if ref.lib.ref_plan_run(plan, s.ctypes.data, s.strides[0], d.ctypes.data, d.strides[0], err, 512):
                raise RuntimeError(err.value.decode())
            counts[t] += 1

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    time.sleep(0.3)  # warm
    c0, t0 = sum(counts), time.perf_counter()
    time.sleep(seconds)
    c1, t1 = sum(counts), time.perf_counter()
    stop.set()
    for th in ths:
        th.join()
    ref.free(plan)
    return (c1 - c0) * dst[0] * dst[1] / (t1 - t0) / 1e6


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=3.0)
    ap.add_argument("--json", default=None)
    args = ap.parse_args()
    build()
    if not reference_available():
        raise SystemExit("oracle/_ref is not built here (the reference checkout is absent)")
    ref = Reference()
    cores = os.cpu_count() or 1
    rows = []
    for wl in WORKLOADS:
        row = {"workload": wl[0], "cores": cores}
        for label, cpu in (("c", 0), ("simd", 1)):
            row[f"{label}_1t"] = round(rate(ref, wl, cpu, 1, args.seconds), 1)
            row[f"{label}_all"] = round(rate(ref, wl, cpu, cores, args.seconds), 1)
        row["simd_over_c_1t"] = round(row["simd_1t"] / row["c_1t"], 2)
        row["simd_over_c_all"] = round(row["simd_all"] / row["c_all"], 2)
        rows.append(row)
        print(json.dumps(row), flush=True)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
