"""Generate tests/golden/depth_golden.npz from zimg's own depth conversion
(src/zimg/depth/, C path CPUClass::NONE), compiled from the reference checkout
by oracle/Makefile into oracle/_ref/libzimgref.so:

    make -C oracle && python tests/golden/make_depth_golden.py

One small seeded plane per (case, plane index) of tests/test_oracle_depth.py's
CASES: the source, and zimg's output for it.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle.oracle import Reference  # noqa: E402
from test_oracle_depth import CASES, make_src  # noqa: E402


def main():
    ref = Reference()
    out = {}
    k = 0
    for c, (fin, fout, dither) in enumerate(CASES):
        rng = np.random.default_rng(7000 + c)
        for plane in range(4):
            src = make_src(rng, fin, 19, 37)
            out[f"case{k}"] = np.int32(c)
            out[f"plane{k}"] = np.int32(plane)
            out[f"src{k}"] = src
            out[f"out{k}"] = ref.depth_convert(src, fin, fout, dither, plane, cpu=0)
            k += 1
    out["n"] = np.int32(k)
    np.savez_compressed(os.path.join(HERE, "depth_golden.npz"), **out)
    print(f"{k} planes")


if __name__ == "__main__":
    main()
