"""Generate tests/golden/unresize_golden.npz from zimg's own unresize
(src/zimg/unresize/, C path CPUClass::NONE), compiled from the reference
checkout by oracle/Makefile:

    make -C oracle && python tests/golden/make_unresize_golden.py

One seeded plane per case of tests/test_oracle_unresize.py's CASES.
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
from test_oracle_unresize import CASES, make_src  # noqa: E402


def main():
    ref = Reference()
    out = {}
    for k, (uw, uh, ow, oh, sw, sh) in enumerate(CASES):
        src = make_src(np.random.default_rng(9000 + k), uh, uw)
        out[f"case{k}"] = np.int32(k)
        out[f"src{k}"] = src
        out[f"out{k}"] = ref.unresize_plane(src, ow, oh, sw, sh, cpu=0)
    out["n"] = np.int32(len(CASES))
    np.savez_compressed(os.path.join(HERE, "unresize_golden.npz"), **out)
    print(f"{len(CASES)} planes")


if __name__ == "__main__":
    main()
