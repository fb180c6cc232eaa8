"""Generate tests/golden/colorspace_golden.npz from zimg's own colorspace
conversion (src/zimg/colorspace/, C path CPUClass::NONE), compiled from the
reference checkout by oracle/Makefile into oracle/_ref/libzimgref.so:

    make -C oracle && python tests/golden/make_colorspace_golden.py

Small seeded planes for every 23rd ordered pair of tests/test_oracle_colorspace.py's
SPACES that zimg converts, under each of its FLAGS: the three source planes and
zimg's three outputs.
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle.oracle import Reference  # noqa: E402
from test_oracle_colorspace import FLAGS, SPACES, planes_for  # noqa: E402


def main():
    ref = Reference()
    out = {}
    k = 0
    for f, kw in enumerate(FLAGS):
        rng = np.random.default_rng(500 + f)
        for n, (cin, cout) in enumerate(itertools.product(SPACES, SPACES)):
            if n % 23 != f % 23 or cin == cout:
                continue
            src = planes_for(rng, 2, 16)
            try:
                dst = ref.colorspace(src, cin, cout, **kw)
            except ValueError:
                continue
            out[f"in{k}"] = np.array(cin, np.int32)
            out[f"out{k}"] = np.array(cout, np.int32)
            out[f"flags{k}"] = np.int32(f)
            out[f"src{k}"] = np.stack(src)
            out[f"dst{k}"] = np.stack(dst)
            k += 1
    out["n"] = np.int32(k)
    np.savez_compressed(os.path.join(HERE, "colorspace_golden.npz"), **out)
    print(f"{k} conversions")


if __name__ == "__main__":
    main()
