"""Unresize (zimg's UnresizeConversion, src/zimg/unresize/): the oracle's C
restatement pinned against zimg's own code compiled from the reference
checkout (C path), and against the committed golden planes made from it."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "unresize_golden.npz")

# (up w, up h, orig w, orig h, shift w, shift h): both axes, one axis, shifts,
# tiny planes, near-identity ratios, strong ones
CASES = [
    (64, 48, 32, 24, 0.0, 0.0),
    (100, 60, 77, 45, 0.0, 0.0),
    (128, 96, 128, 48, 0.0, 0.0),
    (96, 64, 50, 64, 0.0, 0.0),
    (80, 60, 40, 30, 0.25, -0.3),
    (200, 150, 33, 17, 0.0, 0.0),
    (37, 23, 19, 11, 0.1, 0.0),
    (5, 4, 3, 2, 0.0, 0.0),
    (64, 64, 64, 64, 0.2, 0.0),
    (256, 144, 255, 143, 0.0, 0.0),
]


def make_src(rng, h, w):
    return rng.random((h, w), dtype=np.float32)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_oracle_matches_zimg(reference, case):
    uw, uh, ow, oh, sw, sh = CASES[case]
    src = make_src(np.random.default_rng(900 + case), uh, uw)
    want = reference.unresize_plane(src, ow, oh, sw, sh, cpu=0)
    got = Oracle().unresize_plane(src, ow, oh, sw, sh)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=str(CASES[case]))


def test_oracle_matches_golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("unresize golden planes not generated")
    data = np.load(GOLDEN)
    o = Oracle()
    for k in range(int(data["n"])):
        uw, uh, ow, oh, sw, sh = CASES[int(data[f"case{k}"])]
        got = o.unresize_plane(data[f"src{k}"], ow, oh, sw, sh)
        np.testing.assert_array_equal(got.view(np.uint32), data[f"out{k}"].view(np.uint32), err_msg=f"golden {k}")


def test_upscale_is_refused():
    with pytest.raises(ValueError):
        Oracle().unresize_plane(np.zeros((10, 10), np.float32), 20, 10)
