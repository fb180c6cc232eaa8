"""Colorspace conversion (zimg's ColorspaceConversion, src/zimg/colorspace/):
the oracle's C restatement pinned against zimg's own code compiled from the
reference checkout (C path, CPUClass::NONE), bit for bit, over every ordered
pair of a set of colorspaces and the option flags, and against the committed
golden planes made from it. No GPU."""
import itertools
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "colorspace_golden.npz")

# (matrix, transfer, primaries) as zimg API codes (zimg.h:283-352)
SPACES = [
    (1, 1, 1),      # BT.709 YUV
    (0, 1, 1),      # BT.709 RGB
    (0, 8, 1),      # linear RGB, BT.709 primaries
    (0, 13, 1),     # sRGB
    (5, 6, 5),      # BT.470BG / BT.601
    (6, 6, 6),      # SMPTE 170M
    (9, 14, 9),     # BT.2020 NCL
    (10, 14, 9),    # BT.2020 CL
    (0, 16, 9),     # RGB PQ, BT.2020
    (9, 16, 9),     # BT.2020 NCL PQ (HDR10)
    (14, 16, 9),    # ICtCp PQ
    (9, 18, 9),     # BT.2020 HLG
    (14, 18, 9),    # ICtCp HLG
    (0, 18, 9),     # RGB HLG
    (8, 1, 1),      # YCgCo
    (4, 4, 4),      # FCC, BT.470M
    (7, 7, 7),      # SMPTE 240M
    (0, 9, 1),      # log 100
    (0, 10, 1),     # log 316
    (0, 11, 1),     # xvYCC
    (0, 12, 1),     # BT.1361
    (0, 17, 10),    # ST 428 XYZ
    (0, 8, 11),     # DCI-P3
    (0, 1, 12),     # Display P3
    (0, 1, 22),     # EBU 3213
    (12, 1, 8),     # chromaticity-derived NCL, film
    (13, 1, 9),     # chromaticity-derived CL
    (2, 2, 2),      # unspecified
]
FLAGS = [dict(), dict(scene=True), dict(approximate=True), dict(adapt=True), dict(peak=1000.0)]


def planes_for(rng, h, w):
    p = [rng.random((h, w), dtype=np.float32) * 1.2 - 0.1 for _ in range(3)]
    p[1] = (p[1] - 0.5).astype(np.float32)
    p[2] = (p[2] - 0.5).astype(np.float32)
    p[0][0, :4] = [0.0, 1.0, 4.5 * 0.018053968510807, 1.0 / 12.0]  # breakpoints of the curves
    return p


def test_api_code_translation():
    from oracle.oracle import csp_internal
    assert csp_internal(1, 1, 1) == (3, 4, 4)      # BT.709 throughout
    assert csp_internal(6, 6, 7) == (2, 4, 3)      # 170M matrix = 601, BT601 transfer = 709, 240M primaries = SMPTE C
    with pytest.raises(KeyError):
        csp_internal(11, 1, 1)                     # ST 2085 YDZDX: no mapping in zimg


@pytest.mark.parametrize("flags", range(len(FLAGS)))
def test_oracle_matches_zimg_all_pairs(reference, flags):
    o = Oracle()
    rng = np.random.default_rng(90 + flags)
    planes = planes_for(rng, 3, 96)
    kw = FLAGS[flags]
    n_conv = 0
    for cin, cout in itertools.product(SPACES, SPACES):
        try:
            want = reference.colorspace(planes, cin, cout, **kw)
        except ValueError:
            with pytest.raises(ValueError):
                o.colorspace(planes, cin, cout, **kw)
            continue
        got, ops = o.colorspace(planes, cin, cout, **kw)
        n_conv += bool(ops)
        for k in range(3):
            np.testing.assert_array_equal(got[k].view(np.uint32), want[k].view(np.uint32),
                                          err_msg=f"{cin} -> {cout} {kw} plane {k} ops {ops}")
    assert n_conv > 300


def test_oracle_matches_golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("colorspace golden planes not generated")
    data = np.load(GOLDEN)
    o = Oracle()
    for k in range(int(data["n"])):
        cin, cout = tuple(int(x) for x in data[f"in{k}"]), tuple(int(x) for x in data[f"out{k}"])
        kw = FLAGS[int(data[f"flags{k}"])]
        got, _ = o.colorspace([data[f"src{k}"][p] for p in range(3)], cin, cout, **kw)
        np.testing.assert_array_equal(np.stack(got).view(np.uint32), data[f"dst{k}"].view(np.uint32),
                                      err_msg=f"golden {k}")
