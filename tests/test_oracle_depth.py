"""Depth conversion (zimg's DepthConversion, src/zimg/depth/): the oracle's C
restatement pinned against zimg's own code compiled from the reference
checkout (C path, CPUClass::NONE), and against the committed golden planes
made from it. No GPU."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, PixelFormat as PF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "depth_golden.npz")

# (pixel in, pixel out, dither): every conversion kind zimg picks
CASES = [
    (PF("byte", 8), PF("word", 10), "none"),               # left shift
    (PF("byte", 8), PF("word", 16), "none"),
    (PF("word", 10, False, True), PF("word", 16, False, True), "none"),
    (PF("word", 10), PF("byte", 8), "none"),               # dither to integer
    (PF("word", 10), PF("byte", 8), "ordered"),
    (PF("word", 16), PF("word", 10), "ordered"),
    (PF("word", 12, True, True), PF("byte", 8, False, True), "ordered"),
    (PF("byte", 8, True), PF("byte", 8), "ordered"),       # full -> limited range
    (PF("byte", 8), PF("byte", 8, True), "none"),
    (PF("float"), PF("byte", 8), "ordered"),
    (PF("float"), PF("word", 10), "none"),
    (PF("float"), PF("word", 16, True), "ordered"),
    (PF("float", None, False, True), PF("byte", 8, False, True), "ordered"),
    (PF("byte", 8), PF("float"), "none"),                  # to float
    (PF("word", 10, False, True), PF("float", None, False, True), "none"),
    (PF("word", 16, True), PF("float"), "none"),
    (PF("word", 10), PF("word", 10), "ordered"),           # equal formats: copy
    (PF("half"), PF("float"), "none"),                     # HALF (IEEE binary16)
    (PF("float"), PF("half"), "none"),
    (PF("byte", 8), PF("half"), "none"),
    (PF("word", 10, False, True), PF("half", None, False, True), "none"),
    (PF("half"), PF("byte", 8), "ordered"),
    (PF("half", None, False, True), PF("word", 10, False, True), "ordered"),
    (PF("word", 10), PF("byte", 8), "random"),              # blue-noise dither
    (PF("float"), PF("word", 16, True), "random"),
    (PF("half"), PF("byte", 8), "random"),
    (PF("byte", 8, True), PF("byte", 8), "random"),
    (PF("word", 12, True, True), PF("byte", 8, False, True), "random"),
    (PF("word", 10), PF("byte", 8), "error_diffusion"),     # Floyd-Steinberg
    (PF("float"), PF("byte", 8), "error_diffusion"),
    (PF("float", None, False, True), PF("word", 10, False, True), "error_diffusion"),
    (PF("half"), PF("word", 16, True), "error_diffusion"),
    (PF("byte", 8), PF("byte", 8, True), "error_diffusion"),
    (PF("word", 16), PF("word", 10), "error_diffusion"),
    (PF("byte", 8, True), PF("word", 9, True), "error_diffusion"),
]


def make_src(rng, f: PF, h, w, special=True):
    if f.type in ("float", "half"):
        x = rng.random((h, w), dtype=np.float32) * 1.25 - 0.125  # out-of-range values exercise the clamp
        x = (x - 0.5).astype(np.float32) if f.chroma else x.astype(np.float32)
        if special:
            # signed zeros, infinities, binary16 subnormals and overflow
            v = np.array([0.0, -0.0, np.inf, -np.inf, 3e-6, 6.1e-5, 70000.0, 65519.0], np.float32)
            x.flat[: min(x.size, v.size)] = v[: min(x.size, v.size)]
        if f.type == "half":
            with np.errstate(over="ignore"):
                return x.astype(np.float16).view(np.uint16)
        return x
    return rng.integers(0, 1 << f.bits, size=(h, w)).astype(f.dtype)


def test_bayer_matrix_first_rows():
    # zimg's matrix rows 0 and 15 (dither.cpp:138,153) from the recursive definition
    o = Oracle()
    assert [o.lib.orc_bayer16(0, j) for j in range(8)] == [0, 192, 48, 240, 12, 204, 60, 252]
    assert [o.lib.orc_bayer16(15, j) for j in range(13, 16)] == [101, 149, 85]
    vals = sorted(o.lib.orc_bayer16(i, j) for i in range(16) for j in range(16))
    assert vals == list(range(256))


def test_depth_modes():
    o = Oracle()
    assert o.depth_mode(PF("byte", 8), PF("word", 10)) == 1
    assert o.depth_mode(PF("float"), PF("byte", 8), "ordered") == 3
    assert o.depth_mode(PF("byte", 8), PF("float")) == 2
    assert o.depth_mode(PF("word", 10), PF("word", 10)) == 0
    assert o.depth_mode(PF("word", 7), PF("word", 10)) == -1          # limited range below 8 bits
    assert o.depth_mode(PF("float"), PF("byte", 8), "random") == 3
    assert o.depth_mode(PF("float"), PF("byte", 8), "error_diffusion") == 3


def test_blue_noise_table_is_zimgs(reference):
    # the library's packed copy of zimg's blue-noise matrix (blue.h:10-13)
    import ctypes
    buf = (ctypes.c_uint8 * 4096)()
    reference.lib.ref_blue_noise_table(buf)
    want = np.frombuffer(bytes(buf), np.uint8).reshape(64, 64)
    o = Oracle()
    got = np.array([[o.lib.orc_blue_noise(i, j) for j in range(64)] for i in range(64)], np.uint8)
    np.testing.assert_array_equal(got, want)


def test_error_diffusion_hand_case():
    # 2 x 3 plane, WORD 10-bit -> BYTE 8-bit limited range: scale 1/4, so the
    # samples 2, 2, 2 / 6, 6, 6 are 0.5 / 1.5 before the error terms; worked
    # through dither.cpp:59-85 by hand.
    o = Oracle()
    src = np.array([[2, 2, 2], [6, 6, 6]], np.uint16)
    got = o.depth_convert(src, PF("word", 10), PF("byte", 8), "error_diffusion")
    # row 0: .5 -> 0 (ties to even, error .5); .5 + .5*7/16 = .71875 -> 1
    #        (error -.28125); .5 - .28125*7/16 = .376953125 -> 0
    # row 1: 1.5 - .28125*3/16 + .5*5/16 = 1.603515625 -> 2 (error
    #        -.396484375); 1.5 - .17346 + .07068 - .08789 + .03125 = 1.34058
    #        -> 1 (error .34058); 1.5 + .14900 + .11780 - .01758 = 1.74923 -> 2
    assert got.tolist() == [[0, 1, 0], [2, 1, 2]]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_oracle_matches_zimg(reference, case):
    fin, fout, dither = CASES[case]
    o = Oracle()
    rng = np.random.default_rng(100 + case)
    src = make_src(rng, fin, 41, 157)
    for plane in range(4):
        want = reference.depth_convert(src, fin, fout, dither, plane, cpu=0)
        got = o.depth_convert(src, fin, fout, dither, plane)
        np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=f"{CASES[case]} plane {plane}")


@pytest.mark.parametrize("dither", ["random", "error_diffusion"])
def test_oracle_matches_zimg_640x480(reference, dither):
    # the size of zimg's own dither tests (test/depth/dither_test.cpp:14-15),
    # every input type to BYTE and WORD
    o = Oracle()
    rng = np.random.default_rng(41)
    for fin in (PF("byte", 8), PF("word", 16), PF("half"), PF("float")):
        src = make_src(rng, fin, 480, 640, special=False)
        for fout in (PF("byte", 8), PF("word", 16)):
            want = reference.depth_convert(src, fin, fout, dither, 1, cpu=0)
            got = o.depth_convert(src, fin, fout, dither, 1)
            np.testing.assert_array_equal(got, want, err_msg=f"{fin} -> {fout}")


def test_oracle_matches_golden():
    if not os.path.exists(GOLDEN):
        pytest.skip("depth golden planes not generated")
    data = np.load(GOLDEN)
    o = Oracle()
    n = int(data["n"])
    for k in range(n):
        fin, fout, dither = CASES[int(data[f"case{k}"])]
        plane = int(data[f"plane{k}"])
        got = o.depth_convert(data[f"src{k}"], fin, fout, dither, plane)
        np.testing.assert_array_equal(got.view(np.uint8), data[f"out{k}"].view(np.uint8), err_msg=f"golden {k}")
