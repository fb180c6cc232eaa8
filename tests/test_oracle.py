"""The oracle (oracle/zimg_oracle.c) pinned against zimg itself.

1. Against the committed golden vectors made by zimg's own code
   (tests/golden/make_golden.py): kernel values, FilterContexts, whole planes.
2. Against zimg's unit-test known answers: filter values
   (test/resize/filter_test.cpp:25-106) and graph shift values
   (test/graph/graphbuilder_test.cpp:239-315).
3. Where the reference build exists (oracle/_ref), against zimg directly on a
   seeded sweep.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


def test_golden_filter_contexts(oracle, golden):
    data, meta = golden
    for i, c in enumerate(meta["ctx"]):
        ctx = oracle.compute_filter(c["kind"], c["src"], c["dst"], c["shift"], c["width"], c["a"], c["b"])
        assert ctx.width == c["filter_width"], c
        np.testing.assert_array_equal(ctx.left, data[f"ctx/{i}/left"], err_msg=str(c))
        np.testing.assert_array_equal(ctx.i16, data[f"ctx/{i}/i16"], err_msg=str(c))
        np.testing.assert_array_equal(ctx.f32.view(np.uint32), data[f"ctx/{i}/f32"].view(np.uint32), err_msg=str(c))


def test_golden_planes(oracle, golden):
    data, meta = golden
    for i, p in enumerate(meta["plane"]):
        src, want = data[f"plane/{i}/src"], data[f"plane/{i}/dst"]
        got = oracle.resize_plane(src, p["dst_w"], p["dst_h"], p["kind"], p["a"], p["b"], depth=p["depth"],
                                  shift_w=p["shift_w"], shift_h=p["shift_h"], subwidth=p["subwidth"],
                                  subheight=p["subheight"], mode="c")
        if p["dtype"] == "u16":
            np.testing.assert_array_equal(got, want, err_msg=p["name"])
            assert p["simd_equal_c"], p["name"]  # zimg's SIMD u16 path equals its C path
        else:
            np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=p["name"])


def test_golden_kernel_values(oracle, golden):
    data, meta = golden
    xs = data["kernel/x"]
    for i, k in enumerate(meta["kernels"]):
        got = np.array(_kernel_values(oracle, k["kind"], xs, k["a"], k["b"]))
        np.testing.assert_array_equal(got, data[f"kernel/{i}/y"], err_msg=str(k))


# --- zimg's own known answers (test/resize/filter_test.cpp) -------------------

def _kernel_values(oracle, kind, xs, a=math.nan, b=math.nan):
    """Values f(x) recovered through a 1->many identity-free path is awkward;
    use the C entry point directly."""
    import ctypes as C
    f = (C.c_byte * 128)()
    assert oracle.lib.orc_filter_init(C.byref(f), O.FILTERS[kind], C.c_double(a), C.c_double(b)) == 0
    oracle.lib.orc_filter_eval.restype = C.c_double
    oracle.lib.orc_filter_eval.argtypes = [C.c_void_p, C.c_double]
    return [oracle.lib.orc_filter_eval(C.byref(f), float(x)) for x in xs]


def test_known_answers_filter_values(oracle):
    # filter_test.cpp:25-32 bilinear
    assert _kernel_values(oracle, "bilinear", [0.5, -0.5]) == [0.5, 0.5]
    # filter_test.cpp:34-43 Catmull-Rom
    assert _kernel_values(oracle, "bicubic", [0.5, -0.5, 1.5, -1.5], 0.0, 0.5) == [0.5625, 0.5625, -0.0625, -0.0625]
    # filter_test.cpp:45-57 Mitchell
    m = _kernel_values(oracle, "bicubic", [0.0, 1.0, 2.0, 0.5, 1.5], 1 / 3, 1 / 3)
    assert m[0] == pytest.approx(8 / 9, rel=1e-15)
    assert m[1] == pytest.approx(1 / 18, abs=1e-15)
    assert m[2] == 0.0
    assert m[3] == pytest.approx(77 / 144, rel=1e-15)
    assert m[4] == pytest.approx(-5 / 144, abs=1e-15)
    # filter_test.cpp:59-96 splines
    assert _kernel_values(oracle, "spline16", [0.5, 1.5]) == pytest.approx([0.575, -0.075], rel=1e-15)
    assert _kernel_values(oracle, "spline36", [0.5, 1.5, 2.5]) == pytest.approx([0.598684, -0.118421, 0.0197368],
                                                                                  abs=1e-6)
    assert _kernel_values(oracle, "spline64", [0.5, 1.5, 2.5, 3.5]) == pytest.approx(
        [0.600352, -0.126760, 0.0316901, -0.00528169], abs=1e-6)


@pytest.mark.parametrize("kind,a,support", [("bilinear", math.nan, 1), ("bicubic", 0.0, 2), ("spline16", math.nan, 2),
                                            ("spline36", math.nan, 3), ("spline64", math.nan, 4),
                                            ("lanczos", 1, 1), ("lanczos", 2, 2), ("lanczos", 3, 3)])
def test_known_answers_interpolating(oracle, kind, a, support):
    # filter_test.cpp:8-20: f(0) = 1, f(+-n) ~ 0, f = 0 just outside the support
    b = 0.5 if kind == "bicubic" else math.nan
    assert _kernel_values(oracle, kind, [0.0], a, b) == [1.0]
    for n in range(1, support + 1):
        v = _kernel_values(oracle, kind, [-n, n], a, b)
        assert abs(v[0]) < 1e-15 and abs(v[1]) < 1e-15
    out = _kernel_values(oracle, kind, [np.nextafter(-support, -np.inf), np.nextafter(support, np.inf)], a, b)
    assert out == [0.0, 0.0]


# --- graph shift known answers (test/graph/graphbuilder_test.cpp) -------------

def _yuv(w, h, sw=0, sh=0, loc=1, parity=0):
    return dict(width=w, height=h, subsample_w=sw, subsample_h=sh, color="yuv", chroma_location=loc,
                field_parity=parity)


def _params(src, dst, plane):
    s, d = O.plane_geometry(src), O.plane_geometry(dst)
    return O.resize_params(s[plane], d[plane])


def test_known_answers_graph_chromaloc_upsample():
    # graphbuilder_test.cpp:239-252: LEFT/BOTTOM 4:2:0 -> 4:4:4
    p = _params(_yuv(64, 48, 1, 1, loc=4), _yuv(64, 48, loc=1), 1)
    assert (p["src_w"], p["src_h"], p["dst_w"], p["dst_h"]) == (32, 24, 64, 48)
    assert (p["shift_w"], p["shift_h"], p["subwidth"], p["subheight"]) == (0.25, -0.25, 32.0, 24.0)


def test_known_answers_graph_chromaloc_downsample():
    # graphbuilder_test.cpp:254-267
    p = _params(_yuv(64, 48, loc=1), _yuv(64, 48, 1, 1, loc=4), 1)
    assert (p["shift_w"], p["shift_h"], p["subwidth"], p["subheight"]) == (-0.5, 0.5, 64.0, 48.0)


def test_known_answers_graph_deinterlace():
    # graphbuilder_test.cpp:269-291
    for parity, sh in ((1, 0.25), (2, -0.25)):
        src, dst = _yuv(64, 48, 0, 1, loc=1, parity=parity), _yuv(64, 48, 0, 1, loc=1)
        p0, p1 = _params(src, dst, 0), _params(src, dst, 1)
        assert (p0["shift_w"], p0["shift_h"], p0["subwidth"], p0["subheight"]) == (0.0, sh, 64.0, 48.0)
        assert (p1["src_w"], p1["src_h"]) == (64, 24)
        assert (p1["shift_w"], p1["shift_h"], p1["subwidth"], p1["subheight"]) == (0.0, sh, 64.0, 24.0)


def test_known_answers_graph_interlace_to_interlace():
    # graphbuilder_test.cpp:293-315
    src, dst = _yuv(64, 48, 1, 1, loc=4, parity=1), _yuv(64, 96, 1, 1, loc=4, parity=1)
    p0, p1 = _params(src, dst, 0), _params(src, dst, 1)
    assert (p0["shift_w"], p0["shift_h"], p0["subwidth"], p0["subheight"]) == (0.0, 0.125, 64.0, 48.0)
    assert (p1["shift_w"], p1["shift_h"], p1["subwidth"], p1["subheight"]) == (0.0, 0.0625, 32.0, 24.0)


# --- direct comparison with zimg, where it is built here ----------------------

def test_oracle_vs_reference_sweep(oracle, reference):
    rng = np.random.default_rng(11)
    kinds = [("point", math.nan, math.nan), ("bilinear", math.nan, math.nan), ("bicubic", 0.0, 0.5),
             ("spline36", math.nan, math.nan), ("spline64", math.nan, math.nan), ("lanczos", 3, math.nan),
             ("lanczos", 4, math.nan)]
    for k, a, b in kinds:
        for _ in range(6):
            sw, sh = int(rng.integers(1, 90)), int(rng.integers(1, 60))
            dw, dh = int(rng.integers(1, 130)), int(rng.integers(1, 80))
            shw, shh = float(rng.normal(0, 2)), float(rng.normal(0, 2))
            fw, fh = float(rng.uniform(0.6, 1.3)), float(rng.uniform(0.6, 1.3))
            depth = int(rng.choice([8, 10, 12, 16]))
            x = rng.integers(0, 1 << depth, size=(sh, sw), dtype=np.uint16)
            kw = dict(depth=depth, shift_w=shw, shift_h=shh, subwidth=sw * fw, subheight=sh * fh)
            np.testing.assert_array_equal(oracle.resize_plane(x, dw, dh, k, a, b, **kw),
                                          reference.resize_plane(x, dw, dh, k, a, b, **kw))
            xf = rng.random((sh, sw), dtype=np.float32)
            kw.pop("depth")
            np.testing.assert_array_equal(oracle.resize_plane(xf, dw, dh, k, a, b, **kw).view(np.uint32),
                                          reference.resize_plane(xf, dw, dh, k, a, b, **kw).view(np.uint32))


def test_plan_order_matches_reference(oracle, reference):
    # resize.cpp:12-18: the pass order is what ResizeConversion builds
    cases = [(1920, 1080, 3840, 2160), (1920, 1080, 1280, 720), (7680, 4320, 480, 270), (64, 64, 6400, 6400),
             (6400, 6400, 64, 64), (720, 480, 1920, 1080), (1920, 540, 1280, 360), (100, 100, 100, 50),
             (100, 100, 50, 100), (100, 100, 100, 100)]
    for sw, sh, dw, dh in cases:
        order = oracle.plan_order(sw, sh, dw, dh)
        p = reference.plan(1, 16, "bilinear", sw, sh, dw, dh)
        try:
            assert reference.lib.ref_plan_num_passes(p) == len(order)
        finally:
            reference.free(p)
    assert oracle.plan_order(1920, 1080, 3840, 2160) == ["h", "v"]
    assert oracle.plan_order(1920, 1080, 1280, 720) == ["v", "h"]
