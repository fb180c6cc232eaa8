"""The product's host planner (zimg_gb300/csrc/filter_plan.cpp via
zg_compute_filter) against zimg's FilterContexts: the golden vectors, the
oracle, and (where built) the reference itself. Bit-exact throughout: the
u16 GPU path can only be bit-exact if its taps are."""
import math

import numpy as np
import pytest


def _same(a, b):
    return (a.filter_width == b.width and np.array_equal(a.left, b.left) and np.array_equal(a.data_i16, b.i16)
            and np.array_equal(a.data.view(np.uint32), b.f32.view(np.uint32)))


def test_planner_vs_golden(lib, golden):
    import zimg_gb300 as zg
    data, meta = golden
    for i, c in enumerate(meta["ctx"]):
        got = zg.compute_filter(c["kind"], c["src"], c["dst"], c["shift"], c["width"], c["a"], c["b"])
        assert got.filter_width == c["filter_width"], c
        np.testing.assert_array_equal(got.left, data[f"ctx/{i}/left"], err_msg=str(c))
        np.testing.assert_array_equal(got.data_i16, data[f"ctx/{i}/i16"], err_msg=str(c))
        np.testing.assert_array_equal(got.data.view(np.uint32), data[f"ctx/{i}/f32"].view(np.uint32), err_msg=str(c))


def test_planner_vs_oracle_sweep(lib, oracle):
    import zimg_gb300 as zg
    rng = np.random.default_rng(3)
    kinds = [("point", math.nan, math.nan), ("bilinear", math.nan, math.nan), ("bicubic", math.nan, math.nan),
             ("bicubic", 1 / 3, 1 / 3), ("spline16", math.nan, math.nan), ("spline36", math.nan, math.nan),
             ("spline64", math.nan, math.nan), ("lanczos", 2, math.nan), ("lanczos", 3, math.nan),
             ("lanczos", 4, math.nan), ("lanczos", 8, math.nan)]
    n = 0
    for k, a, b in kinds:
        for _ in range(40):
            src = int(rng.choice([1, 2, 3, int(rng.integers(1, 3000))]))
            dst = int(rng.choice([1, 2, int(rng.integers(1, 3000))]))
            shift = float(rng.choice([0.0, 0.25, -0.25, rng.normal(0, 5)]))
            width = src * float(rng.choice([1.0, rng.uniform(0.5, 1.5)]))
            got = zg.compute_filter(k, src, dst, shift, width, a, b)
            want = oracle.compute_filter(k, src, dst, shift, width, a, b)
            assert _same(got, want), (k, a, src, dst, shift, width)
            n += 1
    assert n == 440


@pytest.mark.parametrize("src,dst,kind,a", [(1920, 3840, "lanczos", 3), (7680, 480, "lanczos", 4),
                                            (6400, 64, "lanczos", 3), (64, 6400, "lanczos", 3),
                                            (1080, 720, "bicubic", math.nan), (540, 360, "lanczos", 3)])
def test_planner_config_sizes(lib, oracle, src, dst, kind, a):
    import zimg_gb300 as zg
    got = zg.compute_filter(kind, src, dst, 0.0, None, a)
    want = oracle.compute_filter(kind, src, dst, 0.0, None, a)
    assert _same(got, want)
    # widths quoted for these ratios
    expect = {(1920, 3840): 6, (7680, 480): 128, (6400, 64): 600}
    if (src, dst) in expect:
        assert got.filter_width == expect[(src, dst)]
    # the int16 rows sum to exactly 1 << 14 (filter.cpp:116-121)
    assert np.all(got.data_i16.astype(np.int64).sum(axis=1) == 16384)


def test_planner_vs_reference_dense(lib, reference):
    import zimg_gb300 as zg
    rng = np.random.default_rng(5)
    for _ in range(300):
        k = str(rng.choice(["point", "bilinear", "bicubic", "spline16", "spline36", "spline64", "lanczos"]))
        a = float(rng.integers(1, 16)) if k == "lanczos" else math.nan
        src, dst = int(rng.integers(1, 2000)), int(rng.integers(1, 2000))
        shift = float(rng.normal(0, 3))
        width = src * float(rng.uniform(0.5, 1.5))
        want = reference.compute_filter(k, src, dst, shift, width, a)
        got = zg.compute_filter(k, src, dst, shift, width, a)
        assert _same(got, want), (k, a, src, dst, shift, width)
