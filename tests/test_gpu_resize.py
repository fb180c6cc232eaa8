"""GPU parity: the CUDA path through the C ABI against the oracle.

u16: bit-exact against zimg's C path (oracle mode "c"), as zimg's own SIMD
tests demand (test/resize/x86/resize_impl_avx2_test.cpp:70, SNR = infinity).
f32 CUDA-core path: bit-exact against the oracle's sequential fused
multiply-add order (mode "fma"); its error against the FP64 oracle must be no
worse than 2x zimg's C path's own error plus 1e-6 (tolerance stated here).
f32 tensor-core passes (3xTF32, summed in another order) are held to that
error bound only.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32_ABS_TOL = 1e-6  # slack added to 2x the C path's max-abs error vs FP64


def to_dev(a):
    import torch
    if a.dtype == np.uint16:
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def empty(h, w, dtype, pad=0, offset=0):
    """Device plane [h, w]; pad extra elements per row and a start offset to
    exercise unaligned strides."""
    import torch
    tdt = torch.int16 if dtype == np.uint16 else torch.float32
    buf = torch.full((h * (w + pad) + offset + 1,), 0, dtype=tdt, device="cuda")
    return buf[offset:offset + h * (w + pad)].view(h, w + pad)[:, :w]


def to_host(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


def run_conversion(src, dst_w, dst_h, kind, a=math.nan, b=math.nan, depth=None, shift_w=0.0, shift_h=0.0,
                   subwidth=None, subheight=None, fusion=True, engine="auto", pad=0, offset=0):
    import torch
    import zimg_gb300 as zg
    h, w = src.shape
    ptype = "word" if src.dtype == np.uint16 else "float"
    conv = zg.ResizeConversion(w, h, ptype).set_filter(kind, a, b).set_dst_width(dst_w).set_dst_height(dst_h) \
        .set_shift_w(shift_w).set_shift_h(shift_h).set_fusion(fusion).set_engine(engine)
    if depth is not None:
        conv.set_depth(depth)
    if subwidth is not None:
        conv.set_subwidth(subwidth)
    if subheight is not None:
        conv.set_subheight(subheight)
    r = conv.create()
    if pad or offset:
        s = empty(h, w, src.dtype, pad, offset)
        s.copy_(to_dev(src))
    else:
        s = to_dev(src)
    d = empty(dst_h, dst_w, src.dtype, pad, offset)
    r.process(s, d)
    torch.cuda.synchronize()
    return to_host(d, src.dtype), r


def make_u16(rng, h, w, depth):
    """FHD-to-UHD test content: 16x16 blocks of uniform noise or smooth waves."""
    out = np.empty((h, w), np.uint16)
    maxv = (1 << depth) - 1
    yy, xx = np.mgrid[0:h, 0:w]
    lx, ly, ph = rng.uniform(64, 512), rng.uniform(64, 512), rng.uniform(0, 2 * np.pi)
    wave = np.round(maxv / 2 + maxv / 2 * np.sin(2 * np.pi * (xx / lx + yy / ly) + ph)).astype(np.uint16)
    noise = rng.integers(0, maxv + 1, size=(h, w), dtype=np.uint16)
    pick = rng.random(((h + 15) // 16, (w + 15) // 16)) < 0.5
    mask = np.kron(pick, np.ones((16, 16), bool))[:h, :w]
    out[...] = np.where(mask, noise, wave)
    return out


# ------------------------------------------------------------------ golden --

def test_golden_planes_on_gpu(cuda, golden, oracle):
    data, meta = golden
    for i, p in enumerate(meta["plane"]):
        src, want = data[f"plane/{i}/src"], data[f"plane/{i}/dst"]
        kw = dict(depth=p["depth"], shift_w=p["shift_w"], shift_h=p["shift_h"], subwidth=p["subwidth"],
                  subheight=p["subheight"])
        if p["dtype"] == "u16":
            for engine in ("auto", "cuda"):
                got, _ = run_conversion(src, p["dst_w"], p["dst_h"], p["kind"], p["a"], p["b"], engine=engine, **kw)
                np.testing.assert_array_equal(got, want, err_msg=(p["name"], engine))
        else:
            kw.pop("depth")
            # CUDA-core kernels: zimg's tap order with fused multiply-adds
            got, _ = run_conversion(src, p["dst_w"], p["dst_h"], p["kind"], p["a"], p["b"], engine="cuda", **kw)
            fma = oracle.resize_plane(src, p["dst_w"], p["dst_h"], p["kind"], p["a"], p["b"], mode="fma", **kw)
            np.testing.assert_array_equal(got.view(np.uint32), fma.view(np.uint32), err_msg=p["name"])
            # against zimg's own (unfused) C path output: tiny reassociation-free difference only
            assert np.max(np.abs(got - want)) < 1e-5, p["name"]
            # the planner's own choice (tensor cores for wide filters): within the FP64 error bound
            got, _ = run_conversion(src, p["dst_w"], p["dst_h"], p["kind"], p["a"], p["b"], **kw)
            _f32_check(oracle, src, got, p["dst_w"], p["dst_h"], p["kind"], p["a"], p["b"], exact=False, **kw)


# ------------------------------------------------- headline configurations --

def test_fhd_to_uhd_u16_lanczos3_bitexact(cuda, oracle):
    rng = np.random.default_rng(0x5EED0001)
    src = make_u16(rng, 1080, 1920, 10)
    got, r = run_conversion(src, 3840, 2160, "lanczos", 3, depth=10)
    assert r.info["num_passes"] == 2 and r.info["first_horizontal"]
    want = oracle.resize_plane(src, 3840, 2160, "lanczos", 3, depth=10, mode="c", nthreads=16)
    np.testing.assert_array_equal(got, want)


def test_fhd_to_uhd_engines_agree(cuda, oracle):
    """Tensor-core fused, CUDA-core fused and separate passes give zimg's bytes."""
    rng = np.random.default_rng(7)
    src = make_u16(rng, 270, 480, 10)
    want = oracle.resize_plane(src, 960, 540, "lanczos", 3, depth=10, mode="c")
    for engine, fusion, expect in (("auto", True, "tensor"), ("cuda", True, "cuda"), ("cuda", False, "passes")):
        got, r = run_conversion(src, 960, 540, "lanczos", 3, depth=10, fusion=fusion, engine=engine)
        assert r.info["engine"] == expect
        np.testing.assert_array_equal(got, want, err_msg=engine)


@pytest.mark.parametrize("depth", [8, 10, 12])
@pytest.mark.parametrize("shape", [(1920, 1080, 3840, 2160), (720, 480, 1920, 1080), (3840, 2160, 1920, 1080),
                                   (333, 97, 1001, 500), (640, 480, 427, 320)])
def test_tensor_core_u16_bitexact(cuda, oracle, depth, shape):
    """The tensor-core path (exact integer arithmetic in fp16 x fp16 -> fp32)."""
    sw, sh, dw, dh = shape
    rng = np.random.default_rng(depth * 1000 + sw)
    src = make_u16(rng, sh, sw, depth)
    for kind, a in (("spline36", math.nan), ("lanczos", 3.0), ("bicubic", math.nan)):
        got, r = run_conversion(src, dw, dh, kind, a, depth=depth, engine="tensor")
        # depth 12: 8192 + sum|tap| * 2^11 reaches 2^24, so exactness cannot be
        # certified and the planner keeps the separate integer passes
        assert r.info["engine"] == ("tensor" if depth <= 10 else "passes"), (shape, kind)
        want = oracle.resize_plane(src, dw, dh, kind, a, depth=depth, mode="c", nthreads=16)
        np.testing.assert_array_equal(got, want, err_msg=str((shape, kind, depth)))


@pytest.mark.parametrize("depth,shape", [(12, (1080, 1920, 2160, 3840)), (16, (1080, 1920, 2160, 3840)),
                                         (12, (2160, 3840, 1080, 1920))])
def test_deep_u16_fused_int32_bitexact(cuda, oracle, depth, shape):
    """u16 planes deeper than the float-exactness proof allows (12-bit HDR,
    16-bit) run the fused CUDA-core kernel in zimg's int32 arithmetic
    (resize_impl.cpp:31-59), bit-exact against zimg's C path at full size,
    H first (upscale) and V first (downscale)."""
    sh, sw, dh, dw = shape
    rng = np.random.default_rng(depth * 7 + sw)
    src = make_u16(rng, sh, sw, depth)
    got, r = run_conversion(src, dw, dh, "lanczos", 3, depth=depth)
    assert r.info["engine"] == "cuda", r.info
    want = oracle.resize_plane(src, dw, dh, "lanczos", 3, depth=depth, mode="c", nthreads=16)
    np.testing.assert_array_equal(got, want, err_msg=str((depth, shape)))


def _f32_check(oracle, src, got, dst_w, dst_h, kind, a=math.nan, b=math.nan, exact=True, **kw):
    fma = oracle.resize_plane(src, dst_w, dst_h, kind, a, b, mode="fma", nthreads=16, **kw)
    if exact:
        np.testing.assert_array_equal(got.view(np.uint32), fma.view(np.uint32))
    f64 = oracle.resize_plane(src, dst_w, dst_h, kind, a, b, mode="f64", nthreads=16, **kw)
    c = oracle.resize_plane(src, dst_w, dst_h, kind, a, b, mode="c", nthreads=16, **kw)
    err_gpu = float(np.max(np.abs(got.astype(np.float64) - f64)))
    err_c = float(np.max(np.abs(c.astype(np.float64) - f64)))
    assert err_gpu <= 2 * err_c + F32_ABS_TOL, (err_gpu, err_c)
    return err_gpu, err_c


def test_bicubic_1080p_to_720p_f32(cuda, oracle):
    rng = np.random.default_rng(0x5EED0002)
    for plane in range(3):
        src = rng.random((1080, 1920), dtype=np.float32)
        for _ in range(32):
            x0, y0 = rng.integers(0, 1920), rng.integers(0, 1080)
            src[y0:y0 + rng.integers(8, 300), x0:x0 + rng.integers(8, 300)] += rng.choice([-1, 1]) * rng.uniform(0.2, 0.5)
        got, r = run_conversion(src, 1280, 720, "bicubic", 0.0, 0.5)
        assert r.info["num_passes"] == 2 and not r.info["first_horizontal"]
        _f32_check(oracle, src, got, 1280, 720, "bicubic", 0.0, 0.5)


def band_limited(rng, h, w, cutoff=0.25):
    x = rng.standard_normal((h, w))
    f = np.fft.rfft2(x)
    fy = np.abs(np.fft.fftfreq(h))[:, None]
    fx = np.fft.rfftfreq(w)[None, :]
    f[(fy > cutoff) | (fx > cutoff)] = 0
    y = np.fft.irfft2(f, s=(h, w))
    y = (y - y.min()) / (y.max() - y.min())
    return y.astype(np.float32)


def test_wide_filter_down16_f32(cuda, oracle):
    rng = np.random.default_rng(0x5EED0003)
    src = band_limited(rng, 1080, 1920)
    got, r = run_conversion(src, 120, 67, "lanczos", 4, engine="cuda")
    assert r.info["engine"] == "passes"
    _f32_check(oracle, src, got, 120, 67, "lanczos", 4)
    # 128 taps per output: the planner puts both passes on the tensor cores (3xTF32)
    got, r = run_conversion(src, 120, 67, "lanczos", 4)
    assert r.info["engine"] == "tensor-passes"
    _f32_check(oracle, src, got, 120, 67, "lanczos", 4, exact=False)


def test_extreme_ratios_f32(cuda, oracle):
    rng = np.random.default_rng(0x5EED0005)
    small = band_limited(rng, 64, 64)
    got, _ = run_conversion(small, 1600, 1600, "lanczos", 3, engine="cuda")
    _f32_check(oracle, small, got, 1600, 1600, "lanczos", 3)
    big = band_limited(rng, 1600, 1600)
    got, _ = run_conversion(big, 16, 16, "lanczos", 3, engine="cuda")
    _f32_check(oracle, big, got, 16, 16, "lanczos", 3)
    got, r = run_conversion(big, 16, 16, "lanczos", 3)  # 600 taps: tensor cores
    assert r.info["engine"] == "tensor-passes"
    _f32_check(oracle, big, got, 16, 16, "lanczos", 3, exact=False)


@pytest.mark.parametrize("kind,a", [("lanczos", 4), ("lanczos", 3), ("bicubic", math.nan), ("spline64", math.nan)])
def test_tensor_core_f32_error_bound(cuda, oracle, kind, a):
    """3xTF32 passes against the FP64 oracle: no worse than twice the C path's
    own error, over shapes that exercise partial output groups, partial
    16-wide tiles, clamped band ends and unaligned planes."""
    rng = np.random.default_rng(abs(hash((kind, a, "tc"))) % 2**32)
    shapes = [((1080, 1920), (67, 120)), ((517, 333), (31, 29)), ((64, 64), (300, 200)), ((130, 7), (9, 3)),
              ((1, 257), (1, 5)), ((257, 1), (5, 1))]
    for (sh, sw), (dh, dw) in shapes:
        src = band_limited(rng, sh, sw) if sh > 1 and sw > 1 else rng.random((sh, sw), dtype=np.float32)
        kw = dict(shift_w=float(rng.normal(0, 2)), shift_h=float(rng.normal(0, 2)))
        pad, off = int(rng.choice([0, 1, 3])), int(rng.choice([0, 1]))
        got, r = run_conversion(src, dw, dh, kind, a, pad=pad, offset=off, engine="tensor", **kw)
        if r.info["num_passes"]:
            assert r.info["engine"] == "tensor-passes", r.info
        _f32_check(oracle, src, got, dw, dh, kind, a, exact=False, **kw)


def test_interlaced_fields_f32(cuda, oracle):
    rng = np.random.default_rng(0x5EED0055)
    frame = band_limited(rng, 1080, 1920)
    for parity, field in ((1, frame[0::2]), (2, frame[1::2])):
        # field -> field of the same parity: graph shift 0.25 - 0.25/(720/1080) (graphbuilder.cpp:167-188,769-776)
        off = -0.25 if parity == 1 else 0.25
        shift_h = -off + off / (360 / 540)
        got, _ = run_conversion(np.ascontiguousarray(field), 1280, 360, "lanczos", 3, shift_h=shift_h)
        _f32_check(oracle, np.ascontiguousarray(field), got, 1280, 360, "lanczos", 3, shift_h=shift_h)


# --------------------------------------------------------------- edge cases --

FILTERS = [("point", math.nan, math.nan), ("bilinear", math.nan, math.nan), ("bicubic", math.nan, math.nan),
           ("bicubic", 1 / 3, 1 / 3), ("spline16", math.nan, math.nan), ("spline36", math.nan, math.nan),
           ("spline64", math.nan, math.nan), ("lanczos", 2, math.nan), ("lanczos", 3, math.nan),
           ("lanczos", 4, math.nan)]


@pytest.mark.parametrize("kind,a,b", FILTERS)
def test_random_shapes_u16_bitexact(cuda, oracle, kind, a, b):
    rng = np.random.default_rng(abs(hash((kind, a))) % 2**32)
    for trial in range(12):
        sw, sh = int(rng.integers(1, 131)), int(rng.integers(1, 131))
        dw, dh = int(rng.integers(1, 131)), int(rng.integers(1, 131))
        depth = int(rng.choice([1, 7, 8, 10, 12, 16]))
        shw = float(rng.choice([0.0, 0.25, -0.25, 3.3, -3.3]))
        shh = float(rng.choice([0.0, 0.25, -0.25, 3.3, -3.3]))
        fw, fh = float(rng.choice([1.0, 0.75, 1.05])), float(rng.choice([1.0, 0.75, 1.05]))
        src = rng.integers(0, 1 << depth, size=(sh, sw), dtype=np.uint16)
        kw = dict(depth=depth, shift_w=shw, shift_h=shh, subwidth=sw * fw, subheight=sh * fh)
        pad, off = int(rng.choice([0, 1, 3])), int(rng.choice([0, 1]))
        got, _ = run_conversion(src, dw, dh, kind, a, b, pad=pad, offset=off, **kw)
        want = oracle.resize_plane(src, dw, dh, kind, a, b, mode="c", **kw)
        np.testing.assert_array_equal(got, want, err_msg=str((sw, sh, dw, dh, kw, pad, off)))


@pytest.mark.parametrize("kind,a,b", FILTERS)
def test_random_shapes_f32(cuda, oracle, kind, a, b):
    rng = np.random.default_rng(abs(hash((kind, a, "f"))) % 2**32)
    for trial in range(8):
        sw, sh = int(rng.integers(1, 131)), int(rng.integers(1, 131))
        dw, dh = int(rng.integers(1, 131)), int(rng.integers(1, 131))
        kw = dict(shift_w=float(rng.normal(0, 2)), shift_h=float(rng.normal(0, 2)),
                  subwidth=sw * float(rng.uniform(0.7, 1.2)), subheight=sh * float(rng.uniform(0.7, 1.2)))
        src = rng.random((sh, sw), dtype=np.float32)
        pad, off = int(rng.choice([0, 1, 3])), int(rng.choice([0, 1]))
        got, _ = run_conversion(src, dw, dh, kind, a, b, pad=pad, offset=off, engine="cuda", **kw)
        fma = oracle.resize_plane(src, dw, dh, kind, a, b, mode="fma", **kw)
        np.testing.assert_array_equal(got.view(np.uint32), fma.view(np.uint32))


def test_identity_is_copy(cuda):
    rng = np.random.default_rng(1)
    src = rng.integers(0, 1024, size=(37, 53), dtype=np.uint16)
    got, r = run_conversion(src, 53, 37, "lanczos", 3, depth=10)
    assert r.info["num_passes"] == 0
    np.testing.assert_array_equal(got, src)


def test_single_passes(cuda, oracle):
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(2)
    src = rng.integers(0, 4096, size=(45, 77), dtype=np.uint16)
    for horizontal, dim in ((True, 131), (False, 19)):
        p = zg.ResizeImplBuilder(77, 45, "word").set_horizontal(horizontal).set_dst_dim(dim).set_depth(12) \
            .set_filter("spline36").set_shift(0.3).create()
        ow, oh = p.output_size
        d = empty(oh, ow, np.uint16)
        p.process(to_dev(src), d)
        torch.cuda.synchronize()
        want = oracle.resize_pass(src, horizontal, dim, "spline36", depth=12, shift=0.3)
        np.testing.assert_array_equal(to_host(d, np.uint16), want)


def test_errors_on_gpu(cuda):
    import torch
    import zimg_gb300 as zg
    r = zg.ResizeConversion(64, 48, "word").set_dst_width(128).set_dst_height(96).set_filter("bilinear").create()
    src = torch.zeros((48, 64), dtype=torch.int16, device="cuda")
    dst = torch.zeros((96, 64), dtype=torch.int16, device="cuda")  # too narrow
    with pytest.raises(zg.ZimgError) as e:
        r.process(src, dst)
    assert e.value.code == 2048
    with pytest.raises(zg.ZimgError):
        zg.ResizeConversion(64, 48, "byte").set_dst_width(10).create()
    with pytest.raises(zg.ZimgError) as e:
        zg.ResizeConversion(64, 48, "word").set_depth(17).set_dst_width(10).create()
    assert e.value.code == 1028


# ---------------------------------------------------------- batch and graph --

def test_batch_matches_single(cuda, oracle):
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(4)
    shapes = [(48, 64, 96, 54), (30, 40, 20, 15), (72, 128, 256, 144), (27, 48, 27, 48)]
    convs, srcs, dsts, wants = [], [], [], []
    for sh, sw, dh, dw in shapes:
        src = rng.integers(0, 1024, size=(sh, sw), dtype=np.uint16)
        convs.append(zg.ResizeConversion(sw, sh, "word").set_depth(10).set_filter("spline36")
                     .set_dst_width(dw).set_dst_height(dh).set_shift_w(-0.25))
        srcs.append(to_dev(src))
        dsts.append(empty(dh, dw, np.uint16))
        wants.append(oracle.resize_plane(src, dw, dh, "spline36", depth=10, shift_w=-0.25))
    b = zg.Batch(convs)
    b.set_io(srcs, dsts)
    for mode in ("plain", "graph"):
        for d in dsts:
            d.zero_()
        (b.process if mode == "plain" else b.process_graph)()
        torch.cuda.synchronize()
        for d, w in zip(dsts, wants):
            np.testing.assert_array_equal(to_host(d, np.uint16), w, err_msg=mode)


def test_batch_work_chunks_repeat(cuda, oracle):
    """Launches whose CTAs take guided chunks of work from a counter (the
    one-launch mixed batch, the CUDA-core streaming batch) leave the counter
    zero for the next launch: every repetition, plain or replayed from a
    graph, writes every output in full and bit-exact."""
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(11)
    # mixed u16 batch in one launch: 2.25x and 1.5x upscales, a 2x downscale
    # and identity planes of one output size (a YUV batch's luma planes)
    u16_shapes = [(240, 320), (360, 640), (1080, 1920), (540, 960), (360, 640), (240, 320), (1080, 1920)]
    convs, srcs, dsts, wants = [], [], [], []
    for sh, sw in u16_shapes:
        src = make_u16(rng, sh, sw, 10)
        convs.append(zg.ResizeConversion(sw, sh, "word").set_depth(10).set_filter("spline36")
                     .set_dst_width(960).set_dst_height(540))
        srcs.append(to_dev(src))
        dsts.append(empty(540, 960, np.uint16))
        wants.append(oracle.resize_plane(src, 960, 540, "spline36", depth=10))
    mixed = zg.Batch(convs)
    mixed.set_io(srcs, dsts)
    assert mixed.launch_count == 1
    # f32 batch on the CUDA-core streaming kernel
    f_convs, f_srcs, f_dsts, f_wants = [], [], [], []
    for k in range(6):
        src = rng.random((270 + 6 * k, 480), dtype=np.float32)
        f_convs.append(zg.ResizeConversion(480, 270 + 6 * k, "float").set_filter("bicubic", 0.0, 0.5)
                       .set_dst_width(320).set_dst_height(180).set_engine("cuda"))
        f_srcs.append(to_dev(src))
        f_dsts.append(empty(180, 320, np.float32))
        f_wants.append(oracle.resize_plane(src, 320, 180, "bicubic", 0.0, 0.5, mode="fma"))
    stream_batch = zg.Batch(f_convs)
    stream_batch.set_io(f_srcs, f_dsts)
    for rep in range(3):
        for mode in ("plain", "graph"):
            for d in dsts + f_dsts:
                d.fill_(-1)
            for b in (mixed, stream_batch):
                (b.process if mode == "plain" else b.process_graph)()
            torch.cuda.synchronize()
            for i, (d, w) in enumerate(zip(dsts, wants)):
                np.testing.assert_array_equal(to_host(d, np.uint16), w, err_msg=(rep, mode, "u16", i))
            for i, (d, w) in enumerate(zip(f_dsts, f_wants)):
                np.testing.assert_array_equal(to_host(d, np.float32).view(np.uint32), w.view(np.uint32),
                                              err_msg=(rep, mode, "f32", i))


def test_batch_identity_planes_copied(cuda):
    """Identity conversions in a batch (no pass, resize.cpp:43-47) are copied
    in the same persistent launch as the chained conversion next to them:
    exact copies for aligned and unaligned planes, u16 and f32."""
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(6)
    cases = [((48, 64), np.uint16, 0, 0), ((37, 53), np.uint16, 3, 1), ((40, 96), np.float32, 0, 0),
             ((17, 33), np.float32, 1, 1)]
    convs, srcs, dsts, wants = [], [], [], []
    for (h, w), dt, pad, off in cases:
        src = (rng.integers(0, 1024, size=(h, w), dtype=np.uint16) if dt == np.uint16
               else rng.random((h, w), dtype=np.float32))
        ptype = "word" if dt == np.uint16 else "float"
        convs.append(zg.ResizeConversion(w, h, ptype).set_depth(10 if dt == np.uint16 else 32)
                     .set_filter("spline36").set_dst_width(w).set_dst_height(h))
        s = empty(h, w, dt, pad, off)
        s.copy_(to_dev(src))
        srcs.append(s)
        dsts.append(empty(h, w, dt, pad, off))
        wants.append(src)
    src = rng.integers(0, 1024, size=(30, 40), dtype=np.uint16)
    convs.append(zg.ResizeConversion(40, 30, "word").set_depth(10).set_filter("spline36").set_dst_width(80)
                 .set_dst_height(60))
    srcs.append(to_dev(src))
    dsts.append(empty(60, 80, np.uint16))
    b = zg.Batch(convs)
    b.set_io(srcs, dsts)
    assert b.launch_count == 1  # the chained conversion and the four identity planes in one launch
    for mode in ("plain", "graph"):
        for d in dsts:
            d.zero_()
        (b.process if mode == "plain" else b.process_graph)()
        torch.cuda.synchronize()
        for d, w, (shape, dt, pad, off) in zip(dsts, wants, cases):
            np.testing.assert_array_equal(to_host(d, dt), w, err_msg=(mode, shape, pad, off))


def test_host_pipeline_matches_oracle(cuda, oracle):
    """HostPipeline: host planes in, host planes out, chunked with copies
    overlapping the launches; u16 bit-exact, over repeated runs."""
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(7)
    shapes = [(48, 64, 96, 54), (30, 40, 20, 15), (72, 128, 256, 144), (27, 48, 27, 48), (40, 40, 40, 40)]
    convs, hsrc, hdst, wants = [], [], [], []
    for sh, sw, dh, dw in shapes:
        src = rng.integers(0, 1024, size=(sh, sw), dtype=np.uint16)
        convs.append(zg.ResizeConversion(sw, sh, "word").set_depth(10).set_filter("spline36")
                     .set_dst_width(dw).set_dst_height(dh))
        hsrc.append(torch.from_numpy(src.view(np.int16)).pin_memory())
        hdst.append(torch.zeros((dh, dw), dtype=torch.int16).pin_memory())
        wants.append(oracle.resize_plane(src, dw, dh, "spline36", depth=10))
    pipe = zg.HostPipeline(convs, chunks=3)
    for _ in range(2):
        for h in hdst:
            h.zero_()
        pipe.run(hsrc, hdst)
        for h, w in zip(hdst, wants):
            np.testing.assert_array_equal(h.numpy().view(np.uint16), w)


def test_batch_autotune_keeps_results(cuda, oracle):
    """The autotuner may swap plans per job kind; u16 outputs stay bit-exact
    and f32 outputs stay within the FP64 error bound, in plain and graph
    launches."""
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(5)
    convs, srcs, dsts, checks = [], [], [], []
    for _ in range(3):  # identical u16 jobs are tuned once
        src = rng.integers(0, 1024, size=(135, 240), dtype=np.uint16)
        convs.append(zg.ResizeConversion(240, 135, "word").set_depth(10).set_filter("lanczos", 3)
                     .set_dst_width(480).set_dst_height(270))
        srcs.append(to_dev(src))
        dsts.append(empty(270, 480, np.uint16))
        checks.append(("u16", src, oracle.resize_plane(src, 480, 270, "lanczos", 3, depth=10)))
    for (sh, sw, dh, dw, kind, a) in ((540, 960, 34, 60, "lanczos", 4), (270, 480, 180, 320, "bicubic", math.nan)):
        src = band_limited(rng, sh, sw)
        convs.append(zg.ResizeConversion(sw, sh, "float").set_filter(kind, a).set_dst_width(dw).set_dst_height(dh))
        srcs.append(to_dev(src))
        dsts.append(empty(dh, dw, np.float32))
        checks.append(("f32", src, (dw, dh, kind, a)))
    b = zg.Batch(convs)
    b.set_io(srcs, dsts)
    b.autotune()
    for mode in ("plain", "graph"):
        for d in dsts:
            d.zero_()
        (b.process if mode == "plain" else b.process_graph)()
        torch.cuda.synchronize()
        for d, (kind, src, want) in zip(dsts, checks):
            if kind == "u16":
                np.testing.assert_array_equal(to_host(d, np.uint16), want, err_msg=mode)
            else:
                dw, dh, fk, fa = want
                _f32_check(oracle, src, to_host(d, np.float32), dw, dh, fk, fa, exact=False)


def test_graph_plane_params_known_answers(cuda):
    """graphbuilder_test.cpp:239-315 through the product's graph builder."""
    import zimg_gb300 as zg

    def fmt(w, h, ssw, ssh, loc, parity=0):
        return zg.image_format(w, h, "float", subsample_w=ssw, subsample_h=ssh, color_family=2,
                               chroma_location=loc, field_parity=parity)

    g = zg.Graph(fmt(64, 48, 1, 1, 4), fmt(64, 48, 0, 0, 1))
    present, p = g.plane_params(1)
    assert present == 2 and (p.src_width, p.src_height, p.dst_width, p.dst_height) == (32, 24, 64, 48)
    assert (p.shift_w, p.shift_h, p.subwidth, p.subheight) == (0.25, -0.25, 32.0, 24.0)
    assert g.plane_params(0)[0] == 1  # luma copied
    g = zg.Graph(fmt(64, 48, 0, 0, 1), fmt(64, 48, 1, 1, 4))
    p = g.plane_params(1)[1]
    assert (p.shift_w, p.shift_h, p.subwidth, p.subheight) == (-0.5, 0.5, 64.0, 48.0)
    for parity, sh in ((1, 0.25), (2, -0.25)):
        g = zg.Graph(fmt(64, 48, 0, 1, 1, parity), fmt(64, 48, 0, 1, 1))
        p0, p1 = g.plane_params(0)[1], g.plane_params(1)[1]
        assert (p0.shift_w, p0.shift_h, p0.subwidth, p0.subheight) == (0.0, sh, 64.0, 48.0)
        assert (p1.shift_w, p1.shift_h, p1.subwidth, p1.subheight) == (0.0, sh, 64.0, 24.0)
    g = zg.Graph(fmt(64, 48, 1, 1, 4, 1), fmt(64, 96, 1, 1, 4, 1))
    p0, p1 = g.plane_params(0)[1], g.plane_params(1)[1]
    assert (p0.shift_w, p0.shift_h, p0.subwidth, p0.subheight) == (0.0, 0.125, 64.0, 48.0)
    assert (p1.shift_w, p1.shift_h, p1.subwidth, p1.subheight) == (0.0, 0.0625, 32.0, 24.0)


def test_graph_yuv420_mpeg2_spline36(cuda, oracle):
    """The mixed-batch shape: YUV 4:2:0 u16, MPEG-2 (left) siting, Spline36 on all planes."""
    import torch
    import zimg_gb300 as zg
    from oracle import oracle as O
    rng = np.random.default_rng(0x5EED0004)
    for (sw, sh) in ((720, 480), (1280, 720), (3840, 2160)):
        sfmt = zg.image_format(sw, sh, "word", subsample_w=1, subsample_h=1, color_family=2, depth=10,
                               chroma_location=0)
        dfmt = zg.image_format(1920, 1080, "word", subsample_w=1, subsample_h=1, color_family=2, depth=10,
                               chroma_location=0)
        g = zg.Graph(sfmt, dfmt, zg.graph_params(resample_filter="spline36", resample_filter_uv="spline36"))
        srcs = [make_u16(rng, sh, sw, 10), make_u16(rng, sh // 2, sw // 2, 10), make_u16(rng, sh // 2, sw // 2, 10)]
        dsts = [empty(1080, 1920, np.uint16), empty(540, 960, np.uint16), empty(540, 960, np.uint16)]
        g.process([to_dev(s) for s in srcs] + [None], dsts + [None])
        torch.cuda.synchronize()
        sgeo = O.plane_geometry(dict(width=sw, height=sh, subsample_w=1, subsample_h=1, color="yuv",
                                     chroma_location=0))
        dgeo = O.plane_geometry(dict(width=1920, height=1080, subsample_w=1, subsample_h=1, color="yuv",
                                     chroma_location=0))
        for p in range(3):
            rp = O.resize_params(sgeo[p], dgeo[p])
            want = oracle.resize_plane(srcs[p], rp["dst_w"], rp["dst_h"], "spline36", depth=10,
                                       shift_w=rp["shift_w"], shift_h=rp["shift_h"], subwidth=rp["subwidth"],
                                       subheight=rp["subheight"], nthreads=16)
            np.testing.assert_array_equal(to_host(dsts[p], np.uint16), want, err_msg=str((sw, sh, p)))
