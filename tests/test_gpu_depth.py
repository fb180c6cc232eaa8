"""GPU parity of the depth conversion (zimg's DepthConversion) through the C
ABI: bit-exact against the oracle's restatement of zimg's C path (which
tests/test_oracle_depth.py pins against zimg's own code), on aligned
planes (vector path), odd widths and offset planes (scalar path), the golden
planes, and a depth -> resize -> depth pipeline."""
import os

import numpy as np
import pytest

from test_oracle_depth import CASES, GOLDEN, make_src

pytestmark = pytest.mark.gpu

TORCH_DT = {"byte": "uint8", "word": "int16", "half": "int16", "float": "float32"}


def to_dev(a):
    import torch
    if a.dtype == np.uint16:
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def empty(h, w, ptype, offset=0):
    import torch
    dt = getattr(torch, TORCH_DT[ptype])
    buf = torch.zeros(h * w + offset + 16, dtype=dt, device="cuda")
    return buf[offset:offset + h * w].view(h, w)


def to_host(t, np_dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if np_dtype == np.uint16 else a


def convert(src, fin, fout, dither, plane, offset=0):
    import torch
    import zimg_gb300 as zg
    h, w = src.shape
    c = zg.DepthConversion(w, h).set_pixel_in(fin.type, fin.bits, fin.fullrange, fin.chroma) \
        .set_pixel_out(fout.type, fout.bits, fout.fullrange, fout.chroma).set_dither_type(dither) \
        .set_plane(plane).create()
    if offset:
        s = empty(h, w, fin.type, offset)
        s.copy_(to_dev(src))
    else:
        s = to_dev(src)
    d = empty(h, w, fout.type, offset)
    c.process(s, d)
    torch.cuda.synchronize()
    return to_host(d, fout.dtype), c.mode


@pytest.mark.parametrize("case", range(len(CASES)))
def test_depth_bitexact(cuda, oracle, case):
    fin, fout, dither = CASES[case]
    rng = np.random.default_rng(300 + case)
    for (h, w), offset in (((64, 256), 0), ((41, 157), 0), ((33, 200), 3)):
        src = make_src(rng, fin, h, w)
        for plane in range(4):
            got, mode = convert(src, fin, fout, dither, plane, offset)
            want = oracle.depth_convert(src, fin, fout, dither, plane)
            np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8),
                                          err_msg=f"{CASES[case]} {h}x{w}+{offset} plane {plane} ({mode})")
        assert mode == {0: "copy", 1: "left_shift", 2: "to_float", 3: "dither"}[oracle.depth_mode(fin, fout, dither)]


ED_PLANES = [
    # (pixel in, pixel out, height, width): whole planes of the usual sizes,
    # a band per warp and several, tall and narrow, wide and short
    (CASES[28][0], CASES[28][1], 1080, 1920),
    (CASES[29][0], CASES[29][1], 2160, 3840),
    (CASES[30][0], CASES[30][1], 540, 960),
    (CASES[31][0], CASES[31][1], 720, 1280),
    (CASES[33][0], CASES[33][1], 5000, 100),
    (CASES[32][0], CASES[32][1], 64, 40000),
    (CASES[34][0], CASES[34][1], 97, 3),
    (CASES[28][0], CASES[28][1], 1, 1),
    (CASES[28][0], CASES[28][1], 4320, 7680),
]


@pytest.mark.parametrize("case", range(len(ED_PLANES)))
def test_error_diffusion_whole_planes(cuda, oracle, case):
    """Floyd-Steinberg over whole planes: one serial recurrence per plane, run
    as a wavefront of bands; equal to the oracle sample for sample."""
    fin, fout, h, w = ED_PLANES[case]
    rng = np.random.default_rng(700 + case)
    src = make_src(rng, fin, h, w, special=False)
    got, mode = convert(src, fin, fout, "error_diffusion", 0)
    want = oracle.depth_convert(src, fin, fout, "error_diffusion", 0)
    assert mode == "dither"
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=f"{h}x{w}")


def test_error_diffusion_non_finite(cuda, oracle):
    """zimg's C path keeps a NaN through the clamp, stores 0 for it and
    carries its NaN error to the samples after and below it; infinities clamp
    to the range ends with a zero error."""
    from oracle.oracle import PixelFormat as PF
    rng = np.random.default_rng(77)
    src = rng.random((300, 500), dtype=np.float32)
    src[7, 11] = np.nan
    src[150, 499] = np.nan
    src[299, 0] = np.nan
    src[40, 40:44] = [np.inf, -np.inf, np.inf, -0.0]
    for fout in (PF("byte", 8), PF("word", 12, True)):
        got, _ = convert(src, PF("float"), fout, "error_diffusion", 0)
        want = oracle.depth_convert(src, PF("float"), fout, "error_diffusion", 0)
        np.testing.assert_array_equal(got, want)
        assert (got[8:, 12:] == 0).any()


def test_random_dither_whole_planes(cuda, oracle):
    """Blue-noise dither on a 1080p plane, all four plane variants (the
    table's offsets by plane index)."""
    from oracle.oracle import PixelFormat as PF
    rng = np.random.default_rng(78)
    src = rng.integers(0, 1 << 16, size=(1080, 1920)).astype(np.uint16)
    for plane in range(4):
        got, _ = convert(src, PF("word", 16), PF("byte", 8), "random", plane)
        want = oracle.depth_convert(src, PF("word", 16), PF("byte", 8), "random", plane)
        np.testing.assert_array_equal(got, want, err_msg=f"plane {plane}")


def test_error_diffusion_too_wide(cuda):
    """A plane whose wavefront shape fits no shared-memory budget is refused
    at creation (ZG_ERROR_UNSUPPORTED_OPERATION), before any launch."""
    import zimg_gb300 as zg
    with pytest.raises(zg.ZimgError) as e:
        zg.DepthConversion(70000, 2000).set_pixel_in("word", 10).set_pixel_out("byte", 8) \
            .set_dither_type("error_diffusion").create()
    assert "error diffusion" in str(e.value)


def test_depth_golden(cuda):
    data = np.load(GOLDEN)
    for k in range(int(data["n"])):
        fin, fout, dither = CASES[int(data[f"case{k}"])]
        got, _ = convert(data[f"src{k}"], fin, fout, dither, int(data[f"plane{k}"]))
        np.testing.assert_array_equal(got.view(np.uint8), data[f"out{k}"].view(np.uint8), err_msg=f"golden {k}")


def test_depth_resize_depth_pipeline(cuda, oracle):
    """8-bit source -> 10-bit (left shift) -> Lanczos-3 2x on the tensor-core
    path -> 8-bit with ordered dither, as zimg's graph chains them."""
    import torch
    import zimg_gb300 as zg
    from oracle.oracle import PixelFormat as PF
    rng = np.random.default_rng(9)
    h, w = 135, 240
    src = rng.integers(16, 236, size=(h, w)).astype(np.uint8)
    f8, f10 = PF("byte", 8), PF("word", 10)
    up = zg.DepthConversion(w, h).set_pixel_in("byte", 8).set_pixel_out("word", 10).create()
    rs = zg.ResizeConversion(w, h, "word").set_depth(10).set_filter("lanczos", 3).set_dst_width(2 * w) \
        .set_dst_height(2 * h).create()
    down = zg.DepthConversion(2 * w, 2 * h).set_pixel_in("word", 10).set_pixel_out("byte", 8) \
        .set_dither_type("ordered").create()
    a = to_dev(src)
    b = torch.empty((h, w), dtype=torch.int16, device="cuda")
    c = torch.empty((2 * h, 2 * w), dtype=torch.int16, device="cuda")
    d = torch.empty((2 * h, 2 * w), dtype=torch.uint8, device="cuda")
    up.process(a, b)
    rs.process(b, c)
    down.process(c, d)
    torch.cuda.synchronize()
    w10 = oracle.depth_convert(src, f8, f10)
    r10 = oracle.resize_plane(w10, 2 * w, 2 * h, "lanczos", 3, depth=10, mode="c")
    want = oracle.depth_convert(r10, f10, f8, "ordered", 0)
    np.testing.assert_array_equal(d.cpu().numpy(), want)
    assert rs.info["engine"] == "tensor"


GRAPH_CASES = [
    # (src type, depth, range, dst type, depth, range, size in, size out, color, dither)
    ("byte", 8, 0, "word", 10, 0, (1920, 1080), (1280, 720), 2, "none"),      # convert, then resize in WORD 10
    ("float", 32, 0, "byte", 8, 0, (640, 360), (1280, 720), 2, "ordered"),   # resize in FLOAT, dither after
    ("byte", 8, 1, "byte", 8, 1, (720, 480), (960, 540), 0, "ordered"),      # full range BYTE: WORD 16 chain
    ("word", 10, 0, "byte", 8, 0, (1280, 720), (1280, 720), 2, "ordered"),   # depth only
    ("word", 16, 1, "float", 32, 0, (400, 300), (800, 600), 1, "none"),      # RGB, to float after resize
    ("half", 16, 0, "half", 16, 0, (1280, 720), (1920, 1080), 2, "none"),    # HALF: resized in FLOAT
    ("half", 16, 0, "byte", 8, 0, (1920, 1080), (960, 540), 2, "ordered"),
    ("float", 32, 0, "byte", 8, 0, (640, 360), (1280, 720), 2, "random"),    # blue-noise dither after resize
    ("word", 16, 1, "byte", 8, 1, (1280, 720), (1920, 1080), 1, "error_diffusion"),  # RGB, diffused after
    ("word", 10, 0, "byte", 8, 0, (1280, 720), (1280, 720), 2, "error_diffusion"),   # depth only
]


@pytest.mark.parametrize("case", range(len(GRAPH_CASES)))
def test_graph_depth_around_resize(cuda, oracle, case):
    """zg_graph with pixel format changes: every plane equals the oracle's
    restatement of zimg's graph chain (depth -> resize -> depth)."""
    import torch
    import zimg_gb300 as zg
    from oracle import oracle as O
    st, sd, sr, dt, dd, dr, (sw, sh), (dw, dh), color, dither = GRAPH_CASES[case]
    sub = 1 if color == 2 else 0
    sfmt = zg.image_format(sw, sh, st, depth=sd, pixel_range=sr, color_family=color, subsample_w=sub,
                           subsample_h=sub, chroma_location=0)
    dfmt = zg.image_format(dw, dh, dt, depth=dd, pixel_range=dr, color_family=color, subsample_w=sub,
                           subsample_h=sub, chroma_location=0)
    dmap = {"none": 0, "ordered": 1, "random": 2, "error_diffusion": 3}
    g = zg.Graph(sfmt, dfmt, zg.graph_params(resample_filter="lanczos", resample_filter_uv="bicubic",
                                             dither_type=dmap[dither]))
    rng = np.random.default_rng(600 + case)
    nplanes = 1 if color == 0 else 3
    sgeo = O.plane_geometry(dict(width=sw, height=sh, subsample_w=sub, subsample_h=sub,
                                 color=["grey", "rgb", "yuv"][color], chroma_location=0))
    dgeo = O.plane_geometry(dict(width=dw, height=dh, subsample_w=sub, subsample_h=sub,
                                 color=["grey", "rgb", "yuv"][color], chroma_location=0))
    srcs, dsts, wants = [], [], []
    for p in range(nplanes):
        uv = color == 2 and p > 0
        fs = O.PixelFormat(st, sd, bool(sr), uv)
        fd = O.PixelFormat(dt, dd, bool(dr), uv)
        ph, pw = sgeo[p]["height"], sgeo[p]["width"]
        # finite samples: dense tap windows carry a non-finite sample further than zimg does
        src = make_src(rng, fs, ph, pw, special=False)
        srcs.append(src)
        dsts.append(empty(dgeo[p]["height"], dgeo[p]["width"], dt))
        same = (sw, sh) == (dw, dh)
        rp = None if same else O.resize_params(sgeo[p], dgeo[p])
        kind = "bicubic" if uv else "lanczos"
        wants.append(O.graph_plane_chain(oracle, src, fs, fd, rp, kind, dither=dither, plane=p))
    g.process([to_dev(s) for s in srcs] + [None] * (4 - nplanes), dsts + [None] * (4 - nplanes))
    torch.cuda.synchronize()
    for p in range(nplanes):
        got = to_host(dsts[p], O.PixelFormat(dt, dd).dtype)
        np.testing.assert_array_equal(got.view(np.uint8), wants[p].view(np.uint8),
                                      err_msg=f"{GRAPH_CASES[case]} plane {p}")


UNRESIZE_GRAPH_CASES = [
    # (src type, depth, range, dst type, depth, range, size in, size out, color, dither)
    ("float", 32, 0, "float", 32, 0, (1280, 720), (960, 540), 0, "none"),   # FLOAT in and out
    ("word", 10, 0, "word", 10, 0, (1920, 1080), (1280, 720), 2, "none"),   # to FLOAT, unresize, back to WORD
    ("byte", 8, 0, "byte", 8, 0, (960, 540), (640, 360), 1, "ordered"),    # RGB BYTE, dithered back
]


@pytest.mark.parametrize("case", range(len(UNRESIZE_GRAPH_CASES)))
def test_graph_unresize(cuda, oracle, case):
    """zimg's graph with resample_filter ZIMG_RESIZE_UNRESIZE (zimg.cpp:21,450;
    graphbuilder.cpp:761-790): every plane converted to FLOAT, unresized to
    the output size, converted to the output format; equal to the oracle's
    chain bit for bit."""
    import torch
    import zimg_gb300 as zg
    from oracle import oracle as O
    st, sd, sr, dt, dd, dr, (sw, sh), (dw, dh), color, dither = UNRESIZE_GRAPH_CASES[case]
    sub = 1 if color == 2 else 0
    sfmt = zg.image_format(sw, sh, st, depth=sd, pixel_range=sr, color_family=color, subsample_w=sub,
                           subsample_h=sub, chroma_location=0)
    dfmt = zg.image_format(dw, dh, dt, depth=dd, pixel_range=dr, color_family=color, subsample_w=sub,
                           subsample_h=sub, chroma_location=0)
    g = zg.Graph(sfmt, dfmt, zg.graph_params(resample_filter="unresize", dither_type={"none": 0, "ordered": 1}[dither]))
    rng = np.random.default_rng(650 + case)
    nplanes = 1 if color == 0 else 3
    cname = ["grey", "rgb", "yuv"][color]
    sgeo = O.plane_geometry(dict(width=sw, height=sh, subsample_w=sub, subsample_h=sub, color=cname, chroma_location=0))
    dgeo = O.plane_geometry(dict(width=dw, height=dh, subsample_w=sub, subsample_h=sub, color=cname, chroma_location=0))
    srcs, dsts, wants = [], [], []
    for p in range(nplanes):
        uv = color == 2 and p > 0
        fs = O.PixelFormat(st, sd, bool(sr), uv)
        fd = O.PixelFormat(dt, dd, bool(dr), uv)
        src = make_src(rng, fs, sgeo[p]["height"], sgeo[p]["width"], special=False)
        srcs.append(src)
        dsts.append(empty(dgeo[p]["height"], dgeo[p]["width"], dt))
        rp = O.resize_params(sgeo[p], dgeo[p])
        wants.append(O.graph_plane_chain(oracle, src, fs, fd, rp, "unresize", dither=dither, plane=p))
    g.process([to_dev(s) for s in srcs] + [None] * (4 - nplanes), dsts + [None] * (4 - nplanes))
    torch.cuda.synchronize()
    for p in range(nplanes):
        got = to_host(dsts[p], O.PixelFormat(dt, dd).dtype)
        np.testing.assert_array_equal(got.view(np.uint8), wants[p].view(np.uint8),
                                      err_msg=f"{UNRESIZE_GRAPH_CASES[case]} plane {p}")


def test_graph_unresize_refusals(cuda):
    """A partial active region (graphbuilder.cpp:761-766) and a larger output
    (bilinear.cpp:109-110) are RESAMPLING_NOT_AVAILABLE."""
    import zimg_gb300 as zg
    params = zg.graph_params(resample_filter="unresize")
    cases = [(zg.image_format(640, 360, "float", active_region=(0.5, 0.0, 600.0, 360.0)), zg.image_format(320, 180, "float")),
             (zg.image_format(640, 360, "float"), zg.image_format(960, 180, "float"))]
    for s, d in cases:
        with pytest.raises(zg.ZimgError) as e:
            zg.Graph(s, d, params)
        assert e.value.code == 3076


ALPHA_CASES = [
    # (src type, depth, range, dst type, depth, range, size in, size out, color,
    #  subsampling in, out, dither, alpha type, premultiplied chain expected)
    ("word", 10, 0, "byte", 8, 0, (640, 360), (640, 360), 2, 1, 1, "ordered", 1, False),   # depth only
    ("byte", 8, 1, "word", 16, 1, (640, 360), (960, 540), 1, 0, 0, "none", 2, False),      # premultiplied input
    ("word", 10, 0, "byte", 8, 0, (1280, 720), (640, 360), 2, 1, 1, "ordered", 1, True),   # straight, resized
    ("float", 32, 0, "float", 32, 0, (400, 300), (600, 450), 1, 0, 0, "none", 1, True),
    ("byte", 8, 0, "byte", 8, 0, (320, 240), (480, 360), 0, 0, 0, "error_diffusion", 1, True),
    ("half", 16, 0, "word", 12, 0, (640, 480), (320, 240), 2, 1, 1, "random", 1, True),
    ("word", 10, 0, "word", 10, 0, (640, 360), (640, 360), 2, 1, 0, "none", 1, True),     # 4:2:0 -> 4:4:4 only
    ("word", 16, 1, "byte", 8, 1, (512, 512), (512, 512), 1, 0, 0, "random", 1, False),    # full-range alpha depth change
]


def _alpha_plane(rng, f, h, w):
    if f.type in ("float", "half"):
        x = (rng.random((h, w), dtype=np.float32) * 1.2 - 0.1).astype(np.float32)  # a little outside [0, 1]
        x[:, : w // 8] = 0.0                                                          # transparent columns
        return x.astype(np.float16).view(np.uint16) if f.type == "half" else x
    x = rng.integers(0, 1 << f.bits, size=(h, w)).astype(f.dtype)
    x[:, : w // 8] = 0
    return x


@pytest.mark.parametrize("case", range(len(ALPHA_CASES)))
def test_graph_alpha(cuda, oracle, case):
    """Graphs with an alpha plane: alpha depth changes (alpha is full range in
    the integer types, graphbuilder.cpp:404-408), premultiplied alpha resized
    plane by plane, and straight alpha through an interpolating resize, which
    zimg premultiplies in FLOAT 4:4:4 (graphbuilder.cpp:594-600,1019-1068);
    every plane equal to the oracle's restatement."""
    import torch
    import zimg_gb300 as zg
    from oracle import oracle as O
    st, sd, sr, dt, dd, dr, (sw, sh), (dw, dh), color, subi, subo, dither, alpha, premul = ALPHA_CASES[case]
    cname = ["grey", "rgb", "yuv"][color]
    sfmt = zg.image_format(sw, sh, st, depth=sd, pixel_range=sr, color_family=color, subsample_w=subi,
                           subsample_h=subi, chroma_location=0, alpha=alpha)
    dfmt = zg.image_format(dw, dh, dt, depth=dd, pixel_range=dr, color_family=color, subsample_w=subo,
                           subsample_h=subo, chroma_location=0, alpha=alpha)
    dmap = {"none": 0, "ordered": 1, "random": 2, "error_diffusion": 3}
    g = zg.Graph(sfmt, dfmt, zg.graph_params(resample_filter="lanczos", resample_filter_uv="bicubic",
                                             dither_type=dmap[dither]))
    rng = np.random.default_rng(800 + case)
    ncolor = 1 if color == 0 else 3
    sgeo = O.plane_geometry(dict(width=sw, height=sh, subsample_w=subi, subsample_h=subi, color=cname,
                                 chroma_location=0))
    dgeo = O.plane_geometry(dict(width=dw, height=dh, subsample_w=subo, subsample_h=subo, color=cname,
                                 chroma_location=0))
    srcs, fss, fds, dsts = [], [], [], []
    for p in range(ncolor):
        uv = color == 2 and p > 0
        fs, fd = O.PixelFormat(st, sd, bool(sr), uv), O.PixelFormat(dt, dd, bool(dr), uv)
        srcs.append(make_src(rng, fs, sgeo[p]["height"], sgeo[p]["width"], special=False))
        fss.append(fs)
        fds.append(fd)
        dsts.append(empty(dgeo[p]["height"], dgeo[p]["width"], dt))
    is_int = lambda t: t in ("byte", "word")  # noqa: E731
    fa_s, fa_d = O.PixelFormat(st, sd, is_int(st), False), O.PixelFormat(dt, dd, is_int(dt), False)
    srcs.append(_alpha_plane(rng, fa_s, sh, sw))
    fss.append(fa_s)
    fds.append(fa_d)
    dsts.append(empty(dh, dw, dt))
    if premul:
        wants = O.graph_straight_alpha(oracle, srcs, fss, fds, sgeo, dgeo, cname, "lanczos", "bicubic", dither)
    else:
        wants = []
        for k in range(ncolor + 1):
            p = 3 if k == ncolor else k
            gs, gd = (sgeo[0], dgeo[0]) if p == 3 or color != 2 else (sgeo[p], dgeo[p])
            rp = None if (sw, sh) == (dw, dh) and subi == subo else O.resize_params(gs, gd)
            kind = "bicubic" if color == 2 and p in (1, 2) else "lanczos"
            wants.append(O.graph_plane_chain(oracle, srcs[k], fss[k], fds[k], rp, kind, dither=dither, plane=p))
    planes_in = [to_dev(s) for s in srcs[:ncolor]] + [None] * (3 - ncolor) + [to_dev(srcs[ncolor])]
    planes_out = dsts[:ncolor] + [None] * (3 - ncolor) + [dsts[ncolor]]
    g.process(planes_in, planes_out)
    torch.cuda.synchronize()
    for k in range(ncolor + 1):
        got = to_host(dsts[k], O.PixelFormat(dt, dd).dtype)
        np.testing.assert_array_equal(got.view(np.uint8), wants[k].view(np.uint8),
                                      err_msg=f"{ALPHA_CASES[case]} plane {k}")
