"""GPU colorspace conversion (zimg's ColorspaceConversion) through the C ABI
against the oracle's restatement of zimg's C path, which
tests/test_oracle_colorspace.py pins bit for bit against zimg's own code.

The plan (which operations, in which order) must match the oracle's exactly,
and plans made of matrices only must match zimg's C path bit for bit (same
float products and sums). Transfer functions use CUDA's powf / logf /
log10f / expf, which may differ from the C library's by a few units in the
last place, and ill-conditioned spots of the curves (PQ near black, the
square root of HLG at zero, the HLG system gamma on near-black luma) can
turn that into large differences between any two float evaluations. So the
bound is the one stated for floating point throughout: against the same
operations evaluated in FP64 (same float parameters), the GPU's error must be
no worse than 2x the C path's, per conversion and plane, with errors measured
relative to max(1, |FP64 value|), plus a slack of 2^-20 (8 units in the last
place at 1.0) where both errors are at the level of rounding: CUDA's log10f,
expf and powf are accurate to about 2 units, the C library's to under 1.
Measured over the 3,442 conversions of the pair sweep the largest ratio of
GPU to C-path error is 1.9."""
import itertools

import numpy as np
import pytest

from test_oracle_colorspace import FLAGS, SPACES, planes_for

pytestmark = pytest.mark.gpu

SLACK = 2.0 ** -20


def to_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_convert(planes, cin, cout, kw, in_place=False, pad=0):
    import torch
    import zimg_gb300 as zg
    h, w = planes[0].shape
    c = zg.ColorspaceConversion(w, h).set_csp_in(*cin).set_csp_out(*cout)
    if "peak" in kw:
        c.set_peak_luminance(kw["peak"])
    c.set_scene_referred(kw.get("scene", False)).set_approximate_gamma(kw.get("approximate", False))
    c.set_chromatic_adaptation(kw.get("adapt", False))
    conv = c.create()
    if pad:
        src = []
        for p in planes:
            buf = torch.zeros((h, w + pad), dtype=torch.float32, device="cuda")
            buf[:, 1:w + 1] = to_dev(p)
            src.append(buf[:, 1:w + 1])
    else:
        src = [to_dev(p) for p in planes]
    dst = src if in_place else [torch.empty((h, w), dtype=torch.float32, device="cuda") for _ in range(3)]
    conv.process(src, dst)
    torch.cuda.synchronize()
    return [d.cpu().numpy() for d in dst], conv.ops


def rel_err(x, ref64):
    """|x - ref| / max(1, |ref|), NaN where both are NaN, inf where only x is."""
    x = x.astype(np.float64)
    both = np.isnan(x) & np.isnan(ref64)
    e = np.abs(x - ref64) / np.maximum(1.0, np.abs(ref64))
    e[np.isnan(e)] = np.inf
    e[both] = 0.0
    e[np.isinf(ref64) & (x == ref64)] = 0.0
    return e


def check(oracle, planes, got, want, ops, what, cin, cout, kw):
    for k in range(3):
        g, w = got[k], want[k]
        both_nan = np.isnan(g) & np.isnan(w)
        if set(ops) <= {"matrix"}:
            np.testing.assert_array_equal(g.view(np.uint32)[~both_nan], w.view(np.uint32)[~both_nan],
                                          err_msg=f"{what} plane {k}: matrix-only plans round as zimg")
    if set(ops) <= {"matrix"}:
        return 0.0
    ref64, _ = oracle.colorspace(planes, cin, cout, fp64=True, **kw)
    worst = 0.0
    for k in range(3):
        eg = float(rel_err(got[k], ref64[k]).max())
        ec = float(rel_err(want[k], ref64[k]).max())
        assert eg <= 2.0 * ec + SLACK, f"{what} plane {k} ops {ops}: GPU error {eg:.3g} vs C path {ec:.3g} (vs FP64)"
        worst = max(worst, eg / (ec + SLACK))
    return worst


@pytest.mark.parametrize("flags", range(len(FLAGS)))
def test_colorspace_all_pairs(cuda, oracle, flags):
    kw = FLAGS[flags]
    rng = np.random.default_rng(1100 + flags)
    planes = planes_for(rng, 4, 64)
    n = 0
    for cin, cout in itertools.product(SPACES, SPACES):
        try:
            want, ops = oracle.colorspace(planes, cin, cout, **kw)
        except ValueError:
            import zimg_gb300 as zg
            with pytest.raises(zg.ZimgError):
                gpu_convert(planes, cin, cout, kw)
            continue
        got, gops = gpu_convert(planes, cin, cout, kw)
        assert gops == ops, f"{cin} -> {cout} {kw}: plan {gops} vs {ops}"
        check(oracle, planes, got, want, ops, f"{cin} -> {cout} {kw}", cin, cout, kw)
        n += 1
    assert n > 300


@pytest.mark.parametrize("pair", [((1, 1, 1), (9, 16, 9)), ((9, 18, 9), (1, 1, 1)), ((0, 13, 1), (14, 16, 9)),
                                  ((10, 14, 9), (0, 1, 12))])
def test_colorspace_full_plane(cuda, oracle, pair):
    """A 1080p frame, vector path; an offset copy of it (scalar path); in place."""
    cin, cout = pair
    rng = np.random.default_rng(1200)
    planes = planes_for(rng, 1080, 1920)
    want, ops = oracle.colorspace(planes, cin, cout)
    got, _ = gpu_convert(planes, cin, cout, {})
    check(oracle, planes, got, want, ops, f"{cin} -> {cout} 1080p", cin, cout, {})
    got2, _ = gpu_convert(planes, cin, cout, {}, pad=3)
    got3, _ = gpu_convert(planes, cin, cout, {}, in_place=True)
    for k in range(3):
        np.testing.assert_array_equal(got2[k], got[k])  # scalar path = vector path
        np.testing.assert_array_equal(got3[k], got[k])  # in place


def test_colorspace_identity_copies(cuda):
    rng = np.random.default_rng(1201)
    planes = planes_for(rng, 17, 33)
    got, ops = gpu_convert(planes, (1, 1, 1), (1, 6, 1), {})  # BT.601 transfer is BT.709
    assert ops == []
    for k in range(3):
        np.testing.assert_array_equal(got[k], planes[k])


def test_colorspace_errors(cuda):
    import zimg_gb300 as zg
    with pytest.raises(zg.ZimgError) as e:
        zg.ColorspaceConversion(8, 8).set_csp_in(1, 1, 1).set_csp_out(2, 2, 2).create()   # no path
    assert e.value.code == 3074
    with pytest.raises(zg.ZimgError) as e:
        zg.ColorspaceConversion(8, 8).set_csp_in(11, 1, 1).set_csp_out(0, 1, 1).create()  # YDZDX: not mapped
    assert e.value.code == 3074
    with pytest.raises(zg.ZimgError) as e:
        zg.ColorspaceConversion(8, 8).set_csp_in(1, 1, 1).set_csp_out(0, 300, 1).create()  # out of range
    assert e.value.code == 2049


GRAPH_CASES = [
    # (src type, depth, range, dst type, depth, range, size in, size out, colour in, out, subsampling in, out,
    #  colorspace in, out (matrix, transfer, primaries), dither, exact)
    ("byte", 8, 0, "byte", 8, 1, (640, 360), (640, 360), "yuv", "rgb", 1, 0, (1, 1, 1), (0, 1, 1), "none", True),
    ("word", 10, 0, "word", 10, 0, (1920, 1080), (1280, 720), "yuv", "yuv", 1, 1, (9, 14, 9), (1, 1, 1), "ordered",
     False),
    ("float", 32, 0, "float", 32, 0, (400, 300), (600, 450), "rgb", "yuv", 0, 1, (0, 13, 1), (1, 1, 1), "none", False),
    ("word", 16, 1, "byte", 8, 0, (640, 480), (640, 480), "rgb", "grey", 0, 0, (0, 1, 1), (1, 1, 1), "none", True),
    ("byte", 8, 1, "byte", 8, 1, (320, 240), (320, 240), "grey", "rgb", 0, 0, (1, 1, 1), (0, 13, 1), "none", False),
    ("word", 10, 0, "word", 10, 0, (640, 360), (640, 360), "grey", "yuv", 0, 1, (1, 1, 1), (1, 1, 1), "none", True),
    ("byte", 8, 0, "byte", 8, 0, (640, 360), (320, 180), "yuv", "grey", 1, 0, (1, 1, 1), (1, 1, 1), "none", True),
    ("half", 16, 0, "float", 32, 0, (640, 360), (640, 360), "yuv", "rgb", 1, 0, (9, 16, 9), (0, 16, 9), "none", True),
    ("word", 10, 0, "byte", 8, 0, (1280, 720), (1920, 1080), "yuv", "yuv", 1, 1, (9, 16, 9), (1, 1, 1),
     "error_diffusion", False),
]


@pytest.mark.parametrize("case", range(len(GRAPH_CASES)))
def test_graph_colorspace(cuda, oracle, case):
    """zg_graph with a colorspace or colour-family change, against the
    oracle's restatement of zimg's graph (connect_color_channels,
    graphbuilder.cpp:975-1014; grey_to_yuv / grey_to_rgb / yuv_to_grey
    :604-659). Conversions made of matrices only (and the family changes
    without a conversion) are bit-exact; with transfer functions, integer
    outputs may differ by one code value where the small float difference
    crosses a rounding boundary, and float outputs stay within 1e-3 of
    max(1, |value|) (the kernel's own bound against FP64 is tested above)."""
    import torch
    import zimg_gb300 as zg
    from oracle import oracle as O
    from test_gpu_depth import empty, to_host
    from test_gpu_depth import to_dev as to_dev_any
    from test_oracle_depth import make_src
    (st, sd, sr, dt, dd, dr, (sw, sh), (dw, dh), ci, co, subi, subo, csi, cso, dither, exact) = GRAPH_CASES[case]
    fam = {"grey": 0, "rgb": 1, "yuv": 2}
    sfmt = zg.image_format(sw, sh, st, depth=sd, pixel_range=sr, color_family=fam[ci], subsample_w=subi,
                           subsample_h=subi, chroma_location=0, matrix_coefficients=csi[0],
                           transfer_characteristics=csi[1], color_primaries=csi[2])
    dfmt = zg.image_format(dw, dh, dt, depth=dd, pixel_range=dr, color_family=fam[co], subsample_w=subo,
                           subsample_h=subo, chroma_location=0, matrix_coefficients=cso[0],
                           transfer_characteristics=cso[1], color_primaries=cso[2])
    dmap = {"none": 0, "ordered": 1, "random": 2, "error_diffusion": 3}
    g = zg.Graph(sfmt, dfmt, zg.graph_params(resample_filter="bicubic", resample_filter_uv="bilinear",
                                             dither_type=dmap[dither]))
    rng = np.random.default_rng(1300 + case)
    sgeo = O.plane_geometry(dict(width=sw, height=sh, subsample_w=subi, subsample_h=subi, color=ci, chroma_location=0))
    dgeo = O.plane_geometry(dict(width=dw, height=dh, subsample_w=subo, subsample_h=subo, color=co, chroma_location=0))
    n_in, n_out = (1 if ci == "grey" else 3), (1 if co == "grey" else 3)
    srcs, fs = [], []
    for p in range(n_in):
        f = O.PixelFormat(st, sd, bool(sr), ci == "yuv" and p > 0)
        x = make_src(rng, f, sgeo[p]["height"], sgeo[p]["width"], special=False)
        if not exact and st in ("byte", "word") and not sr:
            # legal video levels: beyond them PQ's curve overflows to inf and
            # a gamut matrix makes NaN, which error diffusion then carries
            # through the rest of the plane (zimg's C path does the same)
            lo, hi = 16 << (f.bits - 8), (240 if f.chroma else 235) << (f.bits - 8)
            x = np.clip(x, lo, hi).astype(x.dtype)
        srcs.append(x)
        fs.append(f)
    fd = [O.PixelFormat(dt, dd, bool(dr), co == "yuv" and p > 0) for p in range(n_out)]
    dsts = [empty(dgeo[p]["height"], dgeo[p]["width"], dt) for p in range(3 if co != "grey" else 1)]
    needs = not (csi == cso or (csi[1:] == cso[1:] and (ci == "grey" or (ci != "rgb" and co == "grey"))))
    if needs:
        wants = O.graph_colorspace(oracle, srcs, fs, fd, sgeo, dgeo, ci, co, csi, cso, "bicubic", "bilinear", dither)
    else:
        # family change alone: luma through its chain; chroma neutral, duplicated or dropped
        rp = None if (sw, sh) == (dw, dh) else O.resize_params(sgeo[0], dgeo[0])
        y = O.graph_plane_chain(oracle, srcs[0], fs[0], fd[0], rp, "bicubic", dither=dither, plane=0)
        wants = [y]
        if ci == "grey" and co == "yuv":
            neutral = (1 << (fd[0].bits - 1)) if dt in ("byte", "word") else 0
            wants += [np.full((dgeo[p]["height"], dgeo[p]["width"]), neutral, fd[0].dtype) for p in (1, 2)]
        elif ci == "grey" and co == "rgb":
            wants += [y.copy(), y.copy()]
    planes_in = [to_dev_any(x) for x in srcs] + [None] * (4 - n_in)
    planes_out = dsts + [None] * (4 - len(dsts))
    g.process(planes_in, planes_out)
    torch.cuda.synchronize()
    for p in range(len(wants)):
        got = to_host(dsts[p], fd[min(p, len(fd) - 1)].dtype)
        want = wants[p]
        what = f"{GRAPH_CASES[case]} plane {p}"
        if exact:
            np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=what)
        elif dt in ("byte", "word"):
            diff = np.abs(got.astype(np.int64) - want.astype(np.int64))
            assert diff.max() <= 1, f"{what}: max difference {diff.max()}"
            assert (diff > 0).mean() < 0.01, f"{what}: {(diff > 0).mean():.4f} of samples differ"
        else:
            err = np.abs(got.astype(np.float64) - want.astype(np.float64)) / np.maximum(1.0, np.abs(want))
            assert np.nanmax(err) <= 1e-3, f"{what}: max relative error {np.nanmax(err):.3g}"
