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
