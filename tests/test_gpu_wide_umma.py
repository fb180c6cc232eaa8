"""The tcgen05 form of the FP32 wide-filter passes (wide_umma.cu): operands
split 3xTF32 in shared memory, accumulators in tensor memory. Like the
mma.sync form it is held to the FP64 error bound of the tensor-core passes:
no worse than twice zimg's C path's own max-abs error plus 1e-6
(test_gpu_resize.py states the same tolerance). ZG_WIDE_KERNEL selects the
form per launch."""
import math

import numpy as np
import pytest

from test_gpu_resize import F32_ABS_TOL, band_limited, empty, to_dev, to_host

pytestmark = pytest.mark.gpu


def run(src, dw, dh, kind, a, pad=0, offset=0, **kw):
    import torch
    import zimg_gb300 as zg
    h, w = src.shape
    r = zg.ResizeConversion(w, h, "float").set_filter(kind, a).set_dst_width(dw).set_dst_height(dh) \
        .set_shift_w(kw.get("shift_w", 0.0)).set_shift_h(kw.get("shift_h", 0.0)).set_engine("tensor").create()
    s = empty(h, w, np.float32, pad, offset)
    s.copy_(to_dev(src))
    d = empty(dh, dw, np.float32, pad, offset)
    r.process(s, d)
    torch.cuda.synchronize()
    return to_host(d, np.float32), r


def bound_check(oracle, src, got, dw, dh, kind, a, **kw):
    f64 = oracle.resize_plane(src, dw, dh, kind, a, mode="f64", nthreads=16, **kw)
    c = oracle.resize_plane(src, dw, dh, kind, a, mode="c", nthreads=16, **kw)
    err_gpu = float(np.max(np.abs(got.astype(np.float64) - f64)))
    err_c = float(np.max(np.abs(c.astype(np.float64) - f64)))
    assert err_gpu <= 2 * err_c + F32_ABS_TOL, (err_gpu, err_c)
    return err_gpu, err_c


# (src h, w) -> (dst h, w): both passes wide; column tiles of 256 and output
# tiles of 64 partial, band ends clamped, bands too wide for the tcgen05 form
# (> 160 taps: the mma.sync form runs)
SHAPES = [((1080, 1920), (67, 120)), ((517, 333), (31, 29)), ((600, 100), (9, 6)), ((1600, 1600), (16, 16)),
          ((130, 260), (9, 17)),
          ((517, 100), (31, 7)),     # 100 columns: one partial 256-column tile
          ((1080, 300), (54, 15))]   # 20x Lanczos-4: 160 taps, the widest band the tcgen05 form takes


@pytest.mark.parametrize("case", range(len(SHAPES)))
@pytest.mark.parametrize("kind,a", [("lanczos", 4), ("spline64", math.nan)])
def test_umma_f32_error_bound(cuda, oracle, monkeypatch, case, kind, a):
    monkeypatch.setenv("ZG_WIDE_KERNEL", "umma")
    rng = np.random.default_rng(4242 + case)
    (sh, sw), (dh, dw) = SHAPES[case]
    src = band_limited(rng, sh, sw)
    kw = dict(shift_w=float(rng.normal(0, 2)), shift_h=float(rng.normal(0, 2)))
    # aligned planes (16-byte base and stride) take the tcgen05 form: rows
    # padded to a multiple of 4 samples
    pad = (-sw) % 4 + 4 * int(rng.choice([0, 1, 3]))
    got, r = run(src, dw, dh, kind, a, pad=pad, **kw)
    assert r.info["engine"] == "tensor-passes", r.info
    bound_check(oracle, src, got, dw, dh, kind, a, **kw)


def test_umma_unaligned_plane_falls_back(cuda, oracle, monkeypatch):
    """A plane the tensor copies cannot address (4-byte offset) runs on the
    mma.sync form, with the same bound."""
    monkeypatch.setenv("ZG_WIDE_KERNEL", "umma")
    rng = np.random.default_rng(99)
    src = band_limited(rng, 517, 333)
    got, _ = run(src, 29, 31, "lanczos", 4, pad=1, offset=1)
    bound_check(oracle, src, got, 29, 31, "lanczos", 4)


def test_umma_and_mma_forms_agree(cuda, monkeypatch):
    """Both forms compute the same 3xTF32 sums; they differ only in the
    tensor core's internal addition order (a few ulp)."""
    rng = np.random.default_rng(7)
    src = band_limited(rng, 1080, 1920)
    outs = []
    for form in ("umma", "mma"):
        monkeypatch.setenv("ZG_WIDE_KERNEL", form)
        outs.append(run(src, 120, 67, "lanczos", 4)[0])
    assert float(np.max(np.abs(outs[0].astype(np.float64) - outs[1]))) < 1e-5


def test_default_choice_full_plane(cuda, oracle, lib, monkeypatch):
    """Without ZG_WIDE_KERNEL the vertical pass of the 16x downscale of a
    7680x4320 plane (150 tiles) takes the tcgen05 form and the horizontal pass
    the mma.sync form; the result is within the FP64 bound."""
    monkeypatch.delenv("ZG_WIDE_KERNEL", raising=False)
    rng = np.random.default_rng(31)
    src = rng.random((4320, 7680), dtype=np.float32)
    lib.zg_wide_forms_used(1)
    got, r = run(src, 480, 270, "lanczos", 4)
    assert lib.zg_wide_forms_used(1) == 3  # both forms ran
    bound_check(oracle, src, got, 480, 270, "lanczos", 4)


def test_batch_wide_jobs_match_single(cuda, lib, monkeypatch):
    """A batch of wide jobs (the bench's path, CUDA graph replay included)
    gives the same bits as the same conversions run one by one."""
    import torch
    import zimg_gb300 as zg
    monkeypatch.delenv("ZG_WIDE_KERNEL", raising=False)
    rng = np.random.default_rng(32)
    srcs = [rng.random((4320, 7680), dtype=np.float32) for _ in range(2)]
    singles = [run(s, 480, 270, "lanczos", 4)[0] for s in srcs]
    b = zg.Batch([zg.ResizeConversion(7680, 4320, "float").set_filter("lanczos", 4).set_dst_width(480)
                  .set_dst_height(270) for _ in srcs])
    dev_s = [to_dev(s) for s in srcs]
    dev_d = [torch.empty((270, 480), device="cuda") for _ in srcs]
    b.set_io(dev_s, dev_d)
    lib.zg_wide_forms_used(1)
    for graph in (False, True):
        for d in dev_d:
            d.zero_()
        if graph:
            b.process_graph()
        else:
            b.process()
        torch.cuda.synchronize()
        for d, want in zip(dev_d, singles):
            np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), want.view(np.uint32), err_msg=str(graph))
    assert lib.zg_wide_forms_used(1) & 2
