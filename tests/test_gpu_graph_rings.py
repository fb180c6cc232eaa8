"""Ring-buffer (line-masked) planes and user callbacks in the graph API, as
zimg_filter_graph_process takes them (zimg.h:387-433,455-484,550-552).

The source planes are rings of a few lines that the unpack callback refills
from whole planes on demand; the destination planes are rings that the pack
callback drains into whole planes. The result must equal the same graph
run on whole planes, bit for bit, and the callbacks must see every step of
lines exactly once, in order. A callback that fails aborts processing with
ZG_ERROR_USER_CALLBACK_FAILED.
"""
import numpy as np
import pytest

from test_gpu_resize import empty, make_u16, to_dev, to_host

pytestmark = pytest.mark.gpu


def _yuv_graph(zg, sw, sh, dw, dh, ptype="word", depth=10):
    sfmt = zg.image_format(sw, sh, ptype, subsample_w=1, subsample_h=1, color_family=2, depth=depth,
                           chroma_location=0)
    dfmt = zg.image_format(dw, dh, ptype, subsample_w=1, subsample_h=1, color_family=2, depth=depth,
                           chroma_location=0)
    return zg.Graph(sfmt, dfmt, zg.graph_params(resample_filter="spline36", resample_filter_uv="spline36"))


@pytest.mark.parametrize("src_lines,dst_lines", [(2, 2), (8, 16), (64, 4)])
def test_graph_ring_buffers_match_whole_planes(cuda, src_lines, dst_lines):
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(0x4171 + src_lines)
    sw, sh, dw, dh = 640, 360, 960, 540
    g = _yuv_graph(zg, sw, sh, dw, dh)
    assert g.input_buffering == 2 and g.output_buffering == 2
    srcs = [to_dev(make_u16(rng, sh, sw, 10)), to_dev(make_u16(rng, sh // 2, sw // 2, 10)),
            to_dev(make_u16(rng, sh // 2, sw // 2, 10))]
    want = [empty(dh, dw, np.uint16), empty(dh // 2, dw // 2, np.uint16), empty(dh // 2, dw // 2, np.uint16)]
    g.process(srcs + [None], want + [None])

    # rings: luma src_lines lines, chroma half of them (4:2:0)
    sr = [torch.zeros((src_lines, sw), dtype=torch.int16, device="cuda"),
          torch.zeros((src_lines // 2, sw // 2), dtype=torch.int16, device="cuda"),
          torch.zeros((src_lines // 2, sw // 2), dtype=torch.int16, device="cuda")]
    dr = [torch.zeros((dst_lines, dw), dtype=torch.int16, device="cuda"),
          torch.zeros((dst_lines // 2, dw // 2), dtype=torch.int16, device="cuda"),
          torch.zeros((dst_lines // 2, dw // 2), dtype=torch.int16, device="cuda")]
    got = [torch.zeros_like(w) for w in want]
    seen_in, seen_out = [], []

    def unpack(i, left, right):
        seen_in.append((i, left, right))
        sr[0][[i & (src_lines - 1), (i + 1) & (src_lines - 1)]] = srcs[0][i:i + 2]
        c = (i // 2) & (src_lines // 2 - 1)
        sr[1][c] = srcs[1][i // 2]
        sr[2][c] = srcs[2][i // 2]
        torch.cuda.synchronize()
        return 0

    def pack(i, left, right):
        seen_out.append((i, left, right))
        got[0][i:i + 2] = dr[0][[i & (dst_lines - 1), (i + 1) & (dst_lines - 1)]]
        c = (i // 2) & (dst_lines // 2 - 1)
        got[1][i // 2] = dr[1][c]
        got[2][i // 2] = dr[2][c]
        torch.cuda.synchronize()
        return 0

    g.process(sr + [None], dr + [None], src_masks=[src_lines - 1, src_lines // 2 - 1, src_lines // 2 - 1, None],
              dst_masks=[dst_lines - 1, dst_lines // 2 - 1, dst_lines // 2 - 1, None], unpack=unpack, pack=pack)
    torch.cuda.synchronize()
    assert seen_in == [(i, 0, sw) for i in range(0, sh, 2)]
    assert seen_out == [(i, 0, dw) for i in range(0, dh, 2)]
    for p in range(3):
        np.testing.assert_array_equal(to_host(got[p], np.uint16), to_host(want[p], np.uint16), err_msg=str(p))


def test_graph_callbacks_on_whole_planes_and_failure(cuda):
    import torch
    import zimg_gb300 as zg
    rng = np.random.default_rng(0x4172)
    g = _yuv_graph(zg, 320, 180, 480, 270)
    srcs = [to_dev(make_u16(rng, 180, 320, 10)), to_dev(make_u16(rng, 90, 160, 10)),
            to_dev(make_u16(rng, 90, 160, 10))]
    dsts = [empty(270, 480, np.uint16), empty(135, 240, np.uint16), empty(135, 240, np.uint16)]
    calls = []
    g.process(srcs + [None], dsts + [None], unpack=lambda i, l, r: calls.append(("u", i)) or 0,
              pack=lambda i, l, r: calls.append(("p", i)) or 0)
    torch.cuda.synchronize()
    assert [c for c in calls if c[0] == "u"] == [("u", i) for i in range(0, 180, 2)]
    assert [c for c in calls if c[0] == "p"] == [("p", i) for i in range(0, 270, 2)]
    with pytest.raises(zg.ZimgError) as e:
        g.process(srcs + [None], dsts + [None], unpack=lambda i, l, r: 1 if i == 10 else 0)
    assert e.value.code == 2  # ZG_ERROR_USER_CALLBACK_FAILED
    with pytest.raises(zg.ZimgError) as e:
        g.process(srcs + [None], dsts + [None], src_masks=[2, None, None, None])  # not 2^n - 1
    assert e.value.code == 2048  # ZG_ERROR_ILLEGAL_ARGUMENT
