"""GPU parity of unresize (zimg's UnresizeConversion) through the C ABI:
bit-exact against the oracle's restatement of zimg's C path (pinned against
zimg's own code by tests/test_oracle_unresize.py), on the cases and golden
planes, a full-HD plane, and a bottom-up source."""
import numpy as np
import pytest

from test_oracle_unresize import CASES, GOLDEN, make_src

pytestmark = pytest.mark.gpu


def run(src, ow, oh, sw=0.0, sh=0.0):
    import torch
    import zimg_gb300 as zg
    uh, uw = src.shape
    u = zg.UnresizeConversion(uw, uh).set_orig_width(ow).set_orig_height(oh).set_shift_w(sw).set_shift_h(sh).create()
    s = torch.from_numpy(np.ascontiguousarray(src)).cuda()
    d = torch.zeros((oh, ow), dtype=torch.float32, device="cuda")
    u.process(s, d)
    torch.cuda.synchronize()
    return d.cpu().numpy()


@pytest.mark.parametrize("case", range(len(CASES)))
def test_unresize_bitexact(cuda, oracle, case):
    uw, uh, ow, oh, sw, sh = CASES[case]
    src = make_src(np.random.default_rng(950 + case), uh, uw)
    np.testing.assert_array_equal(run(src, ow, oh, sw, sh).view(np.uint32),
                                  oracle.unresize_plane(src, ow, oh, sw, sh).view(np.uint32), err_msg=str(CASES[case]))


def test_unresize_golden(cuda):
    data = np.load(GOLDEN)
    for k in range(int(data["n"])):
        uw, uh, ow, oh, sw, sh = CASES[int(data[f"case{k}"])]
        np.testing.assert_array_equal(run(data[f"src{k}"], ow, oh, sw, sh).view(np.uint32),
                                      data[f"out{k}"].view(np.uint32), err_msg=f"golden {k}")


def test_unresize_full_hd(cuda, oracle):
    src = make_src(np.random.default_rng(99), 1080, 1920)
    np.testing.assert_array_equal(run(src, 1280, 720).view(np.uint32),
                                  oracle.unresize_plane(src, 1280, 720).view(np.uint32))
