"""GPU parity of the chained u16 kernel's two forms, and its bounded waits.

The TMA form (producer warp, mbarrier pipeline) is the default wherever the
source planes admit a tensor map; ZG_CHAIN_TMA=0 selects the cp.async form,
which also runs planes that are not 16-byte aligned. The switch is read once
per process, so the conversions run in a child process with the variable
set; the parent checks the child's planes against the oracle (u16:
bit-exact against zimg's C path) and that no bounded pipeline wait ran out.

test_bounded_wait_runs_out makes one consumer wait of the TMA form run out
on purpose: a test hook stops the producer of CTA 0 from arming one group's
stage (no copy is issued for it) and shortens every wait to 1 ms. The
kernel must return on its own, the pipeline status must name the wait, and
the next conversion on the same context must be bit-exact again.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (src_w, src_h, dst_w, dst_h, filter, depth): H-first upscales, a V-first
# downscale with a 3-window vertical filter, odd sizes
SINGLE = [
    (1920, 1080, 3840, 2160, "lanczos", 10),
    (720, 480, 1920, 1080, "spline36", 10),
    (3840, 2160, 1920, 1080, "spline36", 10),
    (333, 97, 1001, 500, "lanczos", 8),
    (640, 480, 427, 320, "bicubic", 10),
]
BATCH = [(720, 480, 1920, 1080), (360, 240, 960, 540), (1280, 720, 1920, 1080), (640, 360, 960, 540),
         (1920, 1080, 1920, 1080)]

CHILD = r"""
import json, os, sys
import numpy as np
import torch
sys.path.insert(0, os.environ["ZG_ROOT"])
import zimg_gb300 as zg

out = sys.argv[1]
cfg = json.load(open(os.path.join(out, "cfg.json")))
lib = zg.load()
lib.zg_pipeline_status(1)
res = {"single_engines": [], "status": []}

def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).cuda()

for i, (sw, sh, dw, dh, kind, depth) in enumerate(cfg["single"]):
    src = np.load(os.path.join(out, f"src{i}.npy"))
    conv = zg.ResizeConversion(sw, sh, "word").set_depth(depth).set_filter(kind).set_dst_width(dw).set_dst_height(dh)
    r = conv.create()
    d = torch.zeros((dh, dw), dtype=torch.int16, device="cuda")
    r.process(dev(src), d)
    torch.cuda.synchronize()
    np.save(os.path.join(out, f"got{i}.npy"), d.cpu().numpy().view(np.uint16))
    res["single_engines"].append(r.info["engine"])
res["status"].append(int(lib.zg_pipeline_status(1)))

convs, srcs, dsts = [], [], []
for i, (sw, sh, dw, dh) in enumerate(cfg["batch"]):
    src = np.load(os.path.join(out, f"bsrc{i}.npy"))
    convs.append(zg.ResizeConversion(sw, sh, "word").set_depth(10).set_filter("spline36")
                 .set_dst_width(dw).set_dst_height(dh))
    srcs.append(dev(src))
    dsts.append(torch.zeros((dh, dw), dtype=torch.int16, device="cuda"))
b = zg.Batch(convs)
b.set_io(srcs, dsts)
for mode in ("plain", "graph"):
    for d in dsts:
        d.zero_()
    (b.process if mode == "plain" else b.process_graph)()
    torch.cuda.synchronize()
    for i, d in enumerate(dsts):
        np.save(os.path.join(out, f"bgot_{mode}{i}.npy"), d.cpu().numpy().view(np.uint16))
res["status"].append(int(lib.zg_pipeline_status(1)))
json.dump(res, open(os.path.join(out, "res.json"), "w"))
"""


def test_cp_async_form_bitexact(cuda, oracle, tmp_path):
    rng = np.random.default_rng(0x7A)
    for i, (sw, sh, dw, dh, kind, depth) in enumerate(SINGLE):
        np.save(tmp_path / f"src{i}.npy", rng.integers(0, 1 << depth, size=(sh, sw), dtype=np.uint16))
    for i, (sw, sh, dw, dh) in enumerate(BATCH):
        np.save(tmp_path / f"bsrc{i}.npy", rng.integers(0, 1024, size=(sh, sw), dtype=np.uint16))
    json.dump({"single": SINGLE, "batch": BATCH}, open(tmp_path / "cfg.json", "w"))
    env = dict(os.environ, ZG_CHAIN_TMA="0", ZG_ROOT=ROOT)
    child = subprocess.run([sys.executable, "-c", CHILD, str(tmp_path)], env=env, capture_output=True, text=True,
                           timeout=600)
    assert child.returncode == 0, child.stderr[-3000:]
    res = json.load(open(tmp_path / "res.json"))
    assert res["status"] == [0, 0], "a pipelined kernel's bounded wait ran out"
    assert "tensor" in res["single_engines"]
    for i, (sw, sh, dw, dh, kind, depth) in enumerate(SINGLE):
        src = np.load(tmp_path / f"src{i}.npy")
        want = oracle.resize_plane(src, dw, dh, kind, depth=depth, mode="c", nthreads=16)
        np.testing.assert_array_equal(np.load(tmp_path / f"got{i}.npy"), want, err_msg=str(SINGLE[i]))
    for i, (sw, sh, dw, dh) in enumerate(BATCH):
        src = np.load(tmp_path / f"bsrc{i}.npy")
        want = oracle.resize_plane(src, dw, dh, "spline36", depth=10, mode="c", nthreads=16)
        for mode in ("plain", "graph"):
            np.testing.assert_array_equal(np.load(tmp_path / f"bgot_{mode}{i}.npy"), want,
                                          err_msg=f"{mode} {BATCH[i]}")


FAULT_CHILD = r"""
import json, os, sys, time
import numpy as np
import torch
sys.path.insert(0, os.environ["ZG_ROOT"])
import zimg_gb300 as zg

out = sys.argv[1]
lib = zg.load()
lib.zg_pipeline_status(1)
src = np.load(os.path.join(out, "src.npy"))
conv = zg.ResizeConversion(1920, 1080, "word").set_depth(10).set_filter("lanczos", 3) \
    .set_dst_width(3840).set_dst_height(2160).create()
d_src = torch.from_numpy(src.view(np.int16)).cuda()
d_dst = torch.zeros((2160, 3840), dtype=torch.int16, device="cuda")
res = {"engine": conv.info["engine"]}
conv.process(d_src, d_dst)  # warm: module loaded, plan uploaded
torch.cuda.synchronize()
res["status_before"] = int(lib.zg_pipeline_status(1))
assert lib.zg_debug_pipeline_fault(0, 1000000) == 0
t0 = time.time()
conv.process(d_src, d_dst)
torch.cuda.synchronize()
res["fault_seconds"] = time.time() - t0
res["status_fault"] = int(lib.zg_pipeline_status(1))
res["status_after_reset"] = int(lib.zg_pipeline_status(0))
assert lib.zg_debug_pipeline_fault(-1, 0) == 0
d_dst.zero_()
conv.process(d_src, d_dst)
torch.cuda.synchronize()
res["status_clean"] = int(lib.zg_pipeline_status(1))
np.save(os.path.join(out, "got.npy"), d_dst.cpu().numpy().view(np.uint16))
json.dump(res, open(os.path.join(out, "res.json"), "w"))
"""


def test_bounded_wait_runs_out(cuda, oracle, tmp_path):
    rng = np.random.default_rng(0x7B)
    src = rng.integers(0, 1024, size=(1080, 1920), dtype=np.uint16)
    np.save(tmp_path / "src.npy", src)
    env = dict(os.environ, ZG_CHAIN_TMA="1", ZG_ROOT=ROOT)
    child = subprocess.run([sys.executable, "-c", FAULT_CHILD, str(tmp_path)], env=env, capture_output=True,
                           text=True, timeout=600)
    assert child.returncode == 0, child.stderr[-3000:]
    res = json.load(open(tmp_path / "res.json"))
    assert res["engine"] == "tensor"
    assert res["status_before"] == 0
    # the consumer's wait for the dropped group (1) or the producer's wait for
    # that stage's release (2), whichever gave up first
    assert res["status_fault"] in (1, 2), res
    assert res["status_after_reset"] == 0
    assert res["fault_seconds"] < 5.0, res
    assert res["status_clean"] == 0
    want = oracle.resize_plane(src, 3840, 2160, "lanczos", 3, depth=10, mode="c", nthreads=16)
    np.testing.assert_array_equal(np.load(tmp_path / "got.npy"), want)
