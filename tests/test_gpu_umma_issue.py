"""The issue model that decides which form the FP32 wide passes use: a
tcgen05.mma.kind::tf32 of M = 128, K = 8 costs about the same number of
cycles whatever its N (16 .. 256), so a banded product with ~10 useful
outputs per 8-input step uses a small fraction of the 5th-generation tensor
core, where the mma.sync form keeps its operands in registers. The probe
(tests/probes/umma_issue_probe.cu) is built with nvcc and run once; the test
prints its table and checks the finding with a loose bound."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_umma_cost_independent_of_n(cuda, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "umma_issue_probe"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", str(exe),
                    os.path.join(HERE, "probes", "umma_issue_probe.cu")], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    print(out)
    rows = {}
    for line in out.splitlines():
        m = re.match(r"N=\s*(\d+) acc=(\d+) (ts|ss): issue ([\d.]+) cyc/mma, complete ([\d.]+) cyc/mma", line)
        assert m and "err=0" in line and "no error" in line, line
        rows[(int(m[1]), int(m[2]), m[3])] = float(m[5])
    # 16x more work per instruction for less than 2x the cycles
    assert rows[(256, 1, "ts")] < 2 * rows[(16, 1, "ts")], rows
