"""The C++ adapter include/zimg_gb300_filter.hpp: a resize pass with the
interface of zimg's graph filters (graphengine::Filter, as used by
ResizeImplH / ResizeImplV). Built against the graphengine stand-in header
the oracle uses; the GPU test drives it like a graph and checks the result
bit for bit against zimg's C path."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp")
INC = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle", "ref")]


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(nvcc))


def test_adapter_compiles():
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", *INC, "-I",
                        os.path.join(_cuda_home(), "include"), SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("horizontal,dst", [(1, 211), (0, 77)])
def test_adapter_resizes_like_zimg(cuda, oracle, tmp_path, horizontal, dst):
    lib_dir = os.path.join(ROOT, "zimg_gb300", "_lib")
    exe = str(tmp_path / "adapter_main")
    cuda_home = _cuda_home()
    r = subprocess.run(["g++", "-std=c++17", "-O1", *INC, "-I", os.path.join(cuda_home, "include"), SRC, "-o", exe,
                        "-L", lib_dir, "-lzimg_gb300", "-L", os.path.join(cuda_home, "lib64"), "-lcudart",
                        "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(8)
    h, w = 93, 130
    src = rng.integers(0, 1024, size=(h, w), dtype=np.uint16)
    src.tofile(tmp_path / "in.raw")
    r = subprocess.run([exe, str(tmp_path / "in.raw"), str(w), str(h), str(horizontal), str(dst), "10",
                        str(tmp_path / "out.raw")], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    ow, oh, step, rows, cols = map(int, r.stdout.split())
    assert (ow, oh) == ((dst, h) if horizontal else (w, dst))
    assert (step, rows, cols) == (oh, h, w)
    got = np.fromfile(tmp_path / "out.raw", dtype=np.uint16).reshape(oh, ow)
    want = oracle.resize_pass(src, bool(horizontal), dst, "spline36", depth=10)
    np.testing.assert_array_equal(got, want)
