"""Shared fixtures. GPU tests are marked ``gpu``; everything else runs on CPU."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "resize_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build
    build()
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.oracle import Reference, reference_available
    if not reference_available():
        pytest.skip("zimg reference build (oracle/_ref) not present on this machine")
    return Reference()


@pytest.fixture(scope="session")
def golden():
    data = np.load(GOLDEN)
    meta = json.loads(bytes(data["meta"]).decode())
    return data, meta


@pytest.fixture(scope="session")
def lib():
    from zimg_gb300 import build as zbuild
    zbuild.build()
    import zimg_gb300
    return zimg_gb300.load()


@pytest.fixture(scope="session")
def cuda(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    torch.cuda.init()
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def pipeline_healthy(request):
    """After every GPU test: no bounded wait inside a pipelined kernel ran out."""
    yield
    if request.node.get_closest_marker("gpu") is None or "cuda" not in request.fixturenames:
        return
    import torch
    torch.cuda.synchronize()
    lib = request.getfixturevalue("lib")
    assert lib.zg_pipeline_status(1) == 0, "a pipelined kernel's bounded wait ran out"
