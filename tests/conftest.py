import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def synthetic_shells(name="synthetic"):
    g = golden(name)
    return [dict(l=int(g["shell_l"][i]), centre=g["shell_centre"][i],
                 expo=g["shell_expo"][i, :g["shell_k"][i]],
                 coef=g["shell_coef"][i, :g["shell_k"][i]]) for i in range(len(g["shell_l"]))]


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gaussium_gb300 import build, _lib
    build.build()
    return _lib.lib()
