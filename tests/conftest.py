import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled libcgx.so")


def float_eq(a, b):
    """gtest EXPECT_FLOAT_EQ: equal to within 4 single-precision ULPs."""
    import numpy as np
    a = np.float32(a)
    b = np.float32(b)
    if a == b:
        return True
    ia = np.array([a], np.float32).view(np.int32)[0]
    ib = np.array([b], np.float32).view(np.int32)[0]
    # map sign-magnitude to a monotone integer line
    ia = ia if ia >= 0 else np.int64(-2**31) - ia
    ib = ib if ib >= 0 else np.int64(-2**31) - ib
    return abs(int(ia) - int(ib)) <= 4


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o
