import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")
    config.addinivalue_line("markers", "timeout(seconds): per-test time limit (pytest-timeout)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


_UT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}
_ST = {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}


def to_dev(a: np.ndarray):
    """Copy a numpy array of any 1/2/4/8-byte dtype to a CUDA tensor of the same bytes."""
    import torch
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(_ST[a.dtype.itemsize]).copy()).cuda()


def from_dev(t, dtype) -> np.ndarray:
    dt = np.dtype(dtype)
    return t.cpu().numpy().view(_ST[dt.itemsize]).view(dt)


def empty_dev(n: int, dtype):
    import torch
    dt = np.dtype(dtype)
    tdt = {1: torch.int8, 2: torch.int16, 4: torch.int32, 8: torch.int64}[dt.itemsize]
    return torch.empty(n, dtype=tdt, device="cuda")


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                                                 np.ascontiguousarray(b).view(np.uint8))
