import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def cuda_available() -> bool:
    try:
        import ctypes

        lib = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import torch

            return torch.cuda.is_available()
        except Exception:
            return False
    n = ctypes.c_int(0)
    return lib.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


def pytest_collection_modifyitems(config, items):
    # a GPU test on a machine without a GPU is an error, not a skip, unless
    # the run deselected GPU tests with -m "not gpu"
    pass
