"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (oracle, host logic, C-ABI symbol checks)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def reference_root():
    """Root of a checkout of the reference tree, from MPCMD_REFERENCE_ROOT
    (None when unset or missing: tests that read the reference decks skip)."""
    r = os.environ.get("MPCMD_REFERENCE_ROOT")
    return r if r and os.path.isdir(r) else None


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def hilbert_order():
    d = np.load(os.path.join(GOLDEN, "hilbert_64x64x32.npz"))
    return d["order"], tuple(int(v) for v in d["box"]), bytes(d["sha256"])
