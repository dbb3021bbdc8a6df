"""Shared fixtures for the spherocyls_gb300 test suite.

Markers: ``gpu`` tests need a CUDA device and call libspherocyl through its C ABI;
everything else runs on the CPU (oracle pinning, host logic, ABI exports).
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REF_PI = 3.14159265358979  # the reference's pi (src/cpp/spherocyl_box.cpp:12)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


def periodic_diff(a, b, period):
    d = np.asarray(a) - np.asarray(b)
    return d - period * np.round(d / period)


@pytest.fixture(scope="session")
def oracle_built():
    import __graft_entry__
    import oracle

    __graft_entry__.ref_env()
    oracle.build(with_ref=None)
    return oracle


@pytest.fixture(scope="session")
def library():
    """libspherocyl, built in-tree (fails loudly when it cannot be built)."""
    import __graft_entry__

    __graft_entry__.build()
    from spherocyls_gb300 import _lib

    return _lib.lib()


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
