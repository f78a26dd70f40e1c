"""Shared fixtures. The package directory starts with a digit, so it is imported by name."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def dense():
    mod = importlib.import_module("2dense_gb300")
    importlib.import_module("2dense_gb300.build").build()
    return mod


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle


def interior(a):
    """Interior cells of a padded Fortran-layout array (ghost width 4)."""
    return a[4:-4, 4:-4, ...]


def rel_linf(a, b):
    """Per-variable max |a-b| / max |b| over the last axis (variables)."""
    out = []
    for v in range(a.shape[-1]):
        den = max(np.abs(b[..., v]).max(), 1e-300)
        out.append(np.abs(a[..., v] - b[..., v]).max() / den)
    return max(out)
