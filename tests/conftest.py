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
    """Relative L-inf error of each conserved field -- density, momentum (the vector
    (rho u, rho v)) and total energy: max over cells of |a-b| / max over cells of |b|.
    Returns the largest of the three. Momentum is measured as a vector so that a component
    that starts at zero (rho u in Rayleigh-Taylor) is not judged against its own tiny scale."""
    out = []
    for fields in ([0], [1, 2], [3]):
        da = np.sqrt(sum((a[..., v] - b[..., v]) ** 2 for v in fields))
        nb = np.sqrt(sum(b[..., v] ** 2 for v in fields))
        out.append(da.max() / max(nb.max(), 1e-300))
    return max(out)
