"""The fast kernels' reciprocal and inverse square root (hardware seed refined by two
Newton-Raphson steps) against CUDA's IEEE divide and square root."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulp_err(a, b):
    return np.abs(a - b) / np.spacing(np.abs(b))


def test_fast_reciprocal_and_rsqrt_within_two_ulp(dense):
    lib = dense.load_library()
    rng = np.random.default_rng(3)
    x = np.concatenate([
        10.0 ** rng.uniform(-280, 280, 200000),       # across the normal range
        rng.uniform(1e-6, 1e3, 200000),                # the range the kernels see
        np.array([1.0, 2.0, 0.5, 3.0, 1e-6, 1.0 + 2.0 ** -52]),
    ])
    out = np.zeros(4 * x.size)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lib.dense_fastmath_check(x.ctypes.data_as(dp), out.ctypes.data_as(dp), x.size)
    assert rc == 0
    out = out.reshape(-1, 4)
    assert ulp_err(out[:, 0], out[:, 1]).max() <= 2.0
    assert ulp_err(out[:, 2], out[:, 3]).max() <= 2.0
