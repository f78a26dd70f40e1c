"""The checkpoint format (gfortran unformatted sequential records of write_date_binary) and the
grid coordinates, on the CPU."""
import struct

import numpy as np
import pytest

from conftest import interior


def record(payload: bytes) -> bytes:
    return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))


def fortran_checkpoint(step, t, ni, nj, cons, x, y, dx, dy) -> bytes:
    return b"".join([
        record(struct.pack("<id", step, t)), record(struct.pack("<i", 1)), record(struct.pack("<i", 1)),
        record(struct.pack("<ii", ni, nj)), record(struct.pack("<ii", 4, 4)),
        record(np.asfortranarray(cons).tobytes(order="F")), record(np.asfortranarray(x).tobytes(order="F")),
        record(np.asfortranarray(y).tobytes(order="F")), record(struct.pack("<dd", dx, dy))])


def test_read_binary_of_a_fortran_checkpoint(dense, tmp_path):
    rng = np.random.default_rng(3)
    ni, nj = 7, 5
    cons = rng.standard_normal((ni + 8, nj + 8, 4))
    x, y = rng.standard_normal((ni, nj)), rng.standard_normal((ni, nj))
    p = tmp_path / "2d_42.dat2d"
    p.write_bytes(fortran_checkpoint(42, 0.125, ni, nj, cons, x, y, 0.5, 0.25))
    c, c2, x2, y2, step, t = dense.read_binary(str(p))
    assert (c.ni, c.nj, c.dx, c.dy, step, t) == (ni, nj, 0.5, 0.25, 42, 0.125)
    np.testing.assert_array_equal(c2, cons)
    np.testing.assert_array_equal(x2, x)
    np.testing.assert_array_equal(y2, y)


def test_read_binary_rejects_bad_files(dense, tmp_path):
    p = tmp_path / "bad.dat2d"
    p.write_bytes(b"\x04\x00\x00\x00abcd\x05\x00\x00\x00")
    with pytest.raises(dense.DenseError) as e:
        dense.read_binary(str(p))
    assert e.value.code == 7
    with pytest.raises(dense.DenseError):
        dense.read_binary(str(tmp_path / "missing.dat2d"))


@pytest.mark.parametrize("bench", [1, 2, 3, 4, 5, 6, 9, 11, 13, 14])
def test_grid_coords_match_the_setups(dense, bench):
    import ctypes
    c, cons, prim, x, y = dense.init_general(dense.config_default(ni=12, nj=10, benchmark=bench))
    lib = dense.load_library()
    dp = ctypes.POINTER(ctypes.c_double)
    gx, gy = np.zeros((12, 10), order="F"), np.zeros((12, 10), order="F")
    vx, vy = np.zeros((13, 11), order="F"), np.zeros((13, 11), order="F")
    assert lib.dense_grid_coords(ctypes.byref(c), *(a.ctypes.data_as(dp) for a in (gx, gy, vx, vy))) == 0
    np.testing.assert_array_equal(gx, x)
    np.testing.assert_array_equal(gy, y)
    off = 1.5 if bench in (3, 13) else 1.0
    shift = 20.0 if bench == 6 else 0.0
    np.testing.assert_array_equal(vx[:, 0], (np.arange(1, 14) - off) * c.dx)
    np.testing.assert_array_equal(vy[0, :], (np.arange(1, 12) - off) * c.dy - shift)
