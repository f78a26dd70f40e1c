"""dense_stage_noalloc: one stage on caller-owned device arrays, with the library's scratch in a
fixed file-scope device array instead of handle buffers. It serves callers that cannot let the
library allocate device memory (their own pool or budget owns every byte). Checked through the
C ABI against the handle path (dense_stage) on two consecutive stages; the caller's arrays are
allocated here by PyTorch, standing in for such a caller's own allocator.

Collected last on purpose: if it fails, a run that stops at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

from conftest import interior, rel_linf

pytestmark = pytest.mark.gpu

CASES = [
    (5, 105, 0, 96, 24),    # double Mach reflection (reads the cell-centre rows), AdaWENO
    (11, 101, 253, 40, 36),  # periodic vortex, LLF + WENO-JS5
]


def to_device(torch, a, nvar, pitch):
    """Fortran (NIp, NJp, nv) host array -> device [nvar][NJp][pitch] doubles."""
    nip, njp = a.shape[0], a.shape[1]
    d = np.zeros((nvar, njp, pitch))
    d[:, :, :nip] = np.transpose(a[:, :, :nvar], (2, 1, 0))
    return torch.from_numpy(d).cuda()


def from_device(t, nip):
    return np.asfortranarray(np.transpose(t.cpu().numpy()[:, :, :nip], (2, 1, 0)))


@pytest.mark.parametrize("bench,split,recon,ni,nj", CASES)
def test_noalloc_stage_matches_handle_stage(dense, bench, split, recon, ni, nj):
    torch = pytest.importorskip("torch")
    lib = dense.load_library()
    cfg = dense.config_default(ni=ni, nj=nj, benchmark=bench, splitting=split, recon=recon, cfl=0.5)
    c, cons, prim, x, y = dense.init_general(cfg)
    nip, njp = ni + 8, nj + 8
    pitch = (nip + 1) & ~1
    vp = ctypes.c_void_p

    cons_d = to_device(torch, cons, 4, pitch)
    prim_d = to_device(torch, prim, 5, pitch)
    cons0_d = torch.zeros_like(cons_d)
    xbot = torch.from_numpy(np.ascontiguousarray(x[:, 0])).cuda()
    xtop = torch.from_numpy(np.ascontiguousarray(x[:, nj - 1])).cuda()
    yleft = torch.from_numpy(np.ascontiguousarray(y[0, :])).cuda()
    stream = torch.cuda.current_stream().cuda_stream

    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        dt = ctypes.c_double(c.dt)
        for irk in (1, 2):  # two calls in a row share the fixed scratch
            rc = lib.dense_stage_noalloc(ctypes.byref(c), irk, 0.0, vp(cons_d.data_ptr()),
                                         vp(prim_d.data_ptr()), vp(cons0_d.data_ptr()),
                                         vp(xbot.data_ptr()), vp(xtop.data_ptr()),
                                         vp(yleft.data_ptr()), ctypes.byref(dt), vp(stream))
            assert rc == 0
            dt_ref = s.stage(irk)
            ref_cons, ref_prim = s.download()
            got_cons = from_device(cons_d, nip)
            got_prim = from_device(prim_d, nip)
            assert dt.value == pytest.approx(dt_ref, rel=1e-12)
            assert rel_linf(interior(got_cons), interior(ref_cons)) <= 1e-12
            np.testing.assert_allclose(interior(got_prim), interior(ref_prim)[..., :5], rtol=1e-12, atol=1e-14)


def _stage(lib, c, irk, cons_d, prim_d, cons0_d, xbot, xtop, yleft, dt, stream):
    vp = ctypes.c_void_p
    return lib.dense_stage_noalloc(ctypes.byref(c), irk, 0.0, vp(cons_d.data_ptr()),
                                   vp(prim_d.data_ptr()), vp(cons0_d.data_ptr()),
                                   vp(xbot.data_ptr()), vp(xtop.data_ptr()), vp(yleft.data_ptr()),
                                   ctypes.byref(dt), vp(stream))


def test_noalloc_reports_a_nan_in_the_state(dense):
    """The device status word is read back after the stage: a NaN planted in the caller's state
    returns DENSE_ERR_NUMERIC with the flag in the error text, and the next clean call succeeds
    (the word is cleared at every call)."""
    torch = pytest.importorskip("torch")
    lib = dense.load_library()
    ni, nj = 40, 36
    cfg = dense.config_default(ni=ni, nj=nj, benchmark=11, splitting=101, recon=253, cfl=0.5)
    c, cons, prim, x, y = dense.init_general(cfg)
    pitch = (ni + 9) & ~1
    bad = cons.copy()
    bad[20, 18, 0] = np.nan
    xbot = torch.from_numpy(np.ascontiguousarray(x[:, 0])).cuda()
    xtop = torch.from_numpy(np.ascontiguousarray(x[:, nj - 1])).cuda()
    yleft = torch.from_numpy(np.ascontiguousarray(y[0, :])).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for state, expect in ((bad, 5), (cons, 0)):  # DENSE_ERR_NUMERIC, then DENSE_OK
        cons_d = to_device(torch, state, 4, pitch)
        prim_d = to_device(torch, prim, 5, pitch)
        cons0_d = torch.zeros_like(cons_d)
        dt = ctypes.c_double(c.dt)
        rc = _stage(lib, c, 1, cons_d, prim_d, cons0_d, xbot, xtop, yleft, dt, stream)
        assert rc == expect
        if expect:
            assert b"0x01" in lib.dense_last_error(None)


def test_noalloc_rejects_an_unknown_kernel_variant(dense):
    lib = dense.load_library()
    cfg = dense.config_default(ni=40, nj=36, benchmark=11, splitting=101, recon=253,
                               dx=0.25, dy=0.25, strict=3)
    dt = ctypes.c_double(0.0)
    dummy = ctypes.c_void_p(16)  # rejected before any device access
    rc = lib.dense_stage_noalloc(ctypes.byref(cfg), 1, 0.0, dummy, dummy, dummy, None, None,
                                 None, ctypes.byref(dt), None)
    assert rc == 1  # DENSE_ERR_ARG
    assert b"strict" in lib.dense_last_error(None)


def test_noalloc_rejects_grids_beyond_the_scratch(dense):
    lib = dense.load_library()
    cfg = dense.config_default(ni=400, nj=400, benchmark=11, splitting=101, recon=253,
                               dx=0.025, dy=0.025)
    dt = ctypes.c_double(0.0)
    vp = ctypes.c_void_p
    # a non-null dummy pointer: the size check rejects the call before any device access
    dummy = vp(16)
    rc = lib.dense_stage_noalloc(ctypes.byref(cfg), 1, 0.0, dummy, dummy, dummy, None, None,
                                 None, ctypes.byref(dt), None)
    assert rc == 10  # DENSE_ERR_LIMIT
    assert b"fixed scratch" in lib.dense_last_error(None)
