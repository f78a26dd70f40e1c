"""Failure detection without a GPU fault: corrupt states and bad indices made on the host must
come back as status flags and error codes, with the device context still usable; handles used
from several host threads at once give the same results as one after another."""
import threading

import numpy as np
import pytest

from conftest import interior

pytestmark = pytest.mark.gpu

FLAG_NAN, FLAG_NEG_RHO, FLAG_P_FLOOR, FLAG_RECON_NOOP = 0x01, 0x02, 0x04, 0x10


def vortex(dense, **kw):
    base = dict(ni=40, nj=32, benchmark=11, splitting=101, recon=255, cfl=0.5, var_eps=4.0)
    base.update(kw)
    return dense.init_general(dense.config_default(**base))


def test_nan_state_is_flagged_and_the_context_survives(dense):
    c, cons, prim, x, y = vortex(dense)
    bad = cons.copy()
    bad[10, 10, 0] = np.nan
    with dense.Solver(c) as s:
        s.upload(bad, None, x, y)
        s.steps(1)
        assert s.status() & FLAG_NAN
        assert s.status() == 0  # reading clears the word
    with dense.Solver(c) as s:  # the context is fine: a clean run still matches itself
        s.upload(cons, prim, x, y)
        s.steps(2)
        assert s.status() & (FLAG_NAN | FLAG_NEG_RHO) == 0


def test_negative_density_and_pressure_floor(dense):
    c, cons, prim, x, y = vortex(dense)
    neg = cons.copy()
    neg[12, 9, 0] = -1.0
    with dense.Solver(c) as s:
        s.upload(neg, None, x, y)
        assert s.status() & FLAG_NEG_RHO
    lowp = cons.copy()
    lowp[15, 15, 3] = 0.5 * (lowp[15, 15, 1] ** 2 + lowp[15, 15, 2] ** 2) / lowp[15, 15, 0] - 0.1
    with dense.Solver(c) as s:
        s.upload(lowp, None, x, y)
        assert s.status() & FLAG_P_FLOOR
        _, p = s.download()
        assert p[15, 15, 3] == np.float64(np.float32(1.0e-6))  # get_primary.f90:58


def test_unknown_reconstruction_is_a_flagged_noop(dense):
    c, cons, prim, x, y = vortex(dense, recon=201)  # the namelist default, not handled
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        s.steps(1)
        assert s.status() & FLAG_RECON_NOOP
        # h stays zero: the stage combines leave the state as it was, up to their own rounding
        np.testing.assert_allclose(interior(s.download(False)), interior(cons), rtol=4e-16, atol=0)


def test_bad_indices_are_error_codes(dense):
    c = vortex(dense)[0]
    for field, value, code in (("splitting", 107, 2), ("benchmark", 12, 3), ("ni", 2, 1)):
        bad = c.copy()
        setattr(bad, field, value)
        with pytest.raises(dense.DenseError) as e:
            dense.Solver(bad)
        assert e.value.code == code
    with dense.Solver(c) as s:
        with pytest.raises(dense.DenseError) as e:
            s.stage(4)
        assert e.value.code == 1
        with pytest.raises(dense.DenseError) as e:
            s.steps(1)  # no state uploaded yet
        assert e.value.code == 8


def test_one_bad_instance_leaves_the_batch_intact(dense):
    setups = [vortex(dense, ni=n, nj=n, var_eps=e) for n, e in ((32, 3.0), (24, 4.0), (40, 2.0))]
    with dense.BatchSolver([s[0] for s in setups]) as b:
        for i, (c, cons, prim, x, y) in enumerate(setups):
            bad = cons.copy()
            if i == 1:
                bad[8, 8, 0] = np.nan
            b.upload(i, bad, None, x, y)
        b.steps(2)
        assert b.status() & FLAG_NAN
        for i in (0, 2):
            c, cons, prim, x, y = setups[i]
            with dense.Solver(c) as s:
                s.upload(cons, None, x, y)
                s.steps(2)
                np.testing.assert_array_equal(interior(b.download(i)), interior(s.download(False)))


def test_handles_on_several_host_threads(dense):
    cases = [vortex(dense, ni=40 + 8 * k, nj=32, var_eps=2.0 + k) for k in range(4)]

    def run(case, out, k):
        c, cons, prim, x, y = case
        with dense.Solver(c) as s:
            s.upload(cons, prim, x, y)
            s.steps(20)
            out[k] = s.download(False)

    serial = {}
    for k, case in enumerate(cases):
        run(case, serial, k)
    par = {}
    threads = [threading.Thread(target=run, args=(case, par, k)) for k, case in enumerate(cases)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k in range(len(cases)):
        np.testing.assert_array_equal(par[k], serial[k])
