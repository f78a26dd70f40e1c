"""The batched form against plain solves: every instance of a batch -- uneven sizes, different
benchmarks, vortex strengths and interface amplitudes, each with its own CFL time step -- must
equal the single-instance solve of the same configuration bit for bit, for every launch
schedule the autotuner can pick."""
import importlib

import numpy as np
import pytest

from conftest import interior

pytestmark = pytest.mark.gpu


def batch_cfgs(dense, split, recon, sizes, seed=5, strict=0):
    rng = np.random.default_rng(seed)
    cfgs = []
    for k, (ni, nj) in enumerate(sizes):
        if k % 2 == 0:  # translating vortex, strength and centre drawn per instance
            cfgs.append(dense.config_default(ni=ni, nj=nj, benchmark=11, splitting=split, recon=recon,
                                             cfl=0.5, strict=strict, var_eps=rng.uniform(1, 5),
                                             var_xc=5 + rng.uniform(-1, 1), var_yc=5 + rng.uniform(-1, 1)))
        else:  # periodic Richtmyer-Meshkov, interface amplitude drawn per instance
            cfgs.append(dense.config_default(ni=ni, nj=nj, benchmark=14, splitting=split, recon=recon,
                                             cfl=0.5, strict=strict, var_amp=rng.uniform(0.01, 0.05)))
    return cfgs


SIZES = [(40, 40), (24, 36), (64, 64), (17, 29), (33, 33), (48, 20)]


def plain(dense, cfg, nsteps, t_end=float("inf")):
    c, cons, prim, x, y = dense.init_general(cfg)
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        s.steps(nsteps, t_end=t_end)
        return s.download(False), s.current_time, s.current_step, s.dt


@pytest.mark.parametrize("split,recon", [(101, 255), (101, 253), (103, 251), (104, 0), (105, 0)])
def test_batch_equals_plain_solves(dense, split, recon):
    cfgs = batch_cfgs(dense, split, recon, SIZES)
    with dense.BatchSolver.from_setups(cfgs) as b:
        b.steps(3)
        for i, cfg in enumerate(cfgs):
            ref, t, step, dt = plain(dense, cfg, 3)
            got = b.download(i)
            np.testing.assert_array_equal(interior(got), interior(ref), err_msg=f"instance {i}")
            bt, bs, bdt = b.time(i)
            assert (bt, bs, bdt) == (t, step, dt)


def test_every_schedule_gives_the_same_bits(dense):
    cfgs = batch_cfgs(dense, 101, 255, SIZES, seed=9)
    ref = None
    for sched in [(0, 0, 0), (1, 2, 1), (2, 1, 2), (1, 1, 0), (2, 2, 1), (3, 3, 0), (0, 4, 2), (3, 4, 1)]:
        with dense.BatchSolver.from_setups(cfgs) as b:
            b.set_schedule(*sched)
            b.steps(2)
            out = [b.download(i) for i in range(len(cfgs))]
        if ref is None:
            ref = out
        for i in range(len(cfgs)):
            np.testing.assert_array_equal(out[i], ref[i], err_msg=f"schedule {sched} instance {i}")


def test_per_instance_time_bounds(dense):
    """Each instance stops at its own step count: the loop bound is per instance, its dt its own."""
    cfgs = batch_cfgs(dense, 101, 255, SIZES[:4], seed=2)
    t_end = 0.05
    with dense.BatchSolver.from_setups(cfgs) as b:
        b.steps(500, t_end=t_end)
        for i, cfg in enumerate(cfgs):
            ref, t, step, dt = plain(dense, cfg, 500, t_end=t_end)
            np.testing.assert_array_equal(interior(b.download(i)), interior(ref))
            assert b.time(i)[:2] == (t, step)


def test_strict_batch_matches_oracle(dense, orc):
    cfgs = batch_cfgs(dense, 101, 255, SIZES[:3], seed=4, strict=1)
    with dense.BatchSolver.from_setups(cfgs) as b:
        b.steps(2)
        for i, cfg in enumerate(cfgs):
            o = orc.OracleSolver(cfg)
            o.steps(2)
            np.testing.assert_array_equal(interior(b.download(i)), interior(o.get_state()[0]))


def test_autotuner_picks_a_valid_schedule(dense, tmp_path, monkeypatch):
    monkeypatch.setenv("DENSE2D_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    at = importlib.reload(importlib.import_module("2dense_gb300.autotune"))
    cfgs = batch_cfgs(dense, 101, 255, SIZES, seed=1)
    best, info = at.tune(cfgs, steps=1, reps=1)
    assert len(best) == 4 and best[3] in (0, 1) and not info["cached"] and len(info["trials"]) >= 4
    assert any(k.endswith(",1") for k in info["trials"])  # the persistent step was timed
    best2, info2 = at.tune(cfgs)
    assert best2 == best and info2["cached"]


# ---- the persistent step (launch mode 1) --------------------------------------------------------

@pytest.mark.parametrize("split,recon", [(101, 255), (101, 253), (102, 255), (103, 251)])
def test_persistent_step_equals_plain_solves(dense, split, recon):
    cfgs = batch_cfgs(dense, split, recon, SIZES, seed=11)
    with dense.BatchSolver.from_setups(cfgs) as b:
        b.set_launch_mode(1)
        assert b.launch_mode() == 1
        n0 = b.launch_count()
        b.steps(3)
        assert not b.status()
        for i, cfg in enumerate(cfgs):
            ref, t, step, dt = plain(dense, cfg, 3)
            np.testing.assert_array_equal(interior(b.download(i)), interior(ref), err_msg=f"instance {i}")
            assert b.time(i) == (t, step, dt)
        # one kernel per step, plus the get_primary of the uploaded states (two launches) and
        # the loop bounds (one)
        assert b.launch_count() - n0 == 3 + 3


def test_persistent_step_every_schedule_gives_the_same_bits(dense):
    cfgs = batch_cfgs(dense, 101, 255, SIZES, seed=9)
    ref = None
    for sched in [(0, 0, 0, 0), (0, 0, 0, 1), (1, 2, 1, 1), (2, 1, 2, 1), (3, 3, 0, 1), (0, 4, 2, 1),
                  (3, 4, 1, 1), (2, 3, 1, 1)]:
        with dense.BatchSolver.from_setups(cfgs) as b:
            b.set_schedule(*sched)
            b.steps(2)
            out = [b.download(i) for i in range(len(cfgs))]
        if ref is None:
            ref = out
        for i in range(len(cfgs)):
            np.testing.assert_array_equal(out[i], ref[i], err_msg=f"schedule {sched} instance {i}")


def test_persistent_step_per_instance_time_bounds(dense):
    """Instances that reach their end time skip their pieces while the others go on."""
    cfgs = batch_cfgs(dense, 101, 255, SIZES[:4], seed=2)
    t_end = 0.05
    with dense.BatchSolver.from_setups(cfgs) as b:
        b.set_launch_mode(1)
        b.steps(500, t_end=t_end)
        for i, cfg in enumerate(cfgs):
            ref, t, step, dt = plain(dense, cfg, 500, t_end=t_end)
            np.testing.assert_array_equal(interior(b.download(i)), interior(ref))
            assert b.time(i)[:2] == (t, step)


def test_persistent_step_rejects_what_it_does_not_cover(dense):
    from importlib import import_module
    abi = import_module("2dense_gb300._abi")
    for split, recon, strict in [(105, 0, 0), (104, 0, 0), (101, 255, 1), (101, 255, 2)]:
        cfgs = batch_cfgs(dense, split, recon, SIZES[:2], strict=strict)
        with dense.BatchSolver.from_setups(cfgs) as b:
            with pytest.raises(dense.DenseError) as e:
                b.set_launch_mode(1)
            assert e.value.code == abi.DENSE_ERR_ARG
            assert b.launch_mode() == 0
            b.steps(1)  # the per-phase launches still run


def test_persistent_wait_gives_up_and_reports(dense):
    """A dependency that never completes (one piece more than the phase has): the waits give up
    after their poll limit, the step returns DENSE_ERR_TIMEOUT with DENSE_FLAG_TIMEOUT in the
    status, and the context stays usable."""
    from importlib import import_module
    abi = import_module("2dense_gb300._abi")
    cfgs = batch_cfgs(dense, 101, 255, SIZES, seed=3)
    with dense.BatchSolver.from_setups(cfgs) as b:
        b.set_launch_mode(1)
        b.hold_instance(2, 2000)
        with pytest.raises(dense.DenseError) as e:
            b.steps(1)
        assert e.value.code == abi.DENSE_ERR_TIMEOUT
        assert b.status() & abi.FLAG_TIMEOUT
        b.hold_instance(-1)
        for i, (c, cons, prim, x, y) in enumerate(dense.init_general(c) for c in cfgs):
            b.upload(i, cons, prim, x, y)
            b.set_time(i, 0.0, 0)
        b.steps(2)
        assert not b.status()
        for i, cfg in enumerate(cfgs):
            ref = plain(dense, cfg, 2)[0]
            np.testing.assert_array_equal(interior(b.download(i)), interior(ref), err_msg=f"instance {i}")
