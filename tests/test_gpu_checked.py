"""The checked variant (dense_config_t.strict = 2): the fast kernels with every index into a
state, face, tape or shared-memory array checked against its array, a bad one reported as
DENSE_FLAG_BOUNDS (and clamped, never dereferenced). Over every scheme and benchmark, both tile
shapes of the component-wise sweeps, every tile variant of the batched form and the adjoint's
taping sweeps it must report no index outside its array and agree with the fast variant to
rounding (relative L-inf <= 1e-13 per conserved field after up to three steps) and with the
oracle to the fast variant's 1e-12. The checks change no arithmetic, but their branches split
the kernels' basic blocks, and the compiler contracts a multiply and an add into an FMA only
within one block, so a few roundings differ from the fast build (upwind5 and AdaWENO come out
bit-identical)."""
import ctypes
import importlib

import pytest
import torch

from conftest import interior, rel_linf
from test_gpu_batch import SIZES, batch_cfgs
from test_gpu_parity import BENCHMARKS, SCHEMES_PERIODIC, make_cfg

pytestmark = pytest.mark.gpu

FLAG_BOUNDS = 0x40
TOL_FAST = 1e-13     # checked against fast: rounding of a few FMA contractions
TOL_ORACLE = 1e-12   # the fast variant's one-step tolerance against the oracle

CASES = ([(b, s, r, 40, 32) for b, s, r in SCHEMES_PERIODIC] + BENCHMARKS + [
    (11, 101, 253, 512, 512),   # component-wise sweeps on their full-height tiles
    (11, 103, 255, 512, 512),
    (5, 105, 0, 480, 120),      # AdaWENO with many characteristic items per block
    (13, 104, 0, 64, 256),
])


def run(dense, cfg, nsteps):
    c, cons, prim, x, y = dense.init_general(cfg)
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        s.steps(nsteps)
        g_cons, g_prim = s.download()
        return g_cons, g_prim, s.status()


@pytest.mark.parametrize("bench,split,recon,ni,nj", CASES)
def test_checked_matches_fast_with_every_index_in_range(dense, bench, split, recon, ni, nj):
    nsteps = 1 if ni * nj > 100_000 else 3
    f_cons, _, f_flags = run(dense, make_cfg(dense, bench, split, recon, ni, nj, strict=0), nsteps)
    c_cons, _, c_flags = run(dense, make_cfg(dense, bench, split, recon, ni, nj, strict=2), nsteps)
    assert not c_flags & FLAG_BOUNDS
    assert c_flags == f_flags
    assert rel_linf(interior(c_cons), interior(f_cons)) <= TOL_FAST


@pytest.mark.parametrize("bench,split,recon,ni,nj", [(11, 101, 253, 48, 40), (5, 105, 0, 96, 24),
                                                     (3, 104, 0, 32, 96), (6, 103, 253, 80, 24)])
def test_checked_one_step_against_the_oracle(dense, orc, bench, split, recon, ni, nj):
    cfg = make_cfg(dense, bench, split, recon, ni, nj, strict=2)
    c_cons, _, flags = run(dense, cfg, 1)
    assert not flags & FLAG_BOUNDS
    o = orc.OracleSolver(make_cfg(dense, bench, split, recon, ni, nj, strict=0))
    o.steps(1)
    assert rel_linf(interior(c_cons), interior(o.get_state()[0])) <= TOL_ORACLE


@pytest.mark.parametrize("split,recon", [(101, 255), (103, 251), (104, 0), (105, 0)])
def test_checked_batch_every_tile_variant(dense, split, recon):
    ref = None
    with dense.BatchSolver.from_setups(batch_cfgs(dense, split, recon, SIZES, strict=0)) as b:
        b.steps(2)
        ref = [b.download(i) for i in range(len(SIZES))]
    for sched in [(0, 0, 0), (1, 1, 1), (2, 2, 2), (3, 3, 0), (0, 4, 1)]:
        with dense.BatchSolver.from_setups(batch_cfgs(dense, split, recon, SIZES, strict=2)) as b:
            b.set_schedule(*sched)
            b.steps(2)
            assert not b.status() & FLAG_BOUNDS, f"schedule {sched}"
            for i in range(len(SIZES)):
                assert rel_linf(interior(b.download(i)), interior(ref[i])) <= TOL_FAST, \
                    f"schedule {sched} instance {i}"


@pytest.mark.parametrize("recon", [251, 253, 255])
def test_checked_adjoint_taping_sweeps(dense, recon):
    adjoint = importlib.import_module("2dense_gb300.adjoint")
    grads = []
    for strict in (0, 2):
        cfg = dense.config_default(ni=40, nj=32, benchmark=11, splitting=101, recon=recon, cfl=0.4,
                                   strict=strict, var_eps=4.0)
        c = dense.init_general(cfg)[0]
        with adjoint.Adjoint(c, checkpoint_every=3) as adj:
            u0 = adjoint.vortex_state(c, 4.0, 5.0, 5.0)
            uT = adj.forward(u0, 7)
            grads.append(adj.backward(uT))
            hs = ctypes.c_void_p()
            assert adj.lib.dense_adjoint_get_solver(adj.h, ctypes.byref(hs)) == 0
            flags = ctypes.c_uint()
            assert adj.lib.dense_status(hs, ctypes.byref(flags)) == 0
            assert not flags.value & FLAG_BOUNDS
    assert float((grads[1] - grads[0]).abs().max() / grads[0].abs().max()) <= 1e-11


def test_strict_must_be_a_known_variant(dense):
    cfg = make_cfg(dense, 11, 101, 253, 16, 16, strict=3)
    c = dense.init_general(cfg)[0]
    with pytest.raises(dense.DenseError):
        dense.Solver(c)
