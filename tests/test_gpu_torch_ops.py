"""torch.ops.dense2d: the PyTorch form against the C ABI's own paths on the same states."""
import importlib

import numpy as np
import pytest
import torch

import torch_step

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(dense):
    return importlib.import_module("2dense_gb300.torch_ops")


def setup(dense, ops, **kw):
    base = dict(ni=40, nj=32, benchmark=11, splitting=101, recon=255, cfl=0.5, var_eps=4.0)
    base.update(kw)
    c, cons, prim, x, y = dense.init_general(dense.config_default(**base))
    return c, cons, ops.padded_state(cons)


@pytest.mark.parametrize("split,recon", [(101, 255), (104, 0), (105, 0)])
def test_steps_op_equals_the_solver(dense, ops, split, recon):
    c, cons, u = setup(dense, ops, splitting=split, recon=recon)
    got = torch.ops.dense2d.steps(u, ops.config_tensor(c), 5, 0.0)
    with dense.Solver(c) as s:
        s.upload(cons)
        s.steps(5)
        ref = s.download(False)
    np.testing.assert_array_equal(got.cpu().numpy().transpose(2, 1, 0)[4:-4, 4:-4], ref[4:-4, 4:-4])


def test_three_stage_ops_make_one_step(dense, ops):
    c, cons, u = setup(dense, ops)
    ct = ops.config_tensor(c)
    u1, dt = torch.ops.dense2d.stage(u, u, ct, 1, 0.0, 0.0)
    u2, _ = torch.ops.dense2d.stage(u1, u, ct, 2, float(dt), 0.0)
    u3, _ = torch.ops.dense2d.stage(u2, u, ct, 3, float(dt), 0.0)
    one = torch.ops.dense2d.steps(u, ct, 1, 0.0)
    assert torch.equal(u3[:, 4:-4, 4:-4], one[:, 4:-4, 4:-4])


@pytest.mark.parametrize("recon", [251, 253, 255])
def test_rhs_op_matches_the_pytorch_step(dense, ops, recon):
    c, cons, u = setup(dense, ops, recon=recon)
    L = torch.ops.dense2d.rhs(u, ops.config_tensor(c))
    ref = torch_step.rhs(u[:, 4:-4, 4:-4].contiguous(), c.gamma, c.dx, c.dy, recon)
    assert float((L - ref).abs().max() / ref.abs().max()) < 1e-12


def test_batched_steps_op_equals_steps(dense, ops):
    sets = [setup(dense, ops, ni=n, nj=m, var_eps=e) for n, m, e in [(40, 32, 3.0), (24, 36, 4.5), (17, 29, 2.0)]]
    cts = [ops.config_tensor(c) for c, _, _ in sets]
    outs = torch.ops.dense2d.batched_steps([u for _, _, u in sets], cts, 4)
    for (c, cons, u), ct, out in zip(sets, cts, outs):
        ref = torch.ops.dense2d.steps(u, ct, 4, 0.0)
        assert torch.equal(out[:, 4:-4, 4:-4], ref[:, 4:-4, 4:-4])
