"""PyTorch form: ``torch.ops.dense2d.{rhs, stage, steps, batched_steps}`` on CUDA float64 tensors.

A state is a tensor of shape (4, nj+8, ni+8) in the memory order of the reference's
``cons(NIp, NJp, 4)`` (i fastest, four ghost layers): the device twin of the host arrays of
``dense_upload``. A configuration travels as a uint8 CPU tensor holding the bytes of a
``dense_config_t`` (``config_tensor``), so every op has a plain tensor schema; one solver handle
(or batch) per distinct configuration is created on first use and kept.

    import importlib, torch
    ops = importlib.import_module("2dense_gb300.torch_ops")
    c = ops.config_tensor(cfg)
    u = torch.ops.dense2d.steps(u0, c, 100, 0.0)          # 100 steps
    L = torch.ops.dense2d.rhs(u, c)                        # (4, nj, ni) right-hand side
    u1, dt = torch.ops.dense2d.stage(u, u, c, 1, 0.0, 0.0) # stage 1 and its CFL time step

All work runs on the library's kernels on the handle's stream, ordered after the work already
queued on PyTorch's current stream and before whatever comes next there; nothing synchronises
the host. The ops do not record autograd history (``2dense_gb300.adjoint.AdjointStep`` is the
differentiable form).
"""
from __future__ import annotations

import ctypes

import torch

from . import _abi
from ._abi import DenseConfig, DenseError
from .solver import BatchSolver, Solver, init_general

_solvers: dict[bytes, Solver] = {}
_batches: dict[bytes, BatchSolver] = {}


def config_tensor(cfg: DenseConfig) -> torch.Tensor:
    """The bytes of a dense_config_t as a uint8 CPU tensor (the ops' configuration argument)."""
    raw = ctypes.string_at(ctypes.byref(cfg), ctypes.sizeof(DenseConfig))
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).clone()


def _config(t: torch.Tensor) -> DenseConfig:
    raw = bytes(t.cpu().contiguous().numpy().tobytes())
    if len(raw) != ctypes.sizeof(DenseConfig):
        raise ValueError("not a dense_config_t tensor (use config_tensor)")
    return DenseConfig.from_buffer_copy(raw)


def _solver(cfg_t: torch.Tensor) -> Solver:
    key = bytes(cfg_t.cpu().numpy().tobytes())
    s = _solvers.get(key)
    if s is None:
        # the setup's grid rows (x, y) feed the double Mach reflection and shear-layer boundary
        # rules; the setup's state itself is replaced by every op's input
        c, cons, prim, x, y = init_general(_config(cfg_t))
        s = Solver(c)
        s.upload(cons, prim, x, y)
        _solvers[key] = s
    return s


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _state(t: torch.Tensor, cfg: DenseConfig) -> torch.Tensor:
    shape = (4, cfg.nj + 8, cfg.ni + 8)
    if not (t.is_cuda and t.dtype == torch.float64 and tuple(t.shape) == shape):
        raise ValueError(f"expected a CUDA float64 state of shape {shape}")
    return t.contiguous()


def _chk(lib, rc, h, batch=False):
    if rc:
        msg = (lib.dense_batch_last_error if batch else lib.dense_last_error)(h)
        raise DenseError(rc, msg.decode() if msg else "")


@torch.library.custom_op("dense2d::steps", mutates_args=())
def steps(cons: torch.Tensor, cfg: torch.Tensor, nsteps: int, t0: float) -> torch.Tensor:
    """nsteps time steps of the state from time t0 (dense_steps); the new state."""
    s = _solver(cfg)
    lib, st = s.lib, _stream()
    cons = _state(cons, s.cfg)
    out = torch.empty_like(cons)
    _chk(lib, lib.dense_upload_device(s.h, _ptr(cons), None, st), s.h)
    _chk(lib, lib.dense_set_time(s.h, float(t0), 0), s.h)
    _chk(lib, lib.dense_steps_device(s.h, int(nsteps), float("inf"), 2**31 - 1, st), s.h)
    _chk(lib, lib.dense_download_device(s.h, _ptr(out), None, st), s.h)
    return out


@steps.register_fake
def _(cons, cfg, nsteps, t0):
    return torch.empty_like(cons)


@torch.library.custom_op("dense2d::rhs", mutates_args=())
def rhs(cons: torch.Tensor, cfg: torch.Tensor) -> torch.Tensor:
    """L(u) = -(dh_xi/dx + dh_eta/dy) of the state after its boundary fill: shape (4, nj, ni)."""
    s = _solver(cfg)
    lib, st = s.lib, _stream()
    cons = _state(cons, s.cfg)
    out = torch.empty((4, s.cfg.nj, s.cfg.ni), dtype=torch.float64, device=cons.device)
    _chk(lib, lib.dense_upload_device(s.h, _ptr(cons), None, st), s.h)
    _chk(lib, lib.dense_rhs_device(s.h, 1, _ptr(out), st), s.h)
    return out


@rhs.register_fake
def _(cons, cfg):
    return cons.new_empty((4, cons.shape[1] - 8, cons.shape[2] - 8))


@torch.library.custom_op("dense2d::stage", mutates_args=())
def stage(cons: torch.Tensor, cons0: torch.Tensor, cfg: torch.Tensor, irk: int, dt: float,
          t: float) -> tuple[torch.Tensor, torch.Tensor]:
    """One stage irk (1..3) of time_rk3_general on the stage input `cons`, `cons0` the step's
    initial state; returns (the stage's output, dt as a 0-d CUDA tensor: the CFL time step for
    stage 1, else the given dt)."""
    s = _solver(cfg)
    lib, st = s.lib, _stream()
    cons = _state(cons, s.cfg)
    cons0 = _state(cons0, s.cfg)
    out = torch.empty_like(cons)
    dtt = torch.full((), float(dt), dtype=torch.float64, device=cons.device)
    _chk(lib, lib.dense_upload_device(s.h, _ptr(cons), None, st), s.h)
    _chk(lib, lib.dense_stage_device(s.h, int(irk), _ptr(cons0) if irk > 1 else None, _ptr(dtt),
                                     float(t), st), s.h)
    _chk(lib, lib.dense_download_device(s.h, _ptr(out), None, st), s.h)
    return out, dtt


@stage.register_fake
def _(cons, cons0, cfg, irk, dt, t):
    return torch.empty_like(cons), cons.new_empty(())


@torch.library.custom_op("dense2d::batched_steps", mutates_args=())
def batched_steps(states: list[torch.Tensor], cfgs: list[torch.Tensor], nsteps: int) -> list[torch.Tensor]:
    """nsteps steps of every instance (the batched form: one launch per phase for all of them,
    each with its own configuration and CFL time step); the new states. Instances start at
    time 0; the batch handle is kept per list of configurations."""
    key = b"".join(bytes(c.cpu().numpy().tobytes()) for c in cfgs)
    b = _batches.get(key)
    if b is None:
        setups = [init_general(_config(c)) for c in cfgs]
        b = BatchSolver([st[0] for st in setups])
        for i, (c, cons, prim, x, y) in enumerate(setups):
            b.upload(i, cons, prim, x, y)
        _batches[key] = b
    lib, st = b.lib, _stream()
    outs = []
    states = [_state(x, c) for x, c in zip(states, b.cfgs)]
    for i, x in enumerate(states):
        _chk(lib, lib.dense_batch_upload_device(b.h, i, _ptr(x), None, st), b.h, True)
        b.set_time(i, 0.0, 0)
    _chk(lib, lib.dense_batch_steps_device(b.h, int(nsteps), float("inf"), 2**31 - 1, st), b.h, True)
    for i, x in enumerate(states):
        out = torch.empty_like(x)
        _chk(lib, lib.dense_batch_download_device(b.h, i, _ptr(out), None, st), b.h, True)
        outs.append(out)
    return outs


@batched_steps.register_fake
def _(states, cfgs, nsteps):
    return [torch.empty_like(x) for x in states]


def padded_state(cons_fortran) -> torch.Tensor:
    """A host cons(NIp, NJp, 4) array (Fortran order) as a (4, NJp, NIp) CUDA tensor."""
    import numpy as np
    a = np.asarray(cons_fortran)
    return torch.from_numpy(np.ascontiguousarray(a.transpose(2, 1, 0))).cuda()
