"""Differentiable form: the discrete adjoint of n time steps behind ``torch.autograd.Function``.

``Adjoint`` owns a forward solver and the adjoint kernels of ``csrc/adjoint.cu`` (LLF, GLF or
Steger-Warming splitting with upwind5 / WENO-JS5 / WENO-Z5, the characteristic WENO-Z scheme
104 or AdaWENO 105, on x- and y-periodic grids or the
reference's benchmarks with extrapolated, mirror and fixed-state sides (1, 2, 3, 4, 5, 9, 13;
the Rayleigh-Taylor ones with their body force) or the shear layer's time-dependent inflow (6),
TVD-RK3, CFL or constant dt).
States are CUDA float64 tensors of the interior, shape (4, nj, ni): conserved variables
(rho, rho u, rho v, E) with i fastest -- the reference's cons(i, j, v) without ghost layers.

    adj = Adjoint(cfg, checkpoint_every=20)
    uT = AdjointStep.apply(u0, adj, 400)      # forward: plain solver, checkpoints every 20 steps
    loss = 0.5 * ((uT[0] - rho_target) ** 2).sum()
    loss.backward()                            # reverse: recompute each segment, adjoint kernels

The gradient is the exact derivative of the discrete scheme, including the time step's
dependence on the state through the CFL condition. Every call goes to the CUDA library.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _abi
from ._abi import DenseConfig, DenseError


def _torch():
    import torch
    return torch


class Adjoint:
    """Forward solver plus adjoint kernels for one grid and scheme (see module docstring)."""

    def __init__(self, cfg: DenseConfig, checkpoint_every: int = 20):
        self.lib = _abi.load_library()
        self.cfg = cfg.copy()
        self.k = int(checkpoint_every)
        h = ctypes.c_void_p()
        rc = self.lib.dense_adjoint_create(ctypes.byref(self.cfg), self.k, ctypes.byref(h))
        if rc:
            raise DenseError(rc, self.lib.dense_adjoint_last_error(None).decode())
        self.h = h
        self.shape = (4, cfg.nj, cfg.ni)
        self.generation = 0  # forwards run so far; backward needs its own forward to be the last
        self.nsteps = -1

    def _chk(self, rc):
        if rc:
            raise DenseError(rc, self.lib.dense_adjoint_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.dense_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _arg(self, t):
        torch = _torch()
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64
                and tuple(t.shape) == self.shape and t.is_contiguous()):
            raise ValueError(f"expected a contiguous CUDA float64 tensor of shape {self.shape}")
        return ctypes.c_void_p(t.data_ptr())

    @staticmethod
    def _stream():
        return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)

    def forward(self, u0, nsteps: int):
        """State after nsteps steps from u0; keeps the checkpoints for ``backward``."""
        torch = _torch()
        u0 = u0.detach().contiguous()
        uT = torch.empty_like(u0)
        self._chk(self.lib.dense_adjoint_forward(self.h, self._arg(u0), int(nsteps), self._arg(uT),
                                                 self._stream()))
        self.generation += 1
        self.nsteps = int(nsteps)
        return uT

    def backward(self, gT):
        """(d uT / d u0)^T gT for the last forward."""
        torch = _torch()
        gT = gT.detach().contiguous()
        g0 = torch.empty_like(gT)
        self._chk(self.lib.dense_adjoint_backward(self.h, self._arg(gT), self._arg(g0), self._stream()))
        return g0

    def rhs_vjp(self, u, v):
        """((dL/du)^T v, v . L(u)) for the right-hand side L of one stage."""
        torch = _torch()
        u, v = u.detach().contiguous(), v.detach().contiguous()
        out = torch.empty_like(u)
        vl = ctypes.c_double()
        self._chk(self.lib.dense_adjoint_rhs_vjp(self.h, self._arg(u), self._arg(v), self._arg(out),
                                                 ctypes.byref(vl), self._stream()))
        return out, vl.value

    def dts(self) -> np.ndarray:
        """Time steps of the last forward."""
        out = np.zeros(max(self.nsteps, 0))
        if self.nsteps > 0:
            self._chk(self.lib.dense_adjoint_get_dts(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                     self.nsteps))
        return out

    def argmax(self) -> np.ndarray:
        """After ``backward``: per step, the cells (j*ni+i) of max(|u|+alpha) and max(|v|+alpha)."""
        out = np.zeros((max(self.nsteps, 0), 2), dtype=np.int32)
        if self.nsteps > 0:
            self._chk(self.lib.dense_adjoint_get_argmax(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                        self.nsteps))
        return out

    def launch_count(self) -> int:
        return int(self.lib.dense_adjoint_launch_count(self.h))

    def solver_state(self):
        """The forward solver's current conserved variables, padded Fortran layout (ni+8, nj+8, 4),
        and its interface fluxes (h_xi, h_eta) of the last stage it ran."""
        hs = ctypes.c_void_p()
        self._chk(self.lib.dense_adjoint_get_solver(self.h, ctypes.byref(hs)))
        c = self.cfg
        dp = ctypes.POINTER(ctypes.c_double)
        cons = np.zeros((c.ni + 8, c.nj + 8, 4), order="F")
        hx = np.zeros((c.ni + 1, c.nj, 4), order="F")
        he = np.zeros((c.nj + 1, c.ni, 4), order="F")
        for rc in (self.lib.dense_download(hs, cons.ctypes.data_as(dp), None),
                   self.lib.dense_get_fluxes(hs, hx.ctypes.data_as(dp), he.ctypes.data_as(dp))):
            if rc:
                raise DenseError(rc, self.lib.dense_last_error(hs).decode())
        return cons, hx, he


def _make_function():
    torch = _torch()

    class AdjointStep(torch.autograd.Function):
        """uT = nsteps time steps from u0; backward runs the discrete adjoint with checkpointing."""

        @staticmethod
        def forward(ctx, u0, adj: Adjoint, nsteps: int):
            uT = adj.forward(u0, nsteps)
            ctx.adj, ctx.nsteps, ctx.generation = adj, nsteps, adj.generation
            ctx.save_for_backward(u0.detach().clone())
            return uT

        @staticmethod
        def backward(ctx, gT):
            adj = ctx.adj
            if adj.generation != ctx.generation:  # another forward ran since: restore this one
                (u0,) = ctx.saved_tensors
                adj.forward(u0, ctx.nsteps)
                ctx.generation = adj.generation
            return adj.backward(gT), None, None

    return AdjointStep


_AdjointStep = None


def __getattr__(name):  # the Function class is built on first use, so importing needs no torch
    global _AdjointStep
    if name == "AdjointStep":
        if _AdjointStep is None:
            _AdjointStep = _make_function()
        return _AdjointStep
    raise AttributeError(name)


def vortex_state(cfg: DenseConfig, eps, xc, yc, drho=None, device="cuda"):
    """Initial state of the translating vortex (benchmark 11) as a differentiable function of its
    strength eps, centre (xc, yc) and an optional density perturbation drho (nj, ni) added at
    fixed velocity and pressure. Same formulas as dense_init_setup for benchmark 11: cell
    centres ((i-1/2) dx, (j-1/2) dy) on [0,10]^2 over the stream (rho, u, v, p) = (1, 1, 1, 1)."""
    torch = _torch()
    g = cfg.gamma
    ni, nj = cfg.ni, cfg.nj
    dx, dy = 10.0 / ni, 10.0 / nj
    x = (torch.arange(ni, dtype=torch.float64, device=device) + 0.5) * dx
    y = (torch.arange(nj, dtype=torch.float64, device=device) + 0.5) * dy
    Y, X = torch.meshgrid(y, x, indexing="ij")
    as_t = lambda s: s if isinstance(s, torch.Tensor) else torch.tensor(float(s), dtype=torch.float64, device=device)
    eps, xc, yc = as_t(eps), as_t(xc), as_t(yc)
    r2 = (X - xc) ** 2 + (Y - yc) ** 2
    rho = (1.0 - (g - 1.0) * eps ** 2 * torch.exp(1.0 - r2) / (8.0 * g * math.pi ** 2)) ** (1.0 / (g - 1.0))
    f = eps / (2.0 * math.pi) * torch.exp((1.0 - r2) / 2.0)
    u = 1.0 - f * (Y - yc)
    v = 1.0 + f * (X - xc)
    p = rho ** g
    if drho is not None:
        rho = rho + drho
    E = p / (g - 1.0) + 0.5 * rho * (u * u + v * v)
    return torch.stack([rho, rho * u, rho * v, E]).contiguous()
