"""TEST INFRASTRUCTURE ONLY: ctypes front end of the CPU oracle (``dense_oracle.cpp``).

``OracleSolver`` holds one block of the reference solver on the host and exposes its hot-path
subroutines (get_primary, boundary_general, flux_splitting_general, time_rk3_general) and the
step loop of general_main.f90:23-38, with the state in the reference's Fortran layout.
"""
from __future__ import annotations

import ctypes
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
_abi = importlib.import_module("2dense_gb300._abi")
DenseConfig = _abi.DenseConfig
default_config = _abi.default_config

_libs: dict[str, ctypes.CDLL] = {}


def load(timed: bool = False) -> ctypes.CDLL:
    name = "liboracle_timed.so" if timed else "liboracle.so"
    if name in _libs:
        return _libs[name]
    from . import build as _build
    paths = _build.build()
    lib = ctypes.CDLL(paths[name])
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    cfgp = ctypes.POINTER(DenseConfig)
    i = ctypes.c_int
    sigs = {
        "oracle_create": (vp, [cfgp]),
        "oracle_destroy": (None, [vp]),
        "oracle_init": (i, [vp, cfgp]),
        "oracle_set_config": (None, [vp, cfgp]),
        "oracle_get_state": (None, [vp, dp, dp]),
        "oracle_set_state": (None, [vp, dp, dp]),
        "oracle_get_grid": (None, [vp, dp, dp]),
        "oracle_get_bodyforce": (None, [vp, dp]),
        "oracle_set_bodyforce": (None, [vp, dp]),
        "oracle_get_fluxes": (None, [vp, dp, dp]),
        "oracle_get_theta": (None, [vp, dp, dp, dp, dp]),
        "oracle_get_scalars": (None, [vp, dp]),
        "oracle_set_time": (None, [vp, ctypes.c_double, i, ctypes.c_double]),
        "oracle_get_primary": (i, [vp]),
        "oracle_boundary": (i, [vp]),
        "oracle_flux": (i, [vp]),
        "oracle_time_rk3": (i, [vp, i]),
        "oracle_stage": (i, [vp, i]),
        "oracle_steps": (i, [vp, i, ctypes.c_double, i]),
        "oracle_threads": (i, []),
        "oracle_set_threads": (None, [i]),
        "oracle_count_step": (i, [cfgp, dp, ctypes.POINTER(ctypes.c_longlong)]),
        "oracle_recon": (i, [i, dp, dp]),
        "oracle_roe_lr": (i, [i, ctypes.c_double, dp, dp, dp, dp, dp]),
        "oracle_branch_costs": (i, [ctypes.c_double, ctypes.POINTER(ctypes.c_longlong)]),
    }
    for fname, (res, args) in sigs.items():
        fn = getattr(lib, fname)
        fn.restype = res
        fn.argtypes = args
    _libs[name] = lib
    return lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleSolver:
    """One reference block on the host. Arrays are float64 in Fortran order:
    cons (NIp, NJp, 4), prim (NIp, NJp, 6), x/y (ni, nj)."""

    def __init__(self, cfg: DenseConfig, init: bool = True, timed: bool = False):
        self.lib = load(timed)
        self.cfg = cfg.copy()
        self.h = self.lib.oracle_create(ctypes.byref(self.cfg))
        self.nip = cfg.ni + 8
        self.njp = cfg.nj + 8
        if init:
            rc = self.lib.oracle_init(self.h, ctypes.byref(self.cfg))
            if rc:
                raise RuntimeError(f"oracle init_general failed: {rc}")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.oracle_destroy(h)
            self.h = None

    # -- state --------------------------------------------------------------------------
    def get_state(self):
        cons = np.zeros((self.nip, self.njp, 4), order="F")
        prim = np.zeros((self.nip, self.njp, 6), order="F")
        self.lib.oracle_get_state(self.h, _dp(cons), _dp(prim))
        return cons, prim

    def set_state(self, cons=None, prim=None):
        c = None if cons is None else np.asfortranarray(cons, dtype=np.float64)
        p = None if prim is None else np.asfortranarray(prim, dtype=np.float64)
        self.lib.oracle_set_state(self.h, None if c is None else _dp(c), None if p is None else _dp(p))

    def set_config(self, cfg: DenseConfig):
        self.cfg = cfg.copy()
        self.lib.oracle_set_config(self.h, ctypes.byref(self.cfg))

    def grid(self):
        x = np.zeros((self.cfg.ni, self.cfg.nj), order="F")
        y = np.zeros((self.cfg.ni, self.cfg.nj), order="F")
        self.lib.oracle_get_grid(self.h, _dp(x), _dp(y))
        return x, y

    def fluxes(self):
        hx = np.zeros((self.cfg.ni + 1, self.cfg.nj, 4), order="F")
        he = np.zeros((self.cfg.nj + 1, self.cfg.ni, 4), order="F")
        self.lib.oracle_get_fluxes(self.h, _dp(hx), _dp(he))
        return hx, he

    def theta(self):
        ni, nj = self.cfg.ni, self.cfg.nj
        txp = np.zeros((4, ni + 1, nj), order="F")
        txn = np.zeros((4, ni + 1, nj), order="F")
        tep = np.zeros((4, nj + 1, ni), order="F")
        ten = np.zeros((4, nj + 1, ni), order="F")
        self.lib.oracle_get_theta(self.h, _dp(txp), _dp(txn), _dp(tep), _dp(ten))
        return txp, txn, tep, ten

    def bodyforce(self):
        bf = np.zeros((self.nip, self.njp, 4), order="F")
        self.lib.oracle_get_bodyforce(self.h, _dp(bf))
        return bf

    def scalars(self) -> dict:
        out = np.zeros(7)
        self.lib.oracle_get_scalars(self.h, _dp(out))
        return {"dt": out[0], "max_eig_i": out[1], "max_eig_j": out[2], "time": out[3],
                "elasp_time": out[4], "step": int(out[5]), "recon_noop": bool(out[6])}

    def set_time(self, t: float, step: int = 0, dt: float | None = None):
        self.lib.oracle_set_time(self.h, t, step, self.cfg.dt if dt is None else dt)

    # -- the hot path ---------------------------------------------------------------------
    def get_primary(self):
        self.lib.oracle_get_primary(self.h)

    def boundary(self):
        rc = self.lib.oracle_boundary(self.h)
        if rc:
            raise RuntimeError(f"boundary_general: {rc}")

    def flux(self):
        rc = self.lib.oracle_flux(self.h)
        if rc:
            raise RuntimeError(f"flux_splitting_general: {rc}")

    def time_rk3(self, irk: int):
        self.lib.oracle_time_rk3(self.h, irk)

    def stage(self, irk: int):
        rc = self.lib.oracle_stage(self.h, irk)
        if rc:
            raise RuntimeError(f"stage {irk}: {rc}")

    def steps(self, n: int, t_end: float = 1e300, total_step: int = 2**31 - 1):
        rc = self.lib.oracle_steps(self.h, n, t_end, total_step)
        if rc:
            raise RuntimeError(f"steps: {rc}")


def count_step_flops(cfg: DenseConfig, cons: np.ndarray | None = None) -> dict:
    """Floating-point operations of one full step of the reference on field values
    (add/sub, mul, div, sqrt each counted as one; transcendental calls counted apart)."""
    lib = load(False)
    out = (ctypes.c_longlong * 16)()
    c = None if cons is None else np.asfortranarray(cons, dtype=np.float64)
    rc = lib.oracle_count_step(ctypes.byref(cfg), None if c is None else _dp(c), out)
    if rc:
        raise RuntimeError(f"count_step: {rc}")
    (add, mul, div, sqrt, transc, cells, p_prim, p_bc, p_flux, p_rk, d_xi, d_eta, n_sm, n_ch,
     n_sm1, n_ch1) = list(out)
    flops = add + mul + div + sqrt
    return {"add": add, "mul": mul, "div": div, "sqrt": sqrt, "transcendental": transc,
            "cells": cells, "flops": flops, "flops_per_cell_update": flops / cells,
            "phase": {"get_primary": p_prim, "boundary": p_bc, "flux": p_flux, "time_rk3": p_rk},
            "flux_dir": {"xi": d_xi, "eta": d_eta},
            "adaweno_branches": {"smooth": n_sm + n_sm1, "char": n_ch + n_ch1,
                                 "smooth_xi": n_sm, "char_xi": n_ch, "smooth_eta": n_sm1, "char_eta": n_ch1}}


def branch_costs(gamma: float = 1.4) -> dict:
    """Operations of one AdaWENO smooth branch and one characteristic branch (one interface,
    one sign); both are independent of the data."""
    lib = load(False)
    out = (ctypes.c_longlong * 2)()
    lib.oracle_branch_costs(gamma, out)
    return {"smooth": out[0], "char": out[1]}


def recon(kind: int, lf) -> np.ndarray:
    """One stencil evaluation: kind 251/253/255 -> [h]; 1 -> WENO-JS weights; 2 -> WENO-Z
    weights and theta."""
    lib = load(False)
    a = np.ascontiguousarray(lf, dtype=np.float64)
    out = np.zeros(4)
    if lib.oracle_recon(kind, _dp(a), _dp(out)):
        raise ValueError(kind)
    return out[:1] if kind > 200 else out[:3 if kind == 1 else 4]


def roe_lr(direction: int, gamma: float, left, right):
    """Roe average (u0,v0,h0,alpha0) of two primitive states (rho,u,v,p) and the eigenvector
    matrices L[c,k] = l(c+1,k+1), R[k,e] = r(k+1,e+1)."""
    lib = load(False)
    le = np.ascontiguousarray(left, dtype=np.float64)
    ri = np.ascontiguousarray(right, dtype=np.float64)
    roe = np.zeros(4)
    L = np.zeros(16)
    R = np.zeros(16)
    lib.oracle_roe_lr(direction, gamma, _dp(le), _dp(ri), _dp(roe), _dp(L), _dp(R))
    return roe, L.reshape(4, 4), R.reshape(4, 4)


def threads() -> int:
    return load(False).oracle_threads()
