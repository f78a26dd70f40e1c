"""ctypes mirror of include/dense2d.h: the configuration struct, status codes and the loader of
the in-tree shared library ``csrc/_build/libdense2d.so``.

The struct layout must match ``dense_config_t`` field for field; ``tests/test_abi.py`` checks the
size against the library's own ``sizeof``.
"""
from __future__ import annotations

import ctypes
import os

DENSE_OK = 0
DENSE_ERR_ARG = 1
DENSE_ERR_SPLITTING = 2
DENSE_ERR_BENCHMARK = 3
DENSE_ERR_CUDA = 4
DENSE_ERR_NUMERIC = 5
DENSE_ERR_TIMEOUT = 6
DENSE_ERR_IO = 7
DENSE_ERR_STATE = 8
DENSE_ERR_NOMEM = 9
DENSE_ERR_LIMIT = 10

FLAG_NAN = 0x01
FLAG_NEG_RHO = 0x02
FLAG_P_FLOOR = 0x04
FLAG_ROE_IMAG = 0x08
FLAG_RECON_NOOP = 0x10
FLAG_TIMEOUT = 0x20
FLAG_BOUNDS = 0x40  # checked variant (strict = 2): an index outside its array

ERROR_NAMES = {
    1: "DENSE_ERR_ARG", 2: "DENSE_ERR_SPLITTING", 3: "DENSE_ERR_BENCHMARK",
    4: "DENSE_ERR_CUDA", 5: "DENSE_ERR_NUMERIC", 6: "DENSE_ERR_TIMEOUT", 7: "DENSE_ERR_IO",
    8: "DENSE_ERR_STATE", 9: "DENSE_ERR_NOMEM", 10: "DENSE_ERR_LIMIT",
}

_c_int = ctypes.c_int
_c_double = ctypes.c_double


class DenseConfig(ctypes.Structure):
    """dense_config_t: the six namelists of input.in (flow_mod_general.f90:50-179)."""

    _fields_ = [
        ("ni", _c_int), ("nj", _c_int), ("bfsize", _c_int), ("neq", _c_int),
        ("benchmark", _c_int), ("if_bodyforce", _c_int), ("if_source", _c_int),
        ("if_viscous", _c_int),
        ("splitting", _c_int), ("recon", _c_int), ("delta", _c_double),
        ("stages", _c_int), ("if_const_dt", _c_int), ("cfl", _c_double), ("dt", _c_double),
        ("total_time", _c_double), ("dt_save", _c_double),
        ("total_step", _c_int), ("save_step", _c_int),
        ("if_save_binary", _c_int), ("if_save_tec", _c_int), ("if_save_theta", _c_int),
        ("gamma", _c_double),
        ("dx", _c_double), ("dy", _c_double),
        ("var_eps", _c_double), ("var_xc", _c_double), ("var_yc", _c_double),
        ("var_amp", _c_double),
        ("omp_thread_num", _c_int), ("if_curve_grid", _c_int), ("if_read_from_file", _c_int),
        ("scheme_vis_index", _c_int),
        ("mach_inf", _c_double), ("reynolds", _c_double),
        ("strict", _c_int),
        ("reserved", _c_int * 7),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}

    def copy(self) -> "DenseConfig":
        c = DenseConfig()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(DenseConfig))
        return c


def default_config(**overrides) -> DenseConfig:
    """The module defaults of flow_mod_general.f90:50-179, plus keyword overrides.

    Mirrors ``dense_config_default`` in the library, so it can be used without loading it.
    """
    c = DenseConfig()
    c.ni = c.nj = 64
    c.bfsize = 4
    c.neq = 4
    c.benchmark = 0
    c.if_bodyforce = c.if_source = c.if_viscous = 0
    c.splitting = 101
    c.recon = 201
    c.delta = 0.5
    c.stages = 3
    c.if_const_dt = 0
    c.cfl = 0.5
    c.dt = 0.01
    c.total_time = 0.0
    c.dt_save = float(ctypes.c_float(0.01).value)
    c.total_step = 1
    c.save_step = 100
    c.if_save_binary = 1
    c.if_save_tec = 1
    c.if_save_theta = 0
    c.gamma = 1.4
    c.dx = c.dy = 0.0
    c.var_eps, c.var_xc, c.var_yc, c.var_amp = 5.0, 5.0, 5.0, 0.0
    c.omp_thread_num = 4
    c.if_curve_grid = c.if_read_from_file = 0
    c.scheme_vis_index = 301
    c.mach_inf = 1.0
    c.reynolds = 500.0
    c.strict = 0
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise KeyError(f"dense_config_t has no field {k!r}")
        setattr(c, k, v)
    return c


def array_sizes(cfg: DenseConfig) -> tuple[int, int, int]:
    """Element counts of the host arrays cons(NIp,NJp,4), prim(NIp,NJp,6), x(ni,nj)."""
    nip = cfg.ni + 2 * 4
    njp = cfg.nj + 2 * 4
    return nip * njp * 4, nip * njp * 6, cfg.ni * cfg.nj


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "csrc", "_build", "libdense2d.so")


class DenseError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load_library(path: str | None = None):
    """Load libdense2d.so (built by ``build.build()``). Raises if it is missing: there is no
    fallback path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    cfgp = ctypes.POINTER(DenseConfig)
    sigs = {
        "dense_config_default": (_c_int, [cfgp]),
        "dense_read_namelist": (_c_int, [ctypes.c_char_p, cfgp]),
        "dense_init_setup": (_c_int, [cfgp, dp, dp, dp, dp]),
        "dense_array_sizes": (_c_int, [cfgp, ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_longlong)]),
        "dense_create": (_c_int, [cfgp, ctypes.POINTER(vp)]),
        "dense_upload": (_c_int, [vp, dp, dp, dp, dp]),
        "dense_stage": (_c_int, [vp, _c_int, _c_double, dp]),
        "dense_steps": (_c_int, [vp, _c_int, _c_double, _c_int, dp,
                                 ctypes.POINTER(_c_int), dp]),
        "dense_download": (_c_int, [vp, dp, dp]),
        "dense_get_max_eig": (_c_int, [vp, dp, dp]),
        "dense_reconfigure": (_c_int, [vp, cfgp]),
        "dense_status": (_c_int, [vp, ctypes.POINTER(ctypes.c_uint)]),
        "dense_last_error": (ctypes.c_char_p, [vp]),
        "dense_destroy": (None, [vp]),
        "dense_get_fluxes": (_c_int, [vp, dp, dp]),
        "dense_launch_count": (ctypes.c_longlong, [vp]),
        "dense_config_size": (_c_int, []),
        "dense_measure_fp64": (_c_int, [_c_int, dp]),
        "dense_get_stream": (_c_int, [vp, ctypes.POINTER(vp)]),
        "dense_steps_async": (_c_int, [vp, _c_int, _c_double, _c_int]),
        "dense_set_time": (_c_int, [vp, _c_double, _c_int]),
        "dense_get_time": (_c_int, [vp, dp, ctypes.POINTER(_c_int), dp]),
        "dense_sync": (_c_int, [vp]),
        "dense_profile_stage": (_c_int, [vp, _c_int, ctypes.POINTER(ctypes.c_float)]),
        "dense_fastmath_check": (_c_int, [dp, dp, _c_int]),
        "dense_batch_create": (_c_int, [_c_int, cfgp, ctypes.POINTER(vp)]),
        "dense_batch_destroy": (None, [vp]),
        "dense_batch_upload": (_c_int, [vp, _c_int, dp, dp, dp, dp]),
        "dense_batch_download": (_c_int, [vp, _c_int, dp, dp]),
        "dense_batch_set_time": (_c_int, [vp, _c_int, _c_double, _c_int]),
        "dense_batch_get_time": (_c_int, [vp, _c_int, dp, ctypes.POINTER(_c_int), dp]),
        "dense_batch_steps": (_c_int, [vp, _c_int, _c_double, _c_int]),
        "dense_batch_steps_async": (_c_int, [vp, _c_int, _c_double, _c_int]),
        "dense_batch_set_schedule": (_c_int, [vp, _c_int, _c_int, _c_int]),
        "dense_batch_schedule_space": (_c_int, [ctypes.POINTER(_c_int)] * 3),
        "dense_batch_set_launch_mode": (_c_int, [vp, _c_int]),
        "dense_batch_get_launch_mode": (_c_int, [vp, ctypes.POINTER(_c_int)]),
        "dense_batch_hold_instance": (_c_int, [vp, _c_int, ctypes.c_longlong]),
        "dense_batch_get_stream": (_c_int, [vp, ctypes.POINTER(vp)]),
        "dense_batch_status": (_c_int, [vp, ctypes.POINTER(ctypes.c_uint)]),
        "dense_batch_launch_count": (ctypes.c_longlong, [vp]),
        "dense_batch_cells": (ctypes.c_longlong, [vp]),
        "dense_batch_last_error": (ctypes.c_char_p, [vp]),
        "dense_count_branches": (_c_int, [vp, _c_int]),
        "dense_get_branch_counts": (_c_int, [vp, ctypes.POINTER(ctypes.c_ulonglong)]),
        "dense_stage_noalloc": (_c_int, [cfgp, _c_int, _c_double, vp, vp, vp, vp, vp, vp, dp, vp]),
        "dense_setup_config": (_c_int, [cfgp]),
        "dense_write_tecplot": (_c_int, [vp, ctypes.c_char_p]),
        "dense_write_binary": (_c_int, [vp, ctypes.c_char_p]),
        "dense_write_theta": (_c_int, [vp, ctypes.c_char_p]),
        "dense_get_theta": (_c_int, [vp, dp]),
        "dense_read_binary": (_c_int, [ctypes.c_char_p, cfgp, dp, dp, dp, ctypes.POINTER(_c_int), dp]),
        "dense_run": (_c_int, [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_c_int)]),
        "dense_grid_coords": (_c_int, [cfgp, dp, dp, dp, dp]),
        "dense_init_device": (_c_int, [vp]),
        "dense_vortex_error": (_c_int, [vp, dp, dp]),
        "dense_batch_init_device": (_c_int, [vp]),
        "dense_upload_device": (_c_int, [vp, vp, vp, vp]),
        "dense_download_device": (_c_int, [vp, vp, vp, vp]),
        "dense_rhs_device": (_c_int, [vp, _c_int, vp, vp]),
        "dense_steps_device": (_c_int, [vp, _c_int, _c_double, _c_int, vp]),
        "dense_stage_device": (_c_int, [vp, _c_int, vp, vp, _c_double, vp]),
        "dense_batch_upload_device": (_c_int, [vp, _c_int, vp, vp, vp]),
        "dense_batch_download_device": (_c_int, [vp, _c_int, vp, vp, vp]),
        "dense_batch_steps_device": (_c_int, [vp, _c_int, _c_double, _c_int, vp]),
        "dense_adjoint_create": (_c_int, [cfgp, _c_int, ctypes.POINTER(vp)]),
        "dense_adjoint_destroy": (None, [vp]),
        "dense_adjoint_forward": (_c_int, [vp, vp, _c_int, vp, vp]),
        "dense_adjoint_backward": (_c_int, [vp, vp, vp, vp]),
        "dense_adjoint_rhs_vjp": (_c_int, [vp, vp, vp, vp, dp, vp]),
        "dense_adjoint_get_dts": (_c_int, [vp, dp, _c_int]),
        "dense_adjoint_get_argmax": (_c_int, [vp, ctypes.POINTER(_c_int), _c_int]),
        "dense_adjoint_get_solver": (_c_int, [vp, ctypes.POINTER(vp)]),
        "dense_adjoint_launch_count": (ctypes.c_longlong, [vp]),
        "dense_adjoint_last_error": (ctypes.c_char_p, [vp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
