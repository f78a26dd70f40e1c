"""Host-side mirror of the reference's per-stage interface, over the C ABI of libdense2d.so.

The reference drives one block through module globals and four argument-less subroutines per
Runge-Kutta stage (source/utility/general_main.f90:26-31):

    call get_primary; call boundary_general; call flux_splitting_general; call time_rk3_general(irk)

``Solver`` keeps the same vocabulary: ``read_par_namelist`` / ``init_general`` build the block,
``stage(irk)`` is the four calls, ``steps`` is the loop of general_main.f90:23-38 on the device,
and the state comes back in the reference's Fortran layout (cons(NIp,NJp,4), prim(NIp,NJp,6)).
Every call goes to the CUDA library; there is no CPU path. Errors raise ``DenseError`` with the
library's status code instead of the reference's ``print; stop``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import DenseConfig, DenseError

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_dp)


def _check(lib, rc: int, h=None):
    if rc != _abi.DENSE_OK:
        msg = lib.dense_last_error(h)
        raise DenseError(rc, msg.decode() if msg else "")


def config_default(**overrides) -> DenseConfig:
    """Module defaults (flow_mod_general.f90:50-179) from the library, plus overrides."""
    lib = _abi.load_library()
    c = DenseConfig()
    _check(lib, lib.dense_config_default(ctypes.byref(c)))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def read_par_namelist(path: str, cfg: DenseConfig | None = None) -> DenseConfig:
    """read_par_namelist (flow_mod_general.f90:297-334): entries in the file override cfg."""
    lib = _abi.load_library()
    c = config_default() if cfg is None else cfg.copy()
    _check(lib, lib.dense_read_namelist(path.encode(), ctypes.byref(c)))
    return c


def setup_config(cfg: DenseConfig) -> DenseConfig:
    """The configuration part of init_general (dx, dy; gamma and the body force for
    Rayleigh-Taylor) without building the arrays."""
    lib = _abi.load_library()
    c = cfg.copy()
    _check(lib, lib.dense_setup_config(ctypes.byref(c)))
    return c


def read_binary(path: str, cfg: DenseConfig | None = None):
    """load_date_binary: (cfg with ni, nj, dx, dy from the file, cons(NIp,NJp,4), x, y, step,
    time) of a checkpoint written by write_binary / the reference."""
    lib = _abi.load_library()
    c = config_default() if cfg is None else cfg.copy()
    _check(lib, lib.dense_read_binary(path.encode(), ctypes.byref(c), None, None, None, None, None))
    cons = np.zeros((c.ni + 8, c.nj + 8, 4), order="F")
    x = np.zeros((c.ni, c.nj), order="F")
    y = np.zeros((c.ni, c.nj), order="F")
    st, t = ctypes.c_int(), ctypes.c_double()
    _check(lib, lib.dense_read_binary(path.encode(), ctypes.byref(c), _ptr(cons), _ptr(x), _ptr(y),
                                      ctypes.byref(st), ctypes.byref(t)))
    return c, cons, x, y, st.value, t.value


def init_general(cfg: DenseConfig):
    """init_general (init_general.f90:13-37): returns (cfg, cons, prim, x, y), with cfg.dx/dy
    (and gamma, if_bodyforce for Rayleigh-Taylor) as the setup leaves them."""
    lib = _abi.load_library()
    c = cfg.copy()
    nip, njp = c.ni + 8, c.nj + 8
    cons = np.zeros((nip, njp, 4), order="F")
    prim = np.zeros((nip, njp, 6), order="F")
    x = np.zeros((c.ni, c.nj), order="F")
    y = np.zeros((c.ni, c.nj), order="F")
    _check(lib, lib.dense_init_setup(ctypes.byref(c), _ptr(cons), _ptr(prim), _ptr(x), _ptr(y)))
    return c, cons, prim, x, y


class Solver:
    """One block of the solver resident on the GPU."""

    def __init__(self, cfg: DenseConfig):
        self.lib = _abi.load_library()
        self.cfg = cfg.copy()
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.dense_create(ctypes.byref(self.cfg), ctypes.byref(h)))
        self.h = h
        self.current_time = 0.0
        self.current_step = 0
        self.dt = cfg.dt

    @classmethod
    def from_setup(cls, cfg: DenseConfig) -> "Solver":
        """init_general + upload: the block as the reference's start-up leaves it."""
        c, cons, prim, x, y = init_general(cfg)
        s = cls(c)
        s.upload(cons, prim, x, y)
        return s

    def close(self):
        if getattr(self, "h", None):
            self.lib.dense_destroy(self.h)
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

    def _chk(self, rc):
        _check(self.lib, rc, self.h)

    # -- state -------------------------------------------------------------------------
    def upload(self, cons, prim=None, x=None, y=None):
        arrs = [None if a is None else np.asfortranarray(a, dtype=np.float64)
                for a in (cons, prim, x, y)]
        self._chk(self.lib.dense_upload(self.h, *[_ptr(a) for a in arrs]))

    def download(self, with_prim: bool = True):
        nip, njp = self.cfg.ni + 8, self.cfg.nj + 8
        cons = np.zeros((nip, njp, 4), order="F")
        prim = np.zeros((nip, njp, 6), order="F") if with_prim else None
        self._chk(self.lib.dense_download(self.h, _ptr(cons), _ptr(prim)))
        return (cons, prim) if with_prim else cons

    def fluxes(self):
        ni, nj = self.cfg.ni, self.cfg.nj
        hx = np.zeros((ni + 1, nj, 4), order="F")
        he = np.zeros((nj + 1, ni, 4), order="F")
        self._chk(self.lib.dense_get_fluxes(self.h, _ptr(hx), _ptr(he)))
        return hx, he

    def max_eig(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._chk(self.lib.dense_get_max_eig(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def status(self) -> int:
        f = ctypes.c_uint()
        self._chk(self.lib.dense_status(self.h, ctypes.byref(f)))
        return f.value

    def reconfigure(self, cfg: DenseConfig):
        self._chk(self.lib.dense_reconfigure(self.h, ctypes.byref(cfg)))
        self.cfg = cfg.copy()

    def launch_count(self) -> int:
        return int(self.lib.dense_launch_count(self.h))

    # -- the hot path ---------------------------------------------------------------------
    def stage(self, irk: int) -> float:
        """get_primary, boundary_general, flux_splitting_general, time_rk3_general(irk)."""
        dt = ctypes.c_double(self.dt)
        self._chk(self.lib.dense_stage(self.h, irk, self.current_time, ctypes.byref(dt)))
        self.dt = dt.value
        return self.dt

    def step(self):
        """One time step of general_main.f90:26-37 through three dense_stage calls."""
        for irk in range(1, self.cfg.stages + 1):
            self.stage(irk)
        self.current_step += 1
        self.current_time = self.current_time + self.dt

    def steps(self, n: int, t_end: float = float("inf"), total_step: int = 2**31 - 1):
        """Up to n steps on the device while current_time < t_end and current_step < total_step.
        Rejects nothing the reference would accept; stops like general_main.f90:23."""
        t = ctypes.c_double(self.current_time)
        s = ctypes.c_int(self.current_step)
        dt = ctypes.c_double(self.dt)
        self._chk(self.lib.dense_steps(self.h, n, t_end, total_step, ctypes.byref(t),
                                       ctypes.byref(s), ctypes.byref(dt)))
        self.current_time, self.current_step, self.dt = t.value, s.value, dt.value

    def init_device(self):
        """The benchmark's initial state computed on the device (benchmarks 11, 13, 14)."""
        self._chk(self.lib.dense_init_device(self.h))
        self.current_time, self.current_step = 0.0, 0

    def vortex_error(self):
        """(mean, max) of |rho - rho_exact| of the translating vortex at the current time."""
        l1, linf = ctypes.c_double(), ctypes.c_double()
        self._chk(self.lib.dense_vortex_error(self.h, ctypes.byref(l1), ctypes.byref(linf)))
        return l1.value, linf.value

    def write_tecplot(self, path: str):
        """write_tec_at_time_cartisian: the Tecplot ASCII file of the current state."""
        self._chk(self.lib.dense_write_tecplot(self.h, path.encode()))

    def write_theta(self, path: str):
        """write_theta_at_time_cartisian: the AdaWENO indicators of the last stage per cell."""
        self._chk(self.lib.dense_write_theta(self.h, path.encode()))

    def theta(self):
        """theta of every (interface, sign) of the last stage: (xi [2, nj, ni+1], eta [2, nj+1, ni]),
        with the splitting 105 and cfg.if_save_theta set."""
        ni, nj = self.cfg.ni, self.cfg.nj
        out = np.zeros(2 * (nj * (ni + 1) + (nj + 1) * ni))
        self._chk(self.lib.dense_get_theta(self.h, _ptr(out)))
        xs = 2 * nj * (ni + 1)
        return out[:xs].reshape(2, nj, ni + 1), out[xs:].reshape(2, nj + 1, ni)

    def write_binary(self, path: str):
        """write_date_binary: the unformatted checkpoint of the current state."""
        self._chk(self.lib.dense_write_binary(self.h, path.encode()))

    def run(self, out_dir: str, namelist: str | None = None) -> int:
        """The loop of general_main.f90 with its saves into out_dir (see dense_run); returns the
        number of saves."""
        n = ctypes.c_int()
        self._chk(self.lib.dense_run(self.h, out_dir.encode(), namelist.encode() if namelist else None,
                                     ctypes.byref(n)))
        t, s, dt = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
        self._chk(self.lib.dense_get_time(self.h, ctypes.byref(t), ctypes.byref(s), ctypes.byref(dt)))
        self.current_time, self.current_step, self.dt = t.value, s.value, dt.value
        return n.value

    def steps_async(self, n: int, t_end: float = float("inf"), total_step: int = 2**31 - 1):
        """``steps`` without waiting; time and step stay on the device (``dense_get_time``)."""
        self._chk(self.lib.dense_steps_async(self.h, n, t_end, total_step))

    def stream(self) -> int:
        """The handle's cudaStream_t, as an integer."""
        s = ctypes.c_void_p()
        self._chk(self.lib.dense_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0


class BatchSolver:
    """Many independent blocks of uneven size advanced together (the batched form).

    Every instance has its own configuration, CFL time step, time and step count; all share the
    splitting, reconstruction and kernel variant. One launch per phase covers the whole batch and
    one CUDA graph covers a step; each instance's results equal a plain ``Solver`` run's."""

    def __init__(self, cfgs):
        self.lib = _abi.load_library()
        self.cfgs = [c.copy() for c in cfgs]
        arr = (DenseConfig * len(cfgs))(*self.cfgs)
        h = ctypes.c_void_p()
        rc = self.lib.dense_batch_create(len(cfgs), arr, ctypes.byref(h))
        if rc:
            raise DenseError(rc, self.lib.dense_batch_last_error(None).decode())
        self.h = h
        self.n = len(cfgs)

    def _chk(self, rc):
        if rc:
            raise DenseError(rc, self.lib.dense_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.dense_batch_destroy(self.h)
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

    def upload(self, i: int, cons, prim=None, x=None, y=None):
        arrs = [None if a is None else np.asfortranarray(a, dtype=np.float64) for a in (cons, prim, x, y)]
        self._chk(self.lib.dense_batch_upload(self.h, i, *[_ptr(a) for a in arrs]))

    def download(self, i: int, with_prim: bool = False):
        c = self.cfgs[i]
        cons = np.zeros((c.ni + 8, c.nj + 8, 4), order="F")
        prim = np.zeros((c.ni + 8, c.nj + 8, 6), order="F") if with_prim else None
        self._chk(self.lib.dense_batch_download(self.h, i, _ptr(cons), _ptr(prim)))
        return (cons, prim) if with_prim else cons

    def set_time(self, i: int, t: float, step: int = 0):
        self._chk(self.lib.dense_batch_set_time(self.h, i, t, step))

    def time(self, i: int):
        t, s, dt = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
        self._chk(self.lib.dense_batch_get_time(self.h, i, ctypes.byref(t), ctypes.byref(s), ctypes.byref(dt)))
        return t.value, s.value, dt.value

    def steps(self, n: int, t_end: float = float("inf"), total_step: int = 2**31 - 1, wait: bool = True):
        fn = self.lib.dense_batch_steps if wait else self.lib.dense_batch_steps_async
        self._chk(fn(self.h, n, t_end, total_step))

    def init_device(self):
        """Every instance's initial state computed on the device (benchmarks 11, 13, 14)."""
        self._chk(self.lib.dense_batch_init_device(self.h))

    def set_schedule(self, xi_variant: int, eta_variant: int, order: int, mode: int | None = None):
        """Tile variants, block order and (when given) launch mode: 0 one launch per phase,
        1 one persistent launch per step."""
        self._chk(self.lib.dense_batch_set_schedule(self.h, xi_variant, eta_variant, order))
        if mode is not None:
            self.set_launch_mode(mode)

    def set_launch_mode(self, mode: int):
        self._chk(self.lib.dense_batch_set_launch_mode(self.h, mode))

    def launch_mode(self) -> int:
        m = ctypes.c_int()
        self._chk(self.lib.dense_batch_get_launch_mode(self.h, ctypes.byref(m)))
        return m.value

    def hold_instance(self, instance: int, spin_limit: int = 0):
        """Failure injection: the persistent step's waits on ``instance`` give up after
        ``spin_limit`` polls (-1 removes the hold)."""
        self._chk(self.lib.dense_batch_hold_instance(self.h, instance, spin_limit))

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._chk(self.lib.dense_batch_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def status(self) -> int:
        f = ctypes.c_uint()
        self._chk(self.lib.dense_batch_status(self.h, ctypes.byref(f)))
        return f.value

    def cells(self) -> int:
        return int(self.lib.dense_batch_cells(self.h))

    def launch_count(self) -> int:
        return int(self.lib.dense_batch_launch_count(self.h))

    @classmethod
    def from_setups(cls, cfgs) -> "BatchSolver":
        """init_general for every instance, then upload: the batch as the setups leave it."""
        setups = [init_general(c) for c in cfgs]
        b = cls([s[0] for s in setups])
        for i, (c, cons, prim, x, y) in enumerate(setups):
            b.upload(i, cons, prim, x, y)
        return b
