"""CPU tests of the C ABI library: it loads, exports every symbol include/dense2d.h declares,
and its host-side parts (defaults, namelist reader, initial setups, argument checks) behave like
the reference. No GPU is touched."""
import ctypes
import importlib
import json
import os
import re

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    text = open(os.path.join(ROOT, "include", "dense2d.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dense_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(dense):
    lib = dense.load_library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_config_struct_size_matches(dense):
    lib = dense.load_library()
    assert lib.dense_config_size() == ctypes.sizeof(dense.DenseConfig)


def test_library_defaults_match_python_mirror(dense):
    a = dense.config_default()
    b = dense.default_config()
    assert a.as_dict() == b.as_dict()
    # flow_mod_general.f90:111,154,156,178,85
    assert (a.splitting, a.recon, a.delta, a.gamma, a.cfl, a.dt) == (101, 201, 0.5, 1.4, 0.5, 0.01)
    assert a.dt_save == float(np.float32(0.01))  # dt_save=0.01 is a default-real literal


@pytest.mark.parametrize("name,expect", [
    ("root", dict(benchmark=5, ni=480, nj=120, splitting=102, recon=255, cfl=0.1, total_time=0.2,
                  dt_save=0.05, dt=0.01, if_save_theta=1, delta=0.5, gamma=1.4, total_step=10000,
                  save_step=100, if_const_dt=0, if_save_binary=0, if_save_tec=1, omp_thread_num=1)),
    ("ivc", dict(benchmark=0, ni=64, nj=64, gamma=1.3999999761581421, total_time=100.0,
                 dt_save=20.0, dt=0.05, if_save_binary=1)),
    ("rt", dict(benchmark=2, ni=120, nj=480, if_bodyforce=1, gamma=1.666667, total_time=1.95)),
    ("double_mach", dict(benchmark=5, splitting=104, recon=255, if_save_theta=0)),
    ("build", dict(benchmark=2, if_bodyforce=0, splitting=104)),
])
def test_namelist_reads_shipped_inputs(dense, name, expect):
    c = dense.read_par_namelist(os.path.join(GOLDEN, "inputs", f"{name}.in"))
    for k, v in expect.items():
        assert getattr(c, k) == v, (k, getattr(c, k), v)


def test_namelist_errors(dense, tmp_path):
    bad = tmp_path / "input.in"
    bad.write_text("&GAS_PARS\n GAMMA= 1.4, NOT_A_NAME=3\n /\n")
    with pytest.raises(dense.DenseError) as e:
        dense.read_par_namelist(str(bad))
    assert e.value.code == 7
    with pytest.raises(dense.DenseError):
        dense.read_par_namelist(str(tmp_path / "missing.in"))
    ok = tmp_path / "ok.in"
    ok.write_text("! comment\n&scheme_pars\n scheme_splitting_index = 104 , delta = 0.25d0 ,\n"
                  " if_save_theta = .true. /\n")
    c = dense.read_par_namelist(str(ok))
    assert (c.splitting, c.delta, c.if_save_theta) == (104, 0.25, 1)


@pytest.mark.parametrize("field,value,code", [
    ("splitting", 106, 2),   # flux_splitting.f90:30-32
    ("benchmark", 10, 3),    # boundary_general.f90:26-28
    ("bfsize", 3, 1),
    ("stages", 2, 1),
    ("ni", 2, 1),
    ("strict", 3, 1),        # variants: 0 fast, 1 strict, 2 checked
    ("strict", -1, 1),
])
def test_create_rejects_bad_config(dense, field, value, code):
    lib = dense.load_library()
    cfg = dense.config_default(ni=16, nj=16, benchmark=11, splitting=101, recon=253, dx=0.1, dy=0.1)
    setattr(cfg, field, value)
    h = ctypes.c_void_p()
    rc = lib.dense_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == code
    assert not h.value
    assert lib.dense_last_error(None)


def test_status_flags_match_python_mirror(dense):
    abi = importlib.import_module("2dense_gb300._abi")
    header = open(os.path.join(ROOT, "include", "dense2d.h")).read()
    for name in ("NAN", "NEG_RHO", "P_FLOOR", "ROE_IMAG", "RECON_NOOP", "TIMEOUT", "BOUNDS"):
        m = re.search(r"#define DENSE_FLAG_%s\s+(0x[0-9a-fA-F]+)u" % name, header)
        assert m, name
        assert getattr(abi, "FLAG_" + name) == int(m.group(1), 16), name


@pytest.mark.parametrize("bench", [1, 2, 3, 4, 5, 6, 9, 11, 13, 14])
def test_initial_setup_bitwise_equals_oracle(dense, orc, bench):
    cfg = dense.config_default(ni=37, nj=29, benchmark=bench, var_amp=0.03)
    c, cons, prim, x, y = dense.init_general(cfg)
    o = orc.OracleSolver(cfg)
    oc, op = o.get_state()
    ox, oy = o.grid()
    np.testing.assert_array_equal(cons, oc)
    np.testing.assert_array_equal(prim, op)
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_array_equal(y, oy)
    assert (c.dx, c.dy, c.gamma, c.if_bodyforce) == (o.cfg.dx, o.cfg.dy, o.cfg.gamma, o.cfg.if_bodyforce)


def test_rt_setup_forces_gamma_and_body_force(dense):
    c, *_ = dense.init_general(dense.config_default(ni=16, nj=32, benchmark=3, gamma=1.4))
    assert c.gamma == 5.0 / 3.0 and c.if_bodyforce == 1  # init_RT_general.f90:9-10


def test_unknown_benchmark_setup(dense):
    with pytest.raises(dense.DenseError) as e:
        dense.init_general(dense.config_default(ni=16, nj=16, benchmark=10))
    assert e.value.code == 3


def test_shock_vortex_post_shock_state_matches_shock_relation(dense):
    """The shock-vortex setup's post-shock state (init_shockvortex_general.f90:264-267) is the
    output of the reference's own shock_relation.py for Mach 1.1."""
    g = json.load(open(os.path.join(GOLDEN, "shock_relation.json")))
    c, cons, prim, x, y = dense.init_general(dense.config_default(ni=40, nj=20, benchmark=9))
    right = prim[-5, 10, :4]  # last interior column (x > 0.5)
    assert right[0] == g["rho"] and right[1] == g["u"] and right[3] == g["p"]


def test_setup_config_matches_init_general(dense):
    """dense_setup_config gives the configuration dense_init_setup leaves, without the arrays."""
    for b in (1, 2, 3, 4, 5, 6, 9, 11, 13, 14):
        c = dense.config_default(ni=40, nj=24, benchmark=b)
        a = dense.init_general(c)[0]
        g = dense.setup_config(c)
        assert (g.dx, g.dy, g.gamma, g.if_bodyforce) == (a.dx, a.dy, a.gamma, a.if_bodyforce), b
