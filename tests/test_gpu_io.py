"""The save path: checkpoint and Tecplot files of the device state, and the driver loop with its
device-side save predicate, against plain solves."""
import struct

import numpy as np
import pytest

from conftest import interior

pytestmark = pytest.mark.gpu


def records(path):
    b = open(path, "rb").read()
    out, k = [], 0
    while k < len(b):
        (n,) = struct.unpack_from("<i", b, k)
        out.append(b[k + 4:k + 4 + n])
        assert struct.unpack_from("<i", b, k + 4 + n)[0] == n
        k += 8 + n
    return out


def tecplot(path):
    lines = open(path).read().splitlines()
    return lines[:3], np.array([float(v) for v in lines[3:]])


def vortex(dense, n=32, **kw):
    base = dict(ni=n, nj=n, benchmark=11, splitting=101, recon=253, cfl=0.5, var_eps=4.0)
    base.update(kw)
    return dense.init_general(dense.config_default(**base))


def test_checkpoint_and_tecplot_of_the_state(dense, tmp_path):
    c, cons, prim, x, y = vortex(dense, n=24)
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        s.steps(3)
        st, pr = s.download()
        s.write_binary(str(tmp_path / "a.dat2d"))
        s.write_tecplot(str(tmp_path / "a.dat"))
        step, t = s.current_step, s.current_time
    r = records(tmp_path / "a.dat2d")
    assert len(r) == 9
    assert struct.unpack("<id", r[0]) == (step, t)
    assert struct.unpack("<ii", r[3]) == (24, 24) and struct.unpack("<ii", r[4]) == (4, 4)
    np.testing.assert_array_equal(np.frombuffer(r[5]).reshape(st.shape, order="F"), st)
    np.testing.assert_array_equal(np.frombuffer(r[6]).reshape((24, 24), order="F"), x)
    c2, cons2, x2, y2, step2, t2 = dense.read_binary(str(tmp_path / "a.dat2d"))
    assert (step2, t2, c2.dx, c2.dy) == (step, t, c.dx, c.dy)
    np.testing.assert_array_equal(cons2, st)
    head, vals = tecplot(tmp_path / "a.dat")
    assert head[1].strip() == 'variables="x","y","rho","u","v","p","alpha"'
    assert "I=" in head[2] and "J=" in head[2] and "CELLCENTERED" in head[2]
    nv, nc = 25 * 25, 24 * 24
    assert vals.size == 2 * nv + 6 * nc
    vx = vals[:nv].reshape((25, 25), order="F")
    np.testing.assert_array_equal(vx[:, 0], np.arange(25) * c.dx)
    blocks = vals[2 * nv:].reshape((6, 24, 24)).transpose(0, 2, 1)  # [var][i][j]
    for v in range(5):
        np.testing.assert_array_equal(blocks[v], interior(pr)[:, :, v])
    np.testing.assert_allclose(blocks[5], np.log(interior(pr)[:, :, 3]) - np.log(interior(pr)[:, :, 0]), rtol=1e-14)


def test_run_saves_like_the_reference_loop(dense, tmp_path):
    c, cons, prim, x, y = vortex(dense, total_step=25, save_step=10, dt_save=1e9, total_time=1e9,
                                 if_save_binary=1, if_save_tec=1)
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        saves = s.run(str(tmp_path))
        final = s.download(False)
        assert s.current_step == 25
    assert saves == 2
    for k in (10, 20):
        assert (tmp_path / f"2d_{k}.dat2d").exists() and (tmp_path / f"2d_{k}.dat").exists()
    assert (tmp_path / "2d_25.dat").exists() and not (tmp_path / "2d_25.dat2d").exists()
    # the timing log of general_main.f90:20,56-58: total loop time and steps, then the average
    log = (tmp_path / "CpuTime.dat").read_text().splitlines()
    assert log[0].split(":")[0].strip() == "Total time and steps" and int(log[0].split()[-1]) == 25
    total = float(log[0].split(":")[1].split()[0])
    assert total > 0 and float(log[1].split(":")[1]) == pytest.approx(total / 25, rel=1e-12)
    with dense.Solver(c) as p:
        p.upload(cons, prim, x, y)
        p.steps(20)
        at20 = p.download(False)
        p.steps(5)
        at25 = p.download(False)
    _, cons20, _, _, step20, _ = dense.read_binary(str(tmp_path / "2d_20.dat2d"))
    assert step20 == 20
    np.testing.assert_array_equal(interior(cons20), interior(at20))
    np.testing.assert_array_equal(interior(final), interior(at25))


def test_run_time_triggered_saves(dense, tmp_path):
    """elasp_time >= dt_save triggers a save; the Tecplot save resets elasp_time."""
    c, cons, prim, x, y = vortex(dense, total_step=40, save_step=1000, dt_save=0.15, total_time=1e9)
    dts = []
    with dense.Solver(c) as p:
        p.upload(cons, prim, x, y)
        for _ in range(40):
            p.steps(1)
            dts.append(p.dt)
    expected, el = [], 0.0
    for k, dt in enumerate(dts, start=1):
        el += dt
        if el >= 0.15:
            expected.append(k)
            el = 0.0
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        saves = s.run(str(tmp_path))
    assert saves == len(expected) and len(expected) >= 2
    for k in expected:
        assert (tmp_path / f"2d_{k}.dat2d").exists()


def test_run_reads_the_namelist_at_saves(dense, tmp_path):
    c, cons, prim, x, y = vortex(dense, total_step=25, save_step=10, dt_save=1e9, total_time=1e9)
    nml = tmp_path / "input.in"
    nml.write_text("&time_step_pars\n total_step = 15\n/\n")
    out = tmp_path / "out"
    out.mkdir()
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        saves = s.run(str(out), namelist=str(nml))
        assert s.current_step == 15
    assert saves == 1 and (out / "2d_15.dat").exists()


@pytest.mark.parametrize("strict", [1, 0])
def test_adaweno_indicators_match_the_oracle(dense, orc, tmp_path, strict):
    """theta of every (interface, sign) of the last stage, and the theta file built from them."""
    cfg = dense.config_default(ni=48, nj=24, benchmark=5, splitting=105, recon=0, cfl=0.5,
                               if_save_theta=1, strict=strict)
    c, cons, prim, x, y = dense.init_general(cfg)
    with dense.Solver(c) as s:
        s.upload(cons, prim, x, y)
        s.steps(3)
        tx, te = s.theta()
        s.write_theta(str(tmp_path / "th.dat"))
    o = orc.OracleSolver(c)
    o.steps(3)
    txp, txn, tep, ten = o.theta()
    ref = [txp[0].T, txn[0].T, tep[0], ten[0]]  # -> [nj][ni+1] and [nj+1][ni]
    got = [tx[0], tx[1], te[0], te[1]]
    for g, r in zip(got, ref):
        if strict:
            np.testing.assert_array_equal(g, r)
        else:
            # theta = 1/(1 + (sum alpha - 1)^2) near shocks amplifies the fast state's 1e-13
            # differences from the reference by the indicator's ~1/(ss + beta) sensitivity
            np.testing.assert_allclose(g, r, rtol=1e-7, atol=1e-15)
    head, vals = tecplot(tmp_path / "th.dat")
    assert head[1].strip() == 'variables="x","y","xp","xn","ep","en"'
    nv, nc = 49 * 25, 48 * 24
    blocks = vals[2 * nv:].reshape(4, 24, 48)
    np.testing.assert_array_equal(blocks[0], np.maximum(tx[0][:, :-1], tx[0][:, 1:]))
    np.testing.assert_array_equal(blocks[3], np.maximum(te[1][:-1, :], te[1][1:, :]))
