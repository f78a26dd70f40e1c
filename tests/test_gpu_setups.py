"""Device-side setups of the variant benchmarks and the vortex error norms."""
import numpy as np
import pytest

from conftest import interior

pytestmark = pytest.mark.gpu

CASES = [dict(benchmark=11, ni=48, nj=40, var_eps=3.5, var_xc=4.4, var_yc=5.7),
         dict(benchmark=13, ni=32, nj=96),
         dict(benchmark=14, ni=48, nj=48, var_amp=0.03)]


def cfg_of(dense, **kw):
    base = dict(splitting=101, recon=255, cfl=0.5)
    base.update(kw)
    return dense.setup_config(dense.config_default(**base))


@pytest.mark.parametrize("kw", CASES)
def test_device_setup_matches_host_setup(dense, kw):
    c = cfg_of(dense, **kw)
    _, cons, prim, x, y = dense.init_general(c)
    with dense.Solver(c) as s:
        s.init_device()
        got = s.download(False)
    scale = np.abs(interior(cons)).max(axis=(0, 1))
    assert (np.abs(interior(got) - interior(cons)).max(axis=(0, 1)) <= 1e-14 * scale + 1e-300).all()


@pytest.mark.parametrize("kw", CASES)
def test_device_setup_then_steps(dense, kw):
    c = cfg_of(dense, **kw)
    _, cons, prim, x, y = dense.init_general(c)
    with dense.Solver(c) as a, dense.Solver(c) as b:
        a.upload(cons, prim, x, y)
        b.init_device()
        a.steps(5)
        b.steps(5)
        ra, rb = a.download(False), b.download(False)
    rel = np.abs(interior(ra) - interior(rb)).max() / np.abs(interior(ra)).max()
    assert rel < 1e-12


def test_batched_device_setup_equals_single(dense):
    cfgs = [cfg_of(dense, **kw) for kw in CASES] + [cfg_of(dense, benchmark=11, ni=20, nj=24, var_eps=2.0)]
    with dense.BatchSolver(cfgs) as b:
        b.init_device()
        b.steps(2)
        for i, c in enumerate(cfgs):
            with dense.Solver(c) as s:
                s.init_device()
                s.steps(2)
                np.testing.assert_array_equal(interior(b.download(i)), interior(s.download(False)))


def exact_rho(c, t):
    x = (np.arange(c.ni) + 0.5) * c.dx
    y = (np.arange(c.nj) + 0.5) * c.dy
    X, Y = np.meshgrid(x, y, indexing="ij")
    rx = X - (c.var_xc + t)
    ry = Y - (c.var_yc + t)
    rx -= 10.0 * np.rint(rx / 10.0)
    ry -= 10.0 * np.rint(ry / 10.0)
    g = c.gamma
    return (1.0 - (g - 1.0) * c.var_eps ** 2 * np.exp(1.0 - (rx * rx + ry * ry)) / (8.0 * g * np.pi ** 2)) ** (1.0 / (g - 1.0))


def test_vortex_error_norms(dense):
    c = cfg_of(dense, benchmark=11, ni=64, nj=64, var_eps=5.0, var_xc=5.0, var_yc=5.0)
    with dense.Solver(c) as s:
        s.init_device()
        l1_0, linf_0 = s.vortex_error()
        assert linf_0 < 1e-12
        s.steps(40)
        l1, linf = s.vortex_error()
        rho = interior(s.download(False))[:, :, 0]
        e = np.abs(rho - exact_rho(c, s.current_time))
    assert l1 == pytest.approx(e.mean(), rel=1e-9)
    assert linf == pytest.approx(e.max(), rel=1e-9)


def test_vortex_error_converges(dense):
    errs = []
    for n in (64, 128):
        c = cfg_of(dense, benchmark=11, ni=n, nj=n, var_eps=5.0, var_xc=5.0, var_yc=5.0, recon=253)
        with dense.Solver(c) as s:
            s.init_device()
            s.steps(10 ** 6, t_end=1.0)
            errs.append(s.vortex_error()[0])
    assert errs[0] / errs[1] > 8.0
