"""The discrete adjoint against autograd through the pure-PyTorch reference step and against
central finite differences of the CUDA forward."""
import importlib

import numpy as np
import pytest
import torch

import torch_step
from test_torch_step import to_state, vortex_cfg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adjoint(dense):
    return importlib.import_module("2dense_gb300.adjoint")


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def perturbed_state(dense, cfg, seed=0, amp=1e-3):
    c, cons, prim, x, y = dense.init_general(cfg)
    U = torch.from_numpy(to_state(cons)).cuda()
    g = torch.Generator(device="cpu").manual_seed(seed)
    U[0] += amp * torch.randn(U.shape[1:], generator=g, dtype=torch.float64).cuda()
    return c, U.contiguous()


@pytest.mark.parametrize("split,recon", [(101, 251), (101, 253), (101, 255), (102, 251), (102, 253),
                                         (102, 255), (103, 251), (103, 253), (103, 255), (104, 0), (105, 0)])
def test_rhs_vjp_matches_autograd(dense, adjoint, split, recon):
    cfg = vortex_cfg(dense, recon, ni=24, nj=20, var_eps=4.0, var_xc=4.6, var_yc=5.3, splitting=split)
    c, U = perturbed_state(dense, cfg)
    v = torch.randn(U.shape, generator=torch.Generator().manual_seed(1), dtype=torch.float64).cuda()
    with adjoint.Adjoint(c) as adj:
        out, vdotl = adj.rhs_vjp(U, v)
    Ut = U.clone().requires_grad_(True)
    L = torch_step.rhs(Ut, c.gamma, c.dx, c.dy, recon, split, delta=c.delta)
    (ref,) = torch.autograd.grad(L, Ut, v)
    L = L.detach()
    # two evaluation orders of derivatives whose WENO weights scale like 1/(1e-6 + beta)^3
    assert rel(out, ref) < 1e-10
    assert abs(vdotl - float((v * L).sum())) < 1e-12 * float((v * L).abs().sum())


@pytest.mark.parametrize("split,recon,const_dt", [(101, 253, 0), (101, 255, 0), (101, 251, 0), (101, 253, 1),
                                                  (102, 253, 0), (102, 255, 0), (102, 251, 1),
                                                  (103, 253, 0), (103, 255, 0), (104, 0, 0), (104, 0, 1),
                                                  (105, 0, 0)])
def test_steps_gradient_matches_autograd(dense, adjoint, split, recon, const_dt):
    """7 steps with checkpoints every 3: two full segments and a partial one."""
    cfg = vortex_cfg(dense, recon, ni=24, nj=20, var_eps=4.0, var_xc=4.6, var_yc=5.3,
                     if_const_dt=const_dt, dt=0.02, splitting=split)
    c, U = perturbed_state(dense, cfg)
    gT = torch.randn(U.shape, generator=torch.Generator().manual_seed(2), dtype=torch.float64).cuda()
    with adjoint.Adjoint(c, checkpoint_every=3) as adj:
        uT = adj.forward(U, 7)
        g0 = adj.backward(gT)
        dts = adj.dts()
    Ut = U.clone().requires_grad_(True)
    ref_T = torch_step.run(Ut, 7, c.gamma, c.dx, c.dy, recon, c.cfl, c.dt if const_dt else None, split,
                           delta=c.delta)
    assert rel(uT, ref_T.detach()) < 1e-12
    (ref,) = torch.autograd.grad(ref_T, Ut, gT)
    assert rel(g0, ref) < 1e-10
    assert np.all(dts > 0) and (not const_dt or np.all(dts == c.dt))


def padded(U):
    """Interior (4, nj, ni) tensor -> Fortran cons(ni+8, nj+8, 4) with empty ghosts."""
    u = U.cpu().numpy()
    cons = np.zeros((u.shape[2] + 8, u.shape[1] + 8, 4), order="F")
    cons[4:-4, 4:-4, :] = u.transpose(2, 1, 0)
    return cons


@pytest.mark.parametrize("split,recon", [(101, 251), (101, 253), (101, 255), (102, 255), (103, 253), (104, 0),
                                         (105, 0)])
def test_taped_recompute_reproduces_the_forward(dense, adjoint, split, recon):
    """The taping sweeps of the reverse pass recompute each segment bit for bit: after a
    backward the solver holds the state after the first segment, equal to a plain solve, and the
    fluxes of a taped stage equal the plain sweep's."""
    cfg = vortex_cfg(dense, recon, ni=40, nj=32, splitting=split)
    c, U = perturbed_state(dense, cfg)
    with adjoint.Adjoint(c, checkpoint_every=5) as adj:
        adj.forward(U, 12)
        adj.backward(torch.ones_like(U))
        cons_b = adj.solver_state()[0]
        adj.rhs_vjp(U, torch.ones_like(U))
        _, hx_t, he_t = adj.solver_state()
    with dense.Solver(c) as s:
        s.upload(padded(U))
        s.steps(5)
        np.testing.assert_array_equal(s.download(False)[4:-4, 4:-4], cons_b[4:-4, 4:-4])
    with dense.Solver(c) as s:
        s.upload(padded(U))
        s.stage(1)
        hx, he = s.fluxes()
        np.testing.assert_array_equal(hx, hx_t)
        np.testing.assert_array_equal(he, he_t)


def test_backward_is_deterministic_and_repeatable(dense, adjoint):
    cfg = vortex_cfg(dense, 253, ni=40, nj=32)
    c, U = perturbed_state(dense, cfg)
    gT = torch.ones_like(U)
    with adjoint.Adjoint(c, checkpoint_every=4) as adj:
        adj.forward(U, 9)
        a = adj.backward(gT)
        b = adj.backward(gT)
    assert torch.equal(a, b)


@pytest.mark.parametrize("split", [101, 102, 103])
def test_autograd_function_in_a_graph(dense, adjoint, split):
    """Loss 1/2 ||rho(T) - rho_target||^2 of a vortex built from (eps, xc, yc) by torch ops:
    autograd chains the vortex's derivatives with the adjoint; checked against central
    differences of the CUDA forward, which must not change the cells of the wave-speed maxima
    (the time step, and GLF's wave speed, are not differentiable where they switch)."""
    cfg = vortex_cfg(dense, 253, ni=48, nj=48, cfl=0.4, splitting=split)
    c = dense.init_general(cfg)[0]
    n, h = 30, 1e-6
    with adjoint.Adjoint(c, checkpoint_every=8) as adj:
        target = adj.forward(adjoint.vortex_state(c, 5.0, 5.0, 5.0), n)[0].clone()
        theta = torch.tensor([4.8, 5.1, 4.9], dtype=torch.float64, device="cuda", requires_grad=True)

        def loss_of(th):
            uT = adjoint.AdjointStep.apply(adjoint.vortex_state(c, th[0], th[1], th[2]), adj, n)
            return 0.5 * ((uT[0] - target) ** 2).sum()

        loss = loss_of(theta)
        loss.backward()
        grad = theta.grad.detach().cpu().numpy()
        am0 = adj.argmax().copy()
        for k in range(3):
            vals, traces = [], []
            for s in (1, -1):
                th = theta.detach().clone()
                th[k] += s * h
                th.requires_grad_(True)
                lk = loss_of(th)
                lk.backward()
                vals.append(float(lk.detach()))
                traces.append(adj.argmax().copy())
            assert np.array_equal(traces[0], traces[1]) and np.array_equal(traces[0], am0)
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - grad[k]) <= 1e-6 * abs(grad[k]), (k, fd, grad[k])


def rough_state(dense, cfg, seed):
    """A seeded positive state of cfg's grid, smooth on the scale of a few cells. On the double
    Mach reflection's grid its scale is the post-shock inflow's (rho 8, p 116.5), so that the
    stages keep the pressure positive next to the inflow ghosts."""
    c = dense.init_general(cfg)[0]
    g = torch.Generator().manual_seed(seed)
    sm = lambda: torch.nn.functional.avg_pool2d(torch.rand(1, 1, c.nj + 4, c.ni + 4, generator=g,
                                                           dtype=torch.float64), 5, 1)[0, 0]
    if cfg.benchmark == 5:
        rho, u, v, p = 4.0 + 4.0 * sm(), 8.0 * sm() - 2.0, 4.0 * sm() - 2.0, 60.0 + 60.0 * sm()
    else:
        rho, u, v, p = 0.5 + 1.5 * sm(), 2.0 * sm() - 1.0, 2.0 * sm() - 1.0, 0.5 + 1.5 * sm()
    U = torch.stack([rho, rho * u, rho * v, p / (c.gamma - 1.0) + 0.5 * rho * (u * u + v * v)])
    return c, U.contiguous().cuda()


@pytest.mark.parametrize("bench,split,recon", [(1, 101, 253), (2, 101, 255), (4, 102, 253), (9, 103, 255),
                                               (2, 103, 251), (1, 102, 255), (3, 101, 253), (13, 102, 255),
                                               (13, 103, 253), (5, 101, 253), (5, 102, 255), (5, 103, 253),
                                               (1, 104, 0), (2, 104, 0), (3, 104, 0), (4, 104, 0), (5, 104, 0),
                                               (9, 104, 0), (13, 104, 0), (1, 105, 0), (2, 105, 0), (3, 105, 0),
                                               (4, 105, 0), (5, 105, 0), (13, 105, 0), (6, 101, 253), (6, 102, 255),
                                               (6, 103, 253), (6, 104, 0), (6, 105, 0)])
def test_rhs_vjp_with_walls_matches_autograd(dense, adjoint, bench, split, recon):
    """The reference's benchmarks with walls -- extrapolated (1: x; 2: top, right; 4, 9: sides;
    5: right), mirror (2: bottom, left; 4, 9: bottom, top; 13: sides; 5: the bottom from x = 1/6)
    and fixed-state sides (3, 13: bottom, top; 5: inflow, top, the bottom before the wall): the
    ghost cells' split sensitivities sent back through the rules (none through a fixed state but
    GLF's global lambda), against autograd through the PyTorch step's ghost layers."""
    cfg = dense.config_default(ni=24, nj=20, benchmark=bench, splitting=split, recon=recon, cfl=0.4)
    c, U = rough_state(dense, cfg, seed=bench * 10 + split % 10)
    v = torch.randn(U.shape, generator=torch.Generator().manual_seed(3), dtype=torch.float64).cuda()
    with adjoint.Adjoint(c) as adj:
        out, vdotl = adj.rhs_vjp(U, v)
    Ut = U.clone().requires_grad_(True)
    L = torch_step.rhs(Ut, c.gamma, c.dx, c.dy, recon, split, bench, delta=c.delta)
    (ref,) = torch.autograd.grad(L, Ut, v)
    assert rel(out, ref) < 1e-10
    assert abs(vdotl - float((v * L.detach()).sum())) < 1e-12 * float((v * L.detach()).abs().sum())


@pytest.mark.parametrize("bench,split,recon", [(4, 101, 253), (2, 102, 255), (1, 103, 253), (3, 101, 253),
                                               (13, 102, 253), (13, 103, 255), (5, 101, 253), (5, 102, 253),
                                               (5, 103, 253), (2, 104, 0), (3, 104, 0), (4, 104, 0),
                                               (5, 104, 0), (13, 104, 0), (3, 105, 0), (4, 105, 0), (5, 105, 0),
                                               (13, 105, 0), (6, 101, 253), (6, 102, 253), (6, 103, 255), (6, 104, 0),
                                               (6, 105, 0)])
def test_steps_gradient_with_walls_matches_autograd(dense, adjoint, bench, split, recon):
    """5 steps with checkpoints every 2 on grids with wall sides, CFL time step; on the
    Rayleigh-Taylor grids (3, 13) with the body force of every stage, whose time-step factor
    carries the step's sensitivity to dt as well; on the double Mach reflection's (5) with its
    top ghosts chosen by each step's start time; on the shear layer's (6) with its inflow
    oscillating in the start time, which every earlier time step moves."""
    cfg = dense.config_default(ni=24, nj=20, benchmark=bench, splitting=split, recon=recon, cfl=0.4)
    c, U = rough_state(dense, cfg, seed=7 + bench)
    gT = torch.randn(U.shape, generator=torch.Generator().manual_seed(5), dtype=torch.float64).cuda()
    with adjoint.Adjoint(c, checkpoint_every=2) as adj:
        uT = adj.forward(U, 5)
        g0 = adj.backward(gT)
    Ut = U.clone().requires_grad_(True)
    ref_T = torch_step.run(Ut, 5, c.gamma, c.dx, c.dy, recon, c.cfl, None, split, bench, delta=c.delta)
    assert rel(uT, ref_T.detach()) < 1e-12
    (ref,) = torch.autograd.grad(ref_T, Ut, gT)
    assert rel(g0, ref) < 1e-10


def test_rejects_unsupported_configurations(dense, adjoint):
    for kw in (dict(recon=0, splitting=106), dict(benchmark=7), dict(ni=6)):
        cfg = dense.init_general(vortex_cfg(dense, 253))[0]
        for k, v in kw.items():
            setattr(cfg, k, v)
        with pytest.raises(dense.DenseError):
            adjoint.Adjoint(cfg)


def test_gradients_at_the_adjoint_configuration_size(dense, adjoint):
    """The adjoint configuration's grid (256 x 256 periodic vortex, LLF + WENO-JS5, CFL 0.4,
    checkpoints every 20 steps) over 40 steps: gradients of 1/2 ||rho(T) - rho_target||^2 with
    respect to (eps, xc, yc) and along a smooth direction of a seeded Gaussian density
    perturbation (amplitude 1e-3) against Richardson-extrapolated central differences,
    (4 FD(h) - FD(2h)) / 3 at h = 1e-6, within 1e-6 relative. The extrapolation removes the
    difference's own h^2 term, which the WENO weights of a field carrying 1e-3 noise make as
    large as 1e-5 relative at h = 1e-6; the larger second step keeps the runs' rounding noise
    (about 1e-12 of the loss) well below the bar."""
    ni = nj = 256
    n, k, h = 40, 20, 1e-6
    cfg = vortex_cfg(dense, 253, ni=ni, nj=nj, cfl=0.4, var_eps=5.0, var_xc=5.0, var_yc=5.0)
    c = dense.init_general(cfg)[0]
    with adjoint.Adjoint(c, checkpoint_every=k) as adj:
        target = adj.forward(adjoint.vortex_state(c, 5.0, 5.0, 5.0), n)[0].clone()
        gen = torch.Generator().manual_seed(2024)
        drho0 = (1e-3 * torch.randn(nj, ni, generator=gen, dtype=torch.float64)).cuda()
        theta0 = torch.tensor([5.0, 5.0, 5.0], dtype=torch.float64, device="cuda")

        def loss_and_grads(th, dr):
            th = th.detach().clone().requires_grad_(True)
            dr = dr.detach().clone().requires_grad_(True)
            uT = adjoint.AdjointStep.apply(adjoint.vortex_state(c, th[0], th[1], th[2], dr), adj, n)
            loss = 0.5 * ((uT[0] - target) ** 2).sum()
            g_th, g_dr = torch.autograd.grad(loss, [th, dr])
            return float(loss.detach()), g_th, g_dr

        _, g_th, g_dr = loss_and_grads(theta0, drho0)
        am0 = adj.argmax().copy()
        xs = (torch.arange(ni, dtype=torch.float64, device="cuda") + 0.5) * 10.0 / ni
        Yg, Xg = torch.meshgrid(xs, xs, indexing="ij")
        bump = torch.exp(-((Xg - 3.0) ** 2 + (Yg - 6.0) ** 2))
        dirs = {"eps": ((1, 0, 0), None, float(g_th[0])), "xc": ((0, 1, 0), None, float(g_th[1])),
                "yc": ((0, 0, 1), None, float(g_th[2])),
                "bump": ((0, 0, 0), bump, float((g_dr * bump).sum()))}
        for name, (dth, ddr, exact) in dirs.items():
            est = {}
            for hh in (h, 2 * h):
                vals = []
                for sgn in (1.0, -1.0):
                    th = theta0 + sgn * hh * torch.tensor(dth, dtype=torch.float64, device="cuda")
                    dr = drho0 + (sgn * hh * ddr if ddr is not None else 0.0)
                    vals.append(loss_and_grads(th, dr)[0])
                    # the time step is not differentiable where the cells of its maxima switch
                    assert np.array_equal(adj.argmax(), am0), name
                est[hh] = (vals[0] - vals[1]) / (2 * hh)
            rich = (4 * est[h] - est[2 * h]) / 3
            assert abs(rich - exact) <= 1e-6 * abs(exact), (name, rich, exact, est)
