"""Pure-PyTorch float64 reference of the time step, for checking the adjoint kernels against
autograd (test infrastructure; never used by the library).

Same scheme as the plain solver: get_primary (get_primary.f90:53-60), LLF splitting with
lambda = |u_n| + alpha per cell (flux_splitting_LLF.f90:67-81) or GLF splitting with lambda the
maximum of |u_n| + alpha over the stage's input (flux_splitting_GLF.f90:13-70, the max_eig_i/j of
get_primary.f90:69-73), or Steger-Warming splitting with the three eigenvalues u_n, u_n -+ alpha
split as (l +- sqrt(l^2 + eps^2))/2, eps = 0.125 (flux_splitting_SW.f90:14-168), upwind5 /
WENO-JS5 / WENO-Z5
reconstruction of F+ and F- at each face (scheme_*_general.f90, weno_mod.f90), the flux
difference, and TVD-RK3 (time_advance_general.f90:9-267) with dt = cfl/(max(|u|+alpha)/dx +
max(|v|+alpha)/dy) of the step's input (or a constant dt). States are (4, nj, ni) tensors of the
interior; periodic neighbours come from torch.roll, and the ghost layers of the benchmarks with
walls from the reference's rules (RULES).
"""
from __future__ import annotations

import math

import torch

SS = float(torch.tensor(1.0e-6, dtype=torch.float32))  # weno_mod.f90:37, a default-real literal
C = (0.1, 0.6, 0.3)


def _recon(f, rec):
    f0, f1, f2, f3, f4 = f
    if rec == 251:
        return (2.0 * f0 - 13.0 * f1 + 47.0 * f2 + 27.0 * f3 - 3.0 * f4) / 60.0
    q0 = 1.0 / 3.0 * f0 - 7.0 / 6.0 * f1 + 11.0 / 6.0 * f2
    q1 = -1.0 / 6.0 * f1 + 5.0 / 6.0 * f2 + 1.0 / 3.0 * f3
    q2 = 1.0 / 3.0 * f2 + 5.0 / 6.0 * f3 - 1.0 / 6.0 * f4
    b0 = 13.0 * (f0 - 2.0 * f1 + f2) ** 2 / 12.0 + (f0 - 4.0 * f1 + 3.0 * f2) ** 2 / 4.0
    b1 = 13.0 * (f1 - 2.0 * f2 + f3) ** 2 / 12.0 + (f1 - f3) ** 2 / 4.0
    b2 = 13.0 * (f2 - 2.0 * f3 + f4) ** 2 / 12.0 + (3.0 * f2 - 4.0 * f3 + f4) ** 2 / 4.0
    if rec == 253:
        a0, a1, a2 = C[0] / (SS + b0) ** 2, C[1] / (SS + b1) ** 2, C[2] / (SS + b2) ** 2
    elif rec == 255:
        tau = (b2 - b0).abs()
        a0 = C[0] * (1.0 + (tau / (SS + b0)) ** 2)
        a1 = C[1] * (1.0 + (tau / (SS + b1)) ** 2)
        a2 = C[2] * (1.0 + (tau / (SS + b2)) ** 2)
    else:
        raise ValueError(rec)
    s = a0 + a1 + a2
    return a0 / s * q0 + a1 / s * q1 + a2 / s * q2


def primitives(U, gamma):
    rho = U[0]
    u = U[1] / rho
    v = U[2] / rho
    p = (gamma - 1.0) * (U[3] - 0.5 * rho * (u * u + v * v))
    a = torch.sqrt(gamma * p / rho)
    return rho, u, v, p, a


def steger_warming(rho, u, v, a, gamma, d):
    """(F+, F-) of the Steger-Warming splitting in direction d (0: x, 1: y)."""
    eps2 = 0.125 ** 2
    g1 = gamma - 1.0
    un, ut = (u, v) if d == 0 else (v, u)
    l1, l2, l3 = un, un - a, un + a
    s1, s2, s3 = (torch.sqrt(l * l + eps2) for l in (l1, l2, l3))
    uu2 = u * u + v * v
    q2, q3 = l2 * l2 + ut * ut, l3 * l3 + ut * ut
    out = []
    for sg in (1.0, -1.0):
        p1, p2, p3 = (l1 + sg * s1) / 2.0, (l2 + sg * s2) / 2.0, (l3 + sg * s3) / 2.0
        wii = (3.0 - gamma) * (p2 + p3) * a * a / (2.0 * g1)
        A = p1 * 2.0 * g1
        c = rho / (2.0 * gamma)
        f0 = (A + p2 + p3) * c
        fn = (A * un + p2 * l2 + p3 * l3) * c
        ft = (A * ut + p2 * ut + p3 * ut) * c
        f3 = (p1 * g1 * uu2 + p2 * 0.5 * q2 + p3 * 0.5 * q3 + wii) * c
        out.append(torch.stack([f0, fn, ft, f3] if d == 0 else [f0, ft, fn, f3]))
    return out


# Ghost rules of the reference's benchmarks with fixed walls (boundary_ivc_general.f90,
# boundary_sedov_general.f90, boundary_rm_general.f90, boundary_shockvortex_general.f90,
# boundary_rt_general.f90), per side (bottom, top, left, right): "P" periodic, "E" the recursive
# 4/3, -1/3 extrapolation, "R" the mirror with the normal velocity negated, "F" a fixed state
# (Rayleigh-Taylor's bottom and top, boundary_rt_general.f90:14-57). Ghost primitives come from
# the rule applied to the interior primitives, not from the ghost conserved variables.
# The double Mach reflection (5, boundary_doublemach_general.f90): "B" its bottom, the mirror
# where the column's centre x >= 1/6 and the fixed post-shock state before it, "T" its top, the
# post-shock state ahead of the moving shock x < 1/6 + (1 + 20 t)/sqrt(3) and the pre-shock
# state behind it (t the step's start time), "F" its post-shock inflow on the left.
RULES = {1: "PPEE", 2: "RERE", 3: "FFPP", 4: "RREE", 5: "BTFE", 6: "RFFE", 9: "RREE", 11: "PPPP",
         13: "FFRR", 14: "PPPP"}
# the fixed states (rho, u, v, p) of the "F" sides: bottom, top
RT_STATES = ((2.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 2.5))
# the stage-3 body-force factor 2.0/3.0 is a default-real literal (time_advance_general.f90:242)
TWO_THIRDS_SINGLE = float(torch.tensor(2.0 / 3.0, dtype=torch.float32))


def fixed_state(gamma, rho, u, v, p):
    """Conserved variables and primitives (rho, u, v, p, alpha) of a fixed ghost state."""
    cons = (rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v))
    prim = (rho, u, v, p, (gamma * p / rho) ** 0.5)
    return cons, prim


def _pad_axis(A, axis, lo, hi, flip, fixed=None):
    """A (nv, nj, ni) padded by 4 ghost layers along axis (2: x, 1: y); flip is the component
    negated by a mirror (the normal momentum, or the normal velocity of the primitives); fixed
    the (low, high) side states of "F" rules as per-component values."""
    n = A.shape[axis]
    take = lambda k: A.narrow(axis, k, 1)
    sign = torch.ones(A.shape[0], dtype=A.dtype, device=A.device)
    sign[flip] = -1.0
    sign = sign.view(-1, 1, 1)

    def as_layer(state, like):  # per-component constants, or a tensor of one ghost layer
        if isinstance(state, torch.Tensor):
            return state.expand_as(like)
        return torch.tensor(state, dtype=A.dtype, device=A.device).view(-1, 1, 1).expand_as(like)

    def side(rule, inner, state=None):  # inner(d): the interior slice at distance d (1 = adjacent)
        if rule == "P":
            return None
        if rule in "FT":
            g = as_layer(state, inner(1))
            return [g for _ in range(4)]
        if rule == "B":  # state = (mirror mask, fixed state)
            mask, fix = state
            return [torch.where(mask, sign * inner(k + 1), as_layer(fix, inner(1))) for k in range(4)]
        if rule == "R":
            return [sign * inner(k + 1) for k in range(4)]
        a, b = inner(1), inner(2)
        out = []
        for _ in range(4):
            g = 4.0 / 3.0 * a - 1.0 / 3.0 * b
            out.append(g)
            b, a = a, g
        return out

    low = side(lo, lambda d: take(d - 1), fixed[0] if fixed else None)
    high = side(hi, lambda d: take(n - d), fixed[1] if fixed else None)
    if low is None:
        low = [take(n - 1 - k) for k in range(4)]
    if high is None:
        high = [take(k) for k in range(4)]
    return torch.cat(list(reversed(low)) + [A] + high, dim=axis)


def ssl_sides(U, gamma, dy, t):
    """The shock / shear layer's side specifications for _rhs_padded: ((bottom, top) of the
    conserved variables, (bottom, top) of the primitives) and the same for (left, right). The
    top ghosts keep the post-shock state the setup gave them (the rule's loop body is empty,
    boundary_ssl_general.f90:47-52); the left inflow (:40-66) is rho 1.6374 above y = 0 and
    0.3626 below, p 0.3327, u = 2.5 + 0.5 tanh(2 y) and v oscillating in the step's start time t
    (a tensor: the time steps make it a function of the state)."""
    nj = U.shape[1]
    y = ((torch.arange(nj, dtype=U.dtype, device=U.device) + 1.0) - 0.5) * dy - 20.0
    post = fixed_state(gamma, 2.1101, 2.9709, -0.1367, float(torch.tensor(0.4754, dtype=torch.float32)))
    rho = torch.where(y >= 0.0, torch.full_like(y, 1.6374), torch.full_like(y, 0.3626))
    pr = torch.full_like(y, 0.3327)
    u = 2.5 + 0.5 * torch.tanh(2.0 * y)
    pie = math.pi
    e = torch.exp(-(y * y) / 10.0)
    v = (0.05 * torch.cos(torch.as_tensor(2.0 * pie * t / (30.0 / 2.68), dtype=U.dtype)) * e
         + 0.05 * torch.cos(torch.as_tensor(2.0 * pie * 2.0 * t / (30.0 / 2.68) + pie / 2.0, dtype=U.dtype)) * e)
    cons, prim = fixed_state(gamma, rho, u, v, pr)
    col = lambda q: torch.stack(list(q)).view(len(q), nj, 1)
    return ((None, post[0]), (None, post[1])), ((col(cons), None), (col(prim), None))


def dmr_sides(U, gamma, dx, t):
    """The double Mach reflection's side specifications for _rhs_padded: ((bottom, top) of the
    conserved variables, (bottom, top) of the primitives, (left) of both)."""
    ni = U.shape[2]
    x = ((torch.arange(ni, dtype=U.dtype, device=U.device) + 1.0) - 0.5) * dx
    post = fixed_state(gamma, 8.0, 8.25 * 3.0 ** 0.5 * 0.5, -8.25 * 0.5, 116.5)
    pre = fixed_state(gamma, 1.4, 0.0, 0.0, 1.0)
    wall = (x >= 1.0 / 6.0).view(1, 1, ni)
    ahead = (x < (1.0 / 6.0 + (1.0 + 20.0 * t) / 3.0 ** 0.5)).view(1, 1, ni)
    col = lambda st: torch.tensor(st, dtype=U.dtype, device=U.device).view(-1, 1, 1)
    top = [torch.where(ahead, col(post[k]), col(pre[k])) for k in range(2)]
    return ((wall, post[0]), top[0]), ((wall, post[1]), top[1]), post


def rhs(U, gamma, dx, dy, rec, split=101, bench=11, t=0.0, delta=0.5):
    """L(U) = -(h_{i+1/2} - h_{i-1/2})/dx - (g_{j+1/2} - g_{j-1/2})/dy; t is the step's start
    time (the double Mach reflection's top ghosts), delta AdaWENO's switch (105)."""
    if bench not in (11, 14) or split in (104, 105):
        if bench in (3, 13):
            fixed = [fixed_state(gamma, *st) for st in RT_STATES]
            ys = ((fixed[0][0], fixed[1][0]), (fixed[0][1], fixed[1][1]))
            return _rhs_padded(U, gamma, dx, dy, rec, split, RULES[bench], ys, delta=delta)
        if bench == 6:
            ys, xs = ssl_sides(U, gamma, dy, t)
            return _rhs_padded(U, gamma, dx, dy, rec, split, RULES[bench], ys, xs, delta)
        if bench == 5:
            yu, yp, post = dmr_sides(U, gamma, dx, t)
            return _rhs_padded(U, gamma, dx, dy, rec, split, RULES[bench], (yu, yp),
                               ((post[0], None), (post[1], None)), delta)
        return _rhs_padded(U, gamma, dx, dy, rec, split, RULES[bench], delta=delta)
    rho, u, v, p, a = primitives(U, gamma)
    out = torch.zeros_like(U)
    for d, (un, h, axis) in enumerate(((u, dx, 2), (v, dy, 1))):
        if split == 103:
            Fp, Fm = steger_warming(rho, u, v, a, gamma, d)
        else:
            lam = un.abs() + a
            if split == 102:
                lam = lam.max()
            P = torch.stack([torch.zeros_like(p), p if d == 0 else torch.zeros_like(p),
                             p if d == 1 else torch.zeros_like(p), un * p])
            Fp = 0.5 * ((un + lam) * U + P)
            Fm = 0.5 * ((un - lam) * U + P)
        sh = lambda F, k: torch.roll(F, shifts=-k, dims=axis)  # element f holds F[f + k]
        # face f (left of cell f): F+ of cells f-3..f+1, F- of cells f+2..f-2
        hp = _recon([sh(Fp, k) for k in (-3, -2, -1, 0, 1)], rec)
        hm = _recon([sh(Fm, k) for k in (2, 1, 0, -1, -2)], rec)
        hf = hp + hm
        out = out - (sh(hf, 1) - hf) / h
    return out


def roe_eigen(gamma, rl, rr, ul, ur, vl, vr, pl, pr, d):
    """Left and right eigenvectors of the Roe average of two cells (scheme_weno5th_CH.f90:44-62,
    get_l_r_vec_xi/_eta of scheme_weno5th_SC.f90:277-328, 607-658): L[c][k] = l(c+1, k+1) (column
    k the k-th left eigenvector), R[k][e] = r(k+1, e+1) (row k the k-th right eigenvector), as
    nested lists of tensors."""
    hl = pl / (gamma - 1.0) / rl + 0.5 * (ul * ul + vl * vl) + pl / rl
    hr = pr / (gamma - 1.0) / rr + 0.5 * (ur * ur + vr * vr) + pr / rr
    sr, sl = torch.sqrt(rr), torch.sqrt(rl)
    den = sr + sl
    u0 = (sr * ur + sl * ul) / den
    v0 = (sr * vr + sl * vl) / den
    h0 = (sr * hr + sl * hl) / den
    c2 = (gamma - 1.0) * (h0 - 0.5 * (u0 * u0 + v0 * v0))
    a0 = torch.sqrt(c2)
    uu0 = 0.5 * (u0 * u0 + v0 * v0)
    hh0 = a0 * a0 / (gamma - 1.0)
    one, zero = torch.ones_like(u0), torch.zeros_like(u0)
    un = u0 if d == 0 else v0
    if d == 0:
        R = [[one, u0 - a0, v0, h0 - a0 * u0], [one, u0, v0, uu0], [zero, zero, one, v0],
             [one, u0 + a0, v0, h0 + a0 * u0]]
    else:
        R = [[one, u0, v0 - a0, h0 - a0 * v0], [one, u0, v0, uu0], [zero, one, zero, u0],
             [one, u0, v0 + a0, h0 + a0 * v0]]
    hu, nu, ia = 0.5 * uu0 / hh0, 0.5 * un / a0, 0.5 / a0
    pu, pv, ih = 0.5 * u0 / hh0, 0.5 * v0 / hh0, 0.5 / hh0
    L = [[None] * 4 for _ in range(4)]
    if d == 0:
        L[0][0], L[1][0], L[2][0], L[3][0] = hu + nu, -pu - ia, -pv, ih
        L[0][3], L[1][3], L[2][3], L[3][3] = hu - nu, -pu + ia, -pv, ih
        L[0][2], L[1][2], L[2][2], L[3][2] = -v0, zero, one, zero
    else:
        L[0][0], L[1][0], L[2][0], L[3][0] = hu + nu, -pu, -pv - ia, ih
        L[0][3], L[1][3], L[2][3], L[3][3] = hu - nu, -pu, -pv + ia, ih
        L[0][2], L[1][2], L[2][2], L[3][2] = -u0, one, zero, zero
    L[0][1], L[1][1], L[2][1], L[3][1] = -uu0 / hh0 + 1.0, u0 / hh0, v0 / hh0, -1.0 / hh0
    return L, R


def weno5z_weights_theta(f):
    """WENO-Z weights of a 5-point stencil and the AdaWENO indicator theta = 1/(1 + (sum alpha -
    1)^2) (weno5z_stencil_omega_theta, weno_mod.f90:82-95)."""
    f0, f1, f2, f3, f4 = f
    b0 = 13.0 * (f0 - 2.0 * f1 + f2) ** 2 / 12.0 + (f0 - 4.0 * f1 + 3.0 * f2) ** 2 / 4.0
    b1 = 13.0 * (f1 - 2.0 * f2 + f3) ** 2 / 12.0 + (f1 - f3) ** 2 / 4.0
    b2 = 13.0 * (f2 - 2.0 * f3 + f4) ** 2 / 12.0 + (3.0 * f2 - 4.0 * f3 + f4) ** 2 / 4.0
    tau = (b2 - b0).abs()
    a0 = C[0] * (1.0 + (tau / (SS + b0)) ** 2)
    a1 = C[1] * (1.0 + (tau / (SS + b1)) ** 2)
    a2 = C[2] * (1.0 + (tau / (SS + b2)) ** 2)
    s = a0 + a1 + a2
    return (a0 / s, a1 / s, a2 / s), 1.0 / (1.0 + (s - 1.0) ** 2)


def _char_faces(Fp, Fm, Pg, gamma, axis, n, d, delta=None):
    """h at the faces 0..n of the characteristic WENO-Z scheme (104, flux_splitting_CH.f90:24-110,
    scheme_weno5th_CH.f90): per face the Roe eigenvectors of its two cells (padded 3 + f and
    4 + f), each sign's five split fluxes projected on them, WENO-Z per characteristic field, and
    the back-projection. With delta, AdaWENO (105, flux_splitting_SC.f90:141-237,
    scheme_weno5th_SC.f90): per face and sign the indicator theta of the scalar surrogate rho +
    F+-(normal momentum) chooses between the component-wise reconstruction with the surrogate's
    WENO-Z weights (theta > delta, SC.f90:110-124) and the characteristic one."""
    sl = lambda F, k: F.narrow(axis, k, n + 1)
    sp = lambda F, k: F.narrow(axis - 1, k, n + 1)  # one primitive's plane
    r_, u_, v_, p_, _ = Pg
    L, R = roe_eigen(gamma, sp(r_, 3), sp(r_, 4), sp(u_, 3), sp(u_, 4), sp(v_, 3), sp(v_, 4),
                     sp(p_, 3), sp(p_, 4), d)
    h = 0.0
    for F, ks in ((Fp, (1, 2, 3, 4, 5)), (Fm, (6, 5, 4, 3, 2))):
        st = [sl(F, k) for k in ks]  # (4, ...) each
        cv = []
        for k in range(4):
            lf = [L[0][k] * f[0] + L[1][k] * f[1] + L[2][k] * f[2] + L[3][k] * f[3] for f in st]
            cv.append(_recon(lf, 255))
        hc = torch.stack([R[0][q] * cv[0] + R[1][q] * cv[1] + R[2][q] * cv[2] + R[3][q] * cv[3]
                          for q in range(4)])
        if delta is not None:
            sur = [sp(r_, k) + f[1 + d] for k, f in zip(ks, st)]
            (w0, w1, w2), theta = weno5z_weights_theta(sur)
            f0, f1, f2, f3, f4 = st
            q0 = 1.0 / 3.0 * f0 - 7.0 / 6.0 * f1 + 11.0 / 6.0 * f2
            q1 = -1.0 / 6.0 * f1 + 5.0 / 6.0 * f2 + 1.0 / 3.0 * f3
            q2 = 1.0 / 3.0 * f2 + 5.0 / 6.0 * f3 - 1.0 / 6.0 * f4
            hs = w0 * q0 + w1 * q1 + w2 * q2
            hc = torch.where(theta > delta, hs, hc)
        h = h + hc
    return h


def _rhs_padded(U, gamma, dx, dy, rec, split, rules, ys=None, xs=None, delta=None):
    """L(U) on a grid with ghost layers filled by the given rules (bottom, top, left, right);
    ys, xs: the states of the y sides (bottom, top) and x sides (left, right) that need them, as
    ((of the conserved variables), (of the primitives))."""
    rho, u, v, p, a = primitives(U, gamma)
    Pr = torch.stack([rho, u, v, p, a])
    out = torch.zeros_like(U)
    for d, (h, axis) in enumerate(((dx, 2), (dy, 1))):
        lo, hi = (rules[2], rules[3]) if d == 0 else (rules[0], rules[1])
        spec = xs if d == 0 else ys
        Ug = _pad_axis(U, axis, lo, hi, 1 + d, spec[0] if spec else None)
        Pg = _pad_axis(Pr, axis, lo, hi, 1 + d, spec[1] if spec else None)
        r_, u_, v_, p_, a_ = Pg
        un = u_ if d == 0 else v_
        if split in (104, 105):  # GLF split, then the characteristic (or AdaWENO) reconstruction
            lam = ((u if d == 0 else v).abs() + a).max()
            zero = torch.zeros_like(p_)
            P = torch.stack([zero, p_ if d == 0 else zero, p_ if d == 1 else zero, un * p_])
            Fp = 0.5 * ((un + lam) * Ug + P)
            Fm = 0.5 * ((un - lam) * Ug + P)
            n = U.shape[axis]
            hf = _char_faces(Fp, Fm, Pg, gamma, axis, n, d, delta if split == 105 else None)
            out = out - (hf.narrow(axis, 1, n) - hf.narrow(axis, 0, n)) / h
            continue
        if split == 103:
            Fp, Fm = steger_warming(r_, u_, v_, a_, gamma, d)
        else:
            lam = un.abs() + a_
            if split == 102:  # the maximum over the interior cells (get_primary.f90:69-73)
                lam = ((u if d == 0 else v).abs() + a).max()
            zero = torch.zeros_like(p_)
            P = torch.stack([zero, p_ if d == 0 else zero, p_ if d == 1 else zero, un * p_])
            Fp = 0.5 * ((un + lam) * Ug + P)
            Fm = 0.5 * ((un - lam) * Ug + P)
        n = U.shape[axis]
        sl = lambda F, k: F.narrow(axis, k, n + 1)  # padded index k + f for faces f = 0..n
        hp = _recon([sl(Fp, k) for k in (1, 2, 3, 4, 5)], rec)
        hm = _recon([sl(Fm, k) for k in (6, 5, 4, 3, 2)], rec)
        hf = hp + hm
        out = out - (hf.narrow(axis, 1, n) - hf.narrow(axis, 0, n)) / h
    return out


def body_force(U):
    """The Rayleigh-Taylor source (0, 0, rho, rho v) of a state (boundary_rt_general.f90:154-155)."""
    zero = torch.zeros_like(U[0])
    return torch.stack([zero, zero, U[0], U[2]])


def time_step(U, gamma, dx, dy, rec, cfl, dt_const=None, split=101, bench=11, bodyforce=None, t=0.0,
              delta=0.5):
    """One TVD-RK3 step; returns (U_next, dt). The body force (Rayleigh-Taylor, benchmarks 3
    and 13 unless bodyforce says otherwise) is added to each stage after the combine, f_s times
    the source of the stage's input with f_s = dt, dt/4 and 2/3 (single precision) dt
    (time_advance_general.f90:79,160,242)."""
    if bodyforce is None:
        bodyforce = bench in (3, 13)
    if dt_const is None:
        _, u, v, _, a = primitives(U, gamma)
        mx = (u.abs() + a).max()
        my = (v.abs() + a).max()
        dt_x, dt_y = dx / mx, dy / my
        dt = cfl * dt_x * dt_y / (dt_x + dt_y)
    else:
        dt = torch.tensor(dt_const, dtype=U.dtype, device=U.device)
    src = (lambda W, f: f * dt * body_force(W)) if bodyforce else (lambda W, f: 0.0)
    L = lambda W: rhs(W, gamma, dx, dy, rec, split, bench, t, delta)
    u1 = U + dt * L(U) + src(U, 1.0)
    u2 = 3.0 / 4.0 * U + 1.0 / 4.0 * u1 + 1.0 / 4.0 * dt * L(u1) + src(u1, 0.25)
    u3 = 1.0 / 3.0 * U + 2.0 / 3.0 * u2 + 2.0 / 3.0 * dt * L(u2) + src(u2, TWO_THIRDS_SINGLE)
    return u3, dt


def run(U, n, gamma, dx, dy, rec, cfl, dt_const=None, split=101, bench=11, bodyforce=None, delta=0.5):
    # the steps' start times, accumulated as the solver does (general_main.f90:34); a tensor
    # carrying the time steps' dependence on the state (the shear layer's inflow reads it)
    t = 0.0
    for _ in range(n):
        U, dt = time_step(U, gamma, dx, dy, rec, cfl, dt_const, split, bench, bodyforce, t, delta)
        t = t + dt
    return U
