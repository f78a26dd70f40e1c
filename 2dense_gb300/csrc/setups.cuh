// setups.cuh — initial states computed on the device for the variant benchmarks that the
// batched and differentiable workloads generate in bulk (11 translating vortex, 13 Rayleigh-Taylor
// with reflective walls, 14 periodic Richtmyer-Meshkov), and the exact solution of the
// translating vortex. Same formulas as dense_init_setup (csrc/host_setup.cpp), with CUDA's pow,
// exp, cos and sqrt: within a few ulp of the host setup, not bit-identical to it.
#pragma once
#include "internal.h"

namespace dense {
namespace setups {

constexpr double kPi = 3.141592653589793;

// Arithmetic with explicit rounding (no FMA contraction), so that every kernel that inlines these
// setups -- the single-block and the batched one, compiled in different units -- gives the same
// bits.
__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double D(double a, double b) { return __ddiv_rn(a, b); }

// (rho, u, v, p) of benchmark `bench` at the cell centre / vertex (x, y); false if the
// benchmark has no device setup
__device__ __forceinline__ bool state_at(int bench, double gamma, double eps, double xc, double yc, double amp,
                                         double x, double y, double& rho, double& u, double& v, double& p) {
    switch (bench) {
    case DENSE_BENCH_IVC_PERIODIC: {  // vortex over the stream (1, 1, 1, 1)
        const double ddx = S(x, xc), ddy = S(y, yc);
        const double r2 = A(M(ddx, ddx), M(ddy, ddy));
        const double g1 = S(gamma, 1.0);
        rho = pow(S(1.0, D(M(M(g1, M(eps, eps)), exp(S(1.0, r2))), M(M(8.0, gamma), M(kPi, kPi)))), D(1.0, g1));
        const double f = M(D(eps, M(2.0, kPi)), exp(D(S(1.0, r2), 2.0)));
        u = S(1.0, M(f, ddy));
        v = A(1.0, M(f, ddx));
        p = pow(rho, gamma);
        return true;
    }
    case DENSE_BENCH_RT_REFLECT: {  // init_RT_general.f90:1-67 (the upper half's default-real 0.025)
        u = 0.0;
        const double c8 = cos(M(M(8.0, kPi), x));
        if (y <= 0.5) {
            rho = 2.0; p = A(M(2.0, y), 1.0);
            v = M(M(-0.025, sqrt(D(M(gamma, p), rho))), c8);
        } else {
            rho = 1.0; p = A(y, 1.5);
            v = M(M(-(double)0.025f, sqrt(D(M(gamma, p), rho))), c8);
        }
        return true;
    }
    case DENSE_BENCH_RM_PERIODIC: {  // Mach 1.2 shock into a density-3 interface of amplitude amp
        const double Ma = 1.2, g = gamma, M2 = M(Ma, Ma);
        const double rho2 = D(M(A(g, 1.0), M2), A(M(S(g, 1.0), M2), 2.0));
        const double p2 = A(1.0, M(D(M(2.0, g), A(g, 1.0)), S(M2, 1.0)));
        const double u2 = M(M(Ma, sqrt(g)), S(1.0, D(1.0, rho2)));
        const double xi_if = A(0.5, M(amp, cos(M(M(2.0, kPi), y))));
        v = 0.0;
        if (x < 0.2) { rho = rho2; u = u2; p = p2; }
        else if (x < xi_if) { rho = 1.0; u = 0.0; p = 1.0; }
        else { rho = 3.0; u = 0.0; p = 1.0; }
        return true;
    }
    default:
        return false;
    }
}

// Cell (i, j) (0-based interior) coordinates: cell centres, except the vertex grid of RT.
__device__ __forceinline__ void coords(int bench, int i, int j, double dx, double dy, double& x, double& y) {
    if (bench == DENSE_BENCH_RT_REFLECT) { x = M(i, dx); y = M(j, dy); }
    else { x = M(A(i, 0.5), dx); y = M(A(j, 0.5), dy); }
}

// Fill interior cell (i, j) of a block: cons and prim as the setups' per-cell assignment.
__device__ __forceinline__ void init_cell(const Params& p, double eps, double xc, double yc, double amp, int i,
                                          int j) {
    double x, y, rho, u, v, pr;
    coords(p.benchmark, i, j, p.dx, p.dy, x, y);
    if (!state_at(p.benchmark, p.gamma, eps, xc, yc, amp, x, y, rho, u, v, pr)) return;
    const long long o = (long long)(j + kB) * p.P + (i + kB);
    p.cons[o] = rho;
    p.cons[p.plane + o] = M(rho, u);
    p.cons[2 * p.plane + o] = M(rho, v);
    p.cons[3 * p.plane + o] = A(D(pr, S(p.gamma, 1.0)), M(M(0.5, rho), A(M(u, u), M(v, v))));
    p.prim[o] = rho;
    p.prim[p.plane + o] = u;
    p.prim[2 * p.plane + o] = v;
    p.prim[3 * p.plane + o] = pr;
    p.prim[4 * p.plane + o] = sqrt(D(M(p.gamma, pr), rho));
}

}  // namespace setups
}  // namespace dense
