// kernels.cu — sm_103a kernels of 2DENSE's per-stage hot path.
//
// This file is compiled three times into the same library:
//   -DDENSE_VARIANT_STRICT=1 -fmad=false : dense::kernels_strict(). Every expression keeps the
//      reference's evaluation order (left to right as written in the Fortran), no FMA is
//      contracted and divide/sqrt are IEEE, so results are bit-identical to the reference's
//      x86-64 arithmetic (except the SSL inflow rule, which calls tanh/cos/exp).
//   -DDENSE_VARIANT_STRICT=0             : dense::kernels_fast(). FMA contraction and the
//      algebraic rewrites marked FAST below; agrees with the reference to ~1e-14 per step.
//   -DDENSE_VARIANT_STRICT=0 -DDENSE_CHECK=1 : dense::kernels_checked(), the debug build of the
//      fast variant: every index into a state, face, tape or shared-memory array is checked
//      against its array (chk below); one outside sets DENSE_FLAG_BOUNDS in the status word and
//      is clamped into the array, so a bad index is reported, never dereferenced.
//
// All arithmetic is FP64. On GB300 the FP64 pipe, not HBM, bounds every kernel here (about
// 4-7 kFLOP per cell-update against 256 B of compulsory traffic), so the kernels are built to
// minimise FP64 instructions: per-cell split fluxes are computed once per tile into shared
// memory, Roe averages and eigenvectors once per interface for both signs, and loop-invariant
// scalars (dt/dx, dt/dy, the GLF wave speed) once per stage.
//
// Layout in HBM (0-based, padded with 4 ghost layers; I = i + 4, J = j + 4 for interior (i,j)):
//   cons[v][J][I]  v = 0..3 (rho, rho u, rho v, E)       row pitch P doubles, plane NJp*P
//   prim[v][J][I]  v = 0..4 (rho, u, v, p, alpha)
//   hx[v][j][f]    f = 0..ni interface between padded columns f+3 and f+4
//   he[v][g][i]    g = 0..nj interface between padded rows g+3 and g+4
#include <cuda_runtime.h>

#include "fastmath.cuh"
#include "internal.h"

#ifndef DENSE_VARIANT_STRICT
#error "DENSE_VARIANT_STRICT must be defined (0 or 1)"
#endif
#ifndef DENSE_CHECK
#define DENSE_CHECK 0
#endif
#if DENSE_VARIANT_STRICT
#define VNS strict_impl
#define FAST 0
#elif DENSE_CHECK
#define VNS checked_impl
#define FAST 1
#else
#define VNS fast_impl
#define FAST 1
#endif

namespace dense {
namespace VNS {

// Index x of an array of n elements. The checked variant flags and clamps one outside [0, n);
// the others compile the test away.
template <class T>
__device__ __forceinline__ T chk(const Params& p, T x, T n) {
#if DENSE_CHECK
    if (x < 0 || x >= n) {
        atomicOr(&p.sc->status, DENSE_FLAG_BOUNDS);
        return x < 0 ? 0 : n - 1;
    }
#else
    (void)p; (void)n;
#endif
    return x;
}

// ---------------------------------------------------------------------------------------------
// weno module constants (source/inv_scheme/weno_mod.f90:3-14,37) and the fast WENO terms
#include "weno_fast.cuh"
constexpr double kPFloor = (double)1.0e-6f;   // get_primary.f90:58
constexpr double kTwoThirdsSP = (double)(2.0f / 3.0f);  // time_advance_general.f90:242

__device__ __forceinline__ double sq(double x) { return x * x; }

// Smoothness indicators of the three 3-point substencils (weno_mod.f90:152-159).
__device__ __forceinline__ void smoothness(const double lf[5], double& is0, double& is1, double& is2) {
    is0 = 13.0 * sq(lf[0] - 2.0 * lf[1] + lf[2]) / 12.0 + sq(lf[0] - 4.0 * lf[1] + 3.0 * lf[2]) / 4.0;
    is1 = 13.0 * sq(lf[1] - 2.0 * lf[2] + lf[3]) / 12.0 + sq(lf[1] - lf[3]) / 4.0;
    is2 = 13.0 * sq(lf[2] - 2.0 * lf[3] + lf[4]) / 12.0 + sq(3.0 * lf[2] - 4.0 * lf[3] + lf[4]) / 4.0;
}

// Third-order candidates (weno_mod.f90:57-59).
__device__ __forceinline__ void candidates(const double lf[5], double& q0, double& q1, double& q2) {
    q0 = a300 * lf[0] + a301 * lf[1] + a302 * lf[2];
    q1 = a310 * lf[1] + a311 * lf[2] + a312 * lf[3];
    q2 = a320 * lf[2] + a321 * lf[3] + a322 * lf[4];
}

// WENO-JS5 (weno5js_stencil + _omega_only + _alpha, weno_mod.f90:98-165)
__device__ __forceinline__ double weno5js(const double lf[5]) {
    double q0, q1, q2, is0, is1, is2;
    candidates(lf, q0, q1, q2);
    smoothness(lf, is0, is1, is2);
    double a0 = c30 / sq(kSS + is0);
    double a1 = c31 / sq(kSS + is1);
    double a2 = c32 / sq(kSS + is2);
    double s = a0 + a1 + a2;
    double w0 = a0 / s, w1 = a1 / s, w2 = a2 / s;
    return w0 * q0 + w1 * q1 + w2 * q2;
}

// WENO-Z alpha (weno5z_stencil_alpha, weno_mod.f90:168-189)
__device__ __forceinline__ void weno5z_alpha(const double lf[5], double& a0, double& a1, double& a2) {
    double is0, is1, is2;
    smoothness(lf, is0, is1, is2);
    double tau5 = fabs(is2 - is0);
    a0 = c30 * (1.0 + sq(tau5 / (kSS + is0)));
    a1 = c31 * (1.0 + sq(tau5 / (kSS + is1)));
    a2 = c32 * (1.0 + sq(tau5 / (kSS + is2)));
}

// WENO-Z5 (weno5z_stencil + _omega_only, weno_mod.f90:50-79)
__device__ __forceinline__ double weno5z(const double lf[5]) {
    double q0, q1, q2, a0, a1, a2;
    candidates(lf, q0, q1, q2);
    weno5z_alpha(lf, a0, a1, a2);
    double s = a0 + a1 + a2;
    double w0 = a0 / s, w1 = a1 / s, w2 = a2 / s;
    return w0 * q0 + w1 * q1 + w2 * q2;
}

// weno5z_stencil_omega_theta (weno_mod.f90:82-95)
__device__ __forceinline__ void weno5z_omega_theta(const double lf[5], double& w0, double& w1,
                                                   double& w2, double& theta) {
    double a0, a1, a2;
    weno5z_alpha(lf, a0, a1, a2);
    double s = a0 + a1 + a2;
    w0 = a0 / s; w1 = a1 / s; w2 = a2 / s;
    theta = 1.0 / (1.0 + sq(s - 1.0));
}

// upwind5 (scheme_upwind5_general.f90:86-90)
__device__ __forceinline__ double upwind5(const double lf[5]) {
    return (2.0 * lf[0] - 13.0 * lf[1] + 47.0 * lf[2] + 27.0 * lf[3] - 3.0 * lf[4]) / 60.0;
}

// ---------------------------------------------------------------------------------------------
// FAST arithmetic. On GB300 an IEEE double divide costs about ten FMA slots of the FP64 pipe,
// and the reference's WENO weights spend seven divides per stencil. The fast variant
//  * takes reciprocals and inverse square roots from the hardware seeds (rcp.approx.ftz.f64,
//    rsqrt.approx.ftz.f64) refined by one third-order step each (with e = 1 - d r, 1/d =
//    r (1 + e + e^2 + ...); with e = 1 - x y^2, 1/sqrt(x) = y (1 + e/2 + 3e^2/8 + ...)), which
//    lands within 2 ulp of the correctly rounded result for the positive normal arguments
//    used here;
//  * writes the WENO weights over a common denominator: with d_k = ss + beta_k,
//    P_k = prod_{j != k} d_j^2 and D = prod_j d_j^2,
//      WENO-JS: alpha_k D = c_k P_k,   WENO-Z: alpha_k D = c_k (D + tau^2 P_k),
//    so h = sum(alpha_k D q_k) / sum(alpha_k D) costs one reciprocal instead of six divides,
//    and the AdaWENO test theta > delta becomes sqrt(1-delta) D > sqrt(delta) (N - D) with
//    N = sum alpha_k D (theta = 1/(1+(sum alpha - 1)^2)), which needs no divide at all.
// Products of squared d_k stay far inside the double range for d_k in [1e-6, 1e40].
// (rcp_nr and rsqrt_nr: fastmath.cuh)


// WENO reconstruction of a stencil no other interface shares (the characteristic fields).
template <bool Z> __device__ __forceinline__ double weno_fast(const double lf[5]) {
    double g[4], d0, d1, d2;
    first_differences(lf, g);
    betas_g(g, d0, d1, d2);
    return weno_from_d<Z>(lf[2], g, d0, d1, d2);
}

// Second-difference term of a smoothness indicator, s = 4 ss + 13/3 A^2 (four times ss + 13/12
// A^2) with A = lm - 2 lc + lr: it depends on one cell and its two neighbours only, so a sweep
// computes it once per cell and sign and each of the three interfaces that use it reads it (the
// "-" sign passes its neighbours in mirrored order, as its stencil reads them).
__device__ __forceinline__ double ind_second(double lm, double lc, double lr) {
    const double a = fma(-2.0, lc, lm) + lr;
    return fma(k133 * a, a, 4.0 * kSS);
}

// The five coefficients of h = sum_k w_k q_k as one 5-point stencil: W[m] lf[m].
__device__ __forceinline__ void stencil_from_weights(double w0, double w1, double w2, double W[5]) {
    W[0] = w0 * a300;
    W[1] = fma(w1, a310, w0 * a301);
    W[2] = fma(w2, a320, fma(w1, a311, w0 * a302));
    W[3] = fma(w2, a321, w1 * a312);
    W[4] = w2 * a322;
}

// The same 5-point stencil from u0 = w0/c0 and u2 = w2/c2 of WENO-Z weights that sum to one
// (w1 = 1 - w0 - w2): the linear weights c_k and the candidates' coefficients fold into constants.
__device__ __forceinline__ void stencil_from_u(double u0, double u2, double W[5]) {
    W[0] = (c30 * a300) * u0;
    W[1] = fma(c30 * (a301 - a310), u0, fma(-c32 * a310, u2, a310));
    W[2] = fma(c30 * (a302 - a311), u0, fma(c32 * (a320 - a311), u2, a311));
    W[3] = fma(-c30 * a312, u0, fma(c32 * (a321 - a312), u2, a312));
    W[4] = (c32 * a322) * u2;
}

// The gradient of a stencil's reconstruction alone (upwind5's is constant), its terms recomputed.
template <int REC>
__device__ __forceinline__ void recon_grad(const double lf[5], double g[5]) {
    if (REC == DENSE_RECON_UPWIND5) {
        g[0] = 2.0 / 60.0; g[1] = -13.0 / 60.0; g[2] = 47.0 / 60.0; g[3] = 27.0 / 60.0; g[4] = -3.0 / 60.0;
        return;
    }
    constexpr bool Z = REC == DENSE_RECON_WENOZ5;
    double gd[4], d0, d1, d2;
    first_differences(lf, gd);
    betas_g(gd, d0, d1, d2);
    const double B[3] = {fma(-3.0, gd[1], gd[0]), gd[1] + gd[2], fma(3.0, gd[2], -gd[3])};
    WenoTerms t;
    weno_terms<Z>(gd, d0, d1, d2, t);
    const double iN = rcp_nr(t.N);
    weno_grad<Z>(gd, B, d0, d1, d2, t, weno_num(t) * iN, iN, g);
}

template <int REC> __device__ __forceinline__ double recon5(const double lf[5]) {
    if (REC == DENSE_RECON_UPWIND5) return upwind5(lf);
#if FAST
    return weno_fast<REC == DENSE_RECON_WENOZ5>(lf);
#else
    if (REC == DENSE_RECON_WENOJS5) return weno5js(lf);
    return weno5z(lf);
#endif
}

// ---------------------------------------------------------------------------------------------
// Flux-vector splittings at one cell. DIR 0 = xi (normal velocity u, momentum component 1),
// DIR 1 = eta (normal velocity v, momentum component 2).

// Lax-Friedrichs family (flux_splitting_LLF.f90:73-81 / :98-106, GLF, CH, SC):
// F+- = 0.5*((un +- lam)*U + (0, p e_n, u_n p))
template <int DIR>
__device__ __forceinline__ void lf_split(const double U[4], double un, double p, double lam,
                                         double fp[4], double fm[4]) {
#if FAST
    // F+- = (u_n U + P)/2 +- (lam/2) U, P = (0, p e_n, u_n p): 16 operations instead of 19.
    // The prim u_n and the conserved U stay separate factors as in the reference: in an
    // extrapolated ghost cell m_n is not rho u_n.
    const double hu = 0.5 * un, hl = 0.5 * lam;
    double G[4];
    G[0] = hu * U[0];
    if (DIR == 0) { G[1] = fma(hu, U[1], 0.5 * p); G[2] = hu * U[2]; }
    else          { G[1] = hu * U[1]; G[2] = fma(hu, U[2], 0.5 * p); }
    G[3] = fma(hu, U[3], hu * p);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        fp[c] = fma(hl, U[c], G[c]);
        fm[c] = fma(-hl, U[c], G[c]);
    }
#else
    const double up = un + lam, um = un - lam, upp = un * p;
    fp[0] = 0.5 * (up * U[0]);
    fm[0] = 0.5 * (um * U[0]);
    if (DIR == 0) {
        fp[1] = 0.5 * (up * U[1] + p); fp[2] = 0.5 * (up * U[2]);
        fm[1] = 0.5 * (um * U[1] + p); fm[2] = 0.5 * (um * U[2]);
    } else {
        fp[1] = 0.5 * (up * U[1]); fp[2] = 0.5 * (up * U[2] + p);
        fm[1] = 0.5 * (um * U[1]); fm[2] = 0.5 * (um * U[2] + p);
    }
    fp[3] = 0.5 * (up * U[3] + upp);
    fm[3] = 0.5 * (um * U[3] + upp);
#endif
}

// Steger-Warming (flux_splitting_SW.f90:42-91 xi, :110-160 eta)
template <int DIR>
__device__ __forceinline__ void sw_split(double rho, double u, double v, double alpha, double gamma,
                                         double fp[4], double fm[4]) {
    const double epsl2 = 0.125 * 0.125;
    const double g1 = gamma - 1.0, two_g1 = 2.0 * (gamma - 1.0), two_g = 2.0 * gamma;
    const double uu2 = u * u + v * v;
    const double un = DIR == 0 ? u : v, ut = DIR == 0 ? v : u;
    const double l1 = un, l2 = un - alpha, l3 = un + alpha;
    const double s1 = sqrt(l1 * l1 + epsl2), s2 = sqrt(l2 * l2 + epsl2), s3 = sqrt(l3 * l3 + epsl2);
    const double a2 = alpha * alpha;
    const double q2 = l2 * l2 + ut * ut, q3 = l3 * l3 + ut * ut;
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
        const double lp1 = sgn == 0 ? (l1 + s1) / 2.0 : (l1 - s1) / 2.0;
        const double lp2 = sgn == 0 ? (l2 + s2) / 2.0 : (l2 - s2) / 2.0;
        const double lp3 = sgn == 0 ? (l3 + s3) / 2.0 : (l3 - s3) / 2.0;
        double* f = sgn == 0 ? fp : fm;
        const double wii = (3.0 - gamma) * (lp2 + lp3) * a2 / two_g1;
        const double A = lp1 * 2.0 * g1;
        f[0] = (A + lp2 + lp3) * rho / two_g;
        const double fn = (A * un + lp2 * l2 + lp3 * l3) * rho / two_g;
        const double ft = (A * ut + lp2 * ut + lp3 * ut) * rho / two_g;
        f[1 + DIR] = fn;
        f[2 - DIR] = ft;
        f[3] = (lp1 * g1 * uu2 + lp2 * 0.5 * q2 + lp3 * 0.5 * q3 + wii) * rho / two_g;
    }
}

// ---------------------------------------------------------------------------------------------
// Roe average (scheme_weno5th_CH.f90:44-62) and eigenvectors (get_l_r_vec_xi/_eta,
// scheme_weno5th_SC.f90:277-328, 607-658). L[c][k] = l(c+1,k+1): column k is the k-th left
// eigenvector; R[k][e] = r(k+1,e+1): row k is the k-th right eigenvector.
struct Eig {
    double L[4][4];
    double R[4][4];
};

__device__ __forceinline__ bool roe_eig(int dir, double gamma, double rhol, double rhor, double ul,
                                        double ur, double vl, double vr, double pl, double pr, Eig& e) {
    const double hl = pl / (gamma - 1.0) / rhol + 0.5 * (ul * ul + vl * vl) + pl / rhol;
    const double hr = pr / (gamma - 1.0) / rhor + 0.5 * (ur * ur + vr * vr) + pr / rhor;
    const double sr = sqrt(rhor), sl = sqrt(rhol), den = sr + sl;
    const double u0 = (sr * ur + sl * ul) / den;
    const double v0 = (sr * vr + sl * vl) / den;
    const double h0 = (sr * hr + sl * hl) / den;
    const double c2 = (gamma - 1.0) * (h0 - 0.5 * (u0 * u0 + v0 * v0));
    const double a0 = sqrt(c2);
    const double uu0 = 0.5 * (u0 * u0 + v0 * v0);
    const double hh0 = a0 * a0 / (gamma - 1.0);
    const double un = dir == 0 ? u0 : v0;
    e.R[0][0] = 1.0; e.R[1][0] = 1.0; e.R[2][0] = 0.0; e.R[3][0] = 1.0;
    if (dir == 0) {
        e.R[0][1] = u0 - a0; e.R[1][1] = u0; e.R[2][1] = 0.0; e.R[3][1] = u0 + a0;
        e.R[0][2] = v0; e.R[1][2] = v0; e.R[2][2] = 1.0; e.R[3][2] = v0;
        e.R[0][3] = h0 - a0 * u0; e.R[1][3] = uu0; e.R[2][3] = v0; e.R[3][3] = h0 + a0 * u0;
    } else {
        e.R[0][1] = u0; e.R[1][1] = u0; e.R[2][1] = 1.0; e.R[3][1] = u0;
        e.R[0][2] = v0 - a0; e.R[1][2] = v0; e.R[2][2] = 0.0; e.R[3][2] = v0 + a0;
        e.R[0][3] = h0 - a0 * v0; e.R[1][3] = uu0; e.R[2][3] = u0; e.R[3][3] = h0 + a0 * v0;
    }
    const double hu = 0.5 * uu0 / hh0, nu = 0.5 * un / a0, ia = 0.5 / a0;
    const double pu = 0.5 * u0 / hh0, pv = 0.5 * v0 / hh0, ih = 0.5 / hh0;
    if (dir == 0) {
        e.L[0][0] = hu + nu; e.L[1][0] = -pu - ia; e.L[2][0] = -pv; e.L[3][0] = ih;
        e.L[0][3] = hu - nu; e.L[1][3] = -pu + ia; e.L[2][3] = -pv; e.L[3][3] = ih;
        e.L[0][2] = -v0; e.L[1][2] = 0.0; e.L[2][2] = 1.0; e.L[3][2] = 0.0;
    } else {
        e.L[0][0] = hu + nu; e.L[1][0] = -pu; e.L[2][0] = -pv - ia; e.L[3][0] = ih;
        e.L[0][3] = hu - nu; e.L[1][3] = -pu; e.L[2][3] = -pv + ia; e.L[3][3] = ih;
        e.L[0][2] = -u0; e.L[1][2] = 1.0; e.L[2][2] = 0.0; e.L[3][2] = 0.0;
    }
    e.L[0][1] = -uu0 / hh0 + 1.0; e.L[1][1] = u0 / hh0; e.L[2][1] = v0 / hh0; e.L[3][1] = -1.0 / hh0;
    return !(c2 < 0.0);
}

// Characteristic-wise WENO-Z at one interface and one sign (scheme_weno5th_CH.f90:66-81).
// F[m][c]: split flux of component c at stencil point m (m = 0..4 <-> -2..2).
__device__ __forceinline__ void char_weno(const Eig& e, const double F[5][4], double h[4]) {
    double cv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double lf[5];
#pragma unroll
        for (int m = 0; m < 5; ++m)
            lf[m] = e.L[0][k] * F[m][0] + e.L[1][k] * F[m][1] + e.L[2][k] * F[m][2] + e.L[3][k] * F[m][3];
        cv[k] = weno5z(lf);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        h[q] = e.R[0][q] * cv[0] + e.R[1][q] * cv[1] + e.R[2][q] * cv[2] + e.R[3][q] * cv[3];
}

// FAST characteristic machinery. The Roe state of the two cells next to an interface from
// their sqrt(rho) and total enthalpy H = gamma/(gamma-1) p/rho + |u|^2/2 (staged once per cell),
// with one reciprocal for the three weighted means and one inverse square root giving both
// alpha0 and 1/alpha0; 1/hh0 = (gamma-1)/alpha0^2. The eigenvector products use the zero and
// unit entries of the matrices of get_l_r_vec_xi/_eta (scheme_weno5th_SC.f90:277-328, 607-658):
// the tangential-shear characteristic is F_t - u_t0 F_0, and the back-projection is
//   h_0 = c0 + c1 + c3,  h_n = u_n0 h_0 + a0 (c3 - c0),  h_t = u_t0 h_0 + c2,
//   h_3 = H0 (c0 + c3) + a0 u_n0 (c3 - c0) + uu0 c1 + u_t0 c2,
// with n the normal and t the tangential momentum component.
struct EigFast {
    double un0, ut0, a0, h0, uu0, a0un0;
    double l00, l10, l20, l30;  // column 0 (acoustic, u_n - a)
    double l01, l11, l21, l31;  // column 1 (entropy)
    double l03, l13, l23;       // column 3 (acoustic, u_n + a); l33 == l30
};

template <int DIR>
__device__ __forceinline__ bool roe_eig_fast(double g1, double sl, double sr, double ul, double ur,
                                             double vl, double vr, double hl, double hr, EigFast& e) {
    const double r = rcp_nr(sl + sr);
    const double u0 = fma(sr, ur, sl * ul) * r;
    const double v0 = fma(sr, vr, sl * vl) * r;
    const double h0 = fma(sr, hr, sl * hl) * r;
    const double uu0 = 0.5 * fma(u0, u0, v0 * v0);
    const double c2 = g1 * (h0 - uu0);
    const double ia = rsqrt_nr(c2);
    const double a0 = c2 * ia;
    const double ihh = g1 * ia * ia;
    const double un0 = DIR == 0 ? u0 : v0, ut0 = DIR == 0 ? v0 : u0;
    e.un0 = un0; e.ut0 = ut0; e.a0 = a0; e.h0 = h0; e.uu0 = uu0; e.a0un0 = a0 * un0;
    const double hu = 0.5 * uu0 * ihh, nu = 0.5 * un0 * ia, ia5 = 0.5 * ia;
    const double pn = 0.5 * un0 * ihh, pt = 0.5 * ut0 * ihh, ih = 0.5 * ihh;
    // rows of the normal (n) and tangential (t) momentum components
    const double ln0 = -pn - ia5, ln3 = -pn + ia5;
    if (DIR == 0) {
        e.l00 = hu + nu; e.l10 = ln0; e.l20 = -pt;
        e.l03 = hu - nu; e.l13 = ln3; e.l23 = -pt;
    } else {
        e.l00 = hu + nu; e.l10 = -pt; e.l20 = ln0;
        e.l03 = hu - nu; e.l13 = -pt; e.l23 = ln3;
    }
    e.l30 = ih;
    e.l01 = fma(-uu0, ihh, 1.0); e.l11 = u0 * ihh; e.l21 = v0 * ihh; e.l31 = -ihh;
    return c2 > 0.0;
}

// Characteristic-wise WENO-Z at one interface and one sign from the stencil's centre split flux
// Fc and its first differences dF[m] = F[m] - F[m+1] (m = 0..3): the projection is linear, so the
// characteristic fields' first differences are the projected differences, and each field's
// reconstruction works from them directly (weno_from_d).
template <int DIR>
__device__ __forceinline__ void char_weno_fast_g(const EigFast& e, const double Fc[4], const double dF[4][4],
                                                 double h[4]) {
    auto proj = [&](const double f[4], double l[4]) {
        l[0] = fma(e.l00, f[0], fma(e.l10, f[1], fma(e.l20, f[2], e.l30 * f[3])));
        l[1] = fma(e.l01, f[0], fma(e.l11, f[1], fma(e.l21, f[2], e.l31 * f[3])));
        l[2] = fma(-e.ut0, f[0], DIR == 0 ? f[2] : f[1]);
        l[3] = fma(e.l03, f[0], fma(e.l13, f[1], fma(e.l23, f[2], e.l30 * f[3])));
    };
    double lc[4], gd[4][4];
    proj(Fc, lc);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        double l[4];
        proj(dF[m], l);
#pragma unroll
        for (int k = 0; k < 4; ++k) gd[k][m] = l[k];
    }
    double c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double d0, d1, d2;
        betas_g(gd[k], d0, d1, d2);
        c[k] = weno_from_d<true>(lc[k], gd[k], d0, d1, d2);
    }
    const double s = c[0] + c[1] + c[3], d = c[3] - c[0];
    const double hn = fma(e.un0, s, e.a0 * d);
    const double ht = fma(e.ut0, s, c[2]);
    h[0] = s;
    h[1 + DIR] = hn;
    h[2 - DIR] = ht;
    h[3] = fma(e.h0, c[0] + c[3], fma(e.a0un0, d, fma(e.uu0, c[1], e.ut0 * c[2])));
}
// The same from the stencil's five split fluxes F[m][c].
template <int DIR>
__device__ __forceinline__ void char_weno_fast(const EigFast& e, const double F[5][4], double h[4]) {
    double dF[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int c = 0; c < 4; ++c) dF[m][c] = F[m][c] - F[m + 1][c];
    char_weno_fast_g<DIR>(e, F[2], dF, h);
}

// ---------------------------------------------------------------------------------------------
// Index helpers
__device__ __forceinline__ long long cidx(const Params& p, int I, int J) {
    return (long long)chk(p, J, p.nj + 2 * kB) * p.P + chk(p, I, p.P);
}
// Face f of line `line` in plane v of direction DIR's face array (xi [nj][ni+1], eta [nj+1][ni]).
template <int DIR>
__device__ __forceinline__ long long fidx(const Params& p, int v, int line, int f) {
    if (DIR == 0) return (long long)v * p.nj * (p.ni + 1) + (long long)chk(p, line, p.nj) * (p.ni + 1) + chk(p, f, p.ni + 1);
    return (long long)v * (p.nj + 1) * p.ni + (long long)chk(p, f, p.nj + 1) * p.ni + chk(p, line, p.ni);
}

// Per-stage scalar work, done by one thread before the sweeps read or the update uses them:
// the CFL time step (time_advance_general.f90:20-24), dt/dx, dt/dy, and the reset of the max
// slot that this stage's update fills for the next stage.
__device__ __forceinline__ void stage_scalars(const Params& p, int irk) {
    Scalars* sc = p.sc;
    const int slot = irk - 1;
    if (irk == 1 && !p.if_const_dt) {
        const double dt_xi = p.dx / sc->maxeig[slot][0];
        const double dt_eta = p.dy / sc->maxeig[slot][1];
        sc->dt = p.cfl * dt_xi * dt_eta / (dt_xi + dt_eta);
    }
    sc->dtdx = sc->dt / p.dx;
    sc->dtdy = sc->dt / p.dy;
    const int next = irk % 3;
    sc->maxeig[next][0] = 0.0;
    sc->maxeig[next][1] = 0.0;
}

// ---------------------------------------------------------------------------------------------
// Component-wise flux kernel (splittings 101/102/103 with reconstructions 251/253/255).
// One thread per interface; the tile's per-cell split fluxes are staged in shared memory.
// xi tile: TX interfaces x TY rows, cells f0+1 .. f0+TX+5; eta tile: TX columns x TY interfaces.
// Dynamic shared memory of one block, in doubles: the split fluxes sF[8][NL][NC] (F+ of the four
// components, then F-) and, for the WENO reconstructions of the fast variant, the indicators'
// second-difference terms sS[8][NL][NC] and the forward differences sG[8][NL][NC] = F(k) - F(k+1)
// along the sweep of the same cells (F+ then F-): a cell's terms serve up to four interfaces.
template <int DIR, int REC, int TX, int TY>
struct CwTile {
    static constexpr int NL = DIR == 0 ? TY : TY + 5;   // smem rows
    static constexpr int NC = DIR == 0 ? TX + 5 : TX;   // smem columns
    static constexpr int NCELL = NL * NC;
    static constexpr bool kStageS = FAST && REC != DENSE_RECON_UPWIND5;
    static constexpr size_t bytes = sizeof(double) * (size_t)NCELL * (kStageS ? 24 : 8);
};

// TZ threads share an interface (threadIdx.z): they stage the tile's cells together and each
// reconstructs the components tz, tz + TZ, ...; the arithmetic of every component is the same
// whatever TZ, so the results do not depend on it.
template <int DIR, int SPL, int REC, int TX, int TY, bool TAPE = false, int TZ = 1>
__device__ __forceinline__ void flux_cw_block(const Params& p, int irk, int bx, int by) {
    static_assert(TZ == 1 || TZ == 2 || TZ == 4, "TZ divides the four components");
    if (!p.sc->active) return;
    using L = CwTile<DIR, REC, TX, TY>;
    constexpr int NL = L::NL, NC = L::NC, NCELL = L::NCELL;
    constexpr bool kStageS = L::kStageS;
    extern __shared__ __align__(16) double dsm[];
    double* const sF = dsm;
    double* const sS = dsm + 8 * NCELL;
    double* const sG = dsm + 16 * NCELL;
    (void)sS; (void)sG; (void)NL;
    auto at = [&](int r, int c) { return chk(p, r, NL) * NC + chk(p, c, NC); };
    // the thread's place in the tile from its linear index (a TX x TY x TZ block, or the
    // persistent kernel's one-dimensional block of as many threads)
    const int lt = threadIdx.x + TX * (threadIdx.y + TY * threadIdx.z);
    const int tx = lt % TX, ty = (lt / TX) % TY, tz = TZ == 1 ? 0 : lt / (TX * TY);
    const int slot = irk - 1;
    if (DIR == 0 && bx == 0 && by == 0 && lt == 0) stage_scalars(p, irk);
    const double lam_g = p.sc->maxeig[slot][DIR];
    const int NIp = p.ni + 2 * kB, NJp = p.nj + 2 * kB;

    // phase 1: split fluxes of the tile's cells
    auto cell = [&](int I, int J, int r, int c) {
        const long long o = cidx(p, I, J);
        double U[4], fp[4], fm[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = p.cons[v * p.plane + o];
        if (SPL == 0) {
            const double un = p.prim[(1 + DIR) * p.plane + o];
            const double pr = p.prim[3 * p.plane + o];
            const double lam = p.splitting == DENSE_SPLIT_LLF ? fabs(un) + p.prim[4 * p.plane + o] : lam_g;
            lf_split<DIR>(U, un, pr, lam, fp, fm);
        } else {
            sw_split<DIR>(p.prim[o], p.prim[p.plane + o], p.prim[2 * p.plane + o], p.prim[4 * p.plane + o],
                          p.gamma, fp, fm);
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) { sF[v * NCELL + at(r, c)] = fp[v]; sF[(4 + v) * NCELL + at(r, c)] = fm[v]; }
    };
    if (DIR == 0) {
        const int f0 = bx * TX, j = by * TY + ty;
        if (j < p.nj)
            for (int k = tx + TX * tz; k < TX + 5; k += TX * TZ) {
                const int I = f0 + 1 + k;
                if (I < NIp) cell(I, j + kB, ty, k);
            }
    } else {
        const int g0 = by * TY, i = bx * TX + tx;
        if (i < p.ni)
            for (int k = ty + TY * tz; k < TY + 5; k += TY * TZ) {
                const int J = g0 + 1 + k;
                if (J < NJp) cell(i + kB, J, k, tx);
            }
    }
    __syncthreads();

    // phase 1b (fast WENO): the indicators' second-difference terms, once per cell and sign for
    // the cells with both neighbours in the tile ("+" reads a cell's neighbours as k-1, k, k+1,
    // "-" as k+1, k, k-1), and the forward differences of the cells with a next neighbour
    if constexpr (kStageS) {
        constexpr int KN = DIR == 0 ? TX + 5 : TY + 5;   // cells along the sweep
        const int tid = tx + ty * TX + tz * TX * TY;
        for (int e = tid; e < 8 * NCELL; e += TX * TY * TZ) {
            const int q = e / NCELL, o = e - q * NCELL;
            const int k = DIR == 0 ? o % NC : o / NC;
            if (k == KN - 1) continue;
            const int st = DIR == 0 ? 1 : NC;             // neighbour along the sweep
            const double* F = sF + q * NCELL + o;
            sG[e] = F[0] - F[st];
            if (k == 0) continue;
            sS[e] = q < 4 ? ind_second(F[-st], F[0], F[st]) : ind_second(F[st], F[0], F[-st]);
        }
        __syncthreads();
    }

    // phase 2: reconstruction at the interface
    int line, f;  // line = row j (xi) or column i (eta); f = interface index
    if (DIR == 0) { line = by * TY + ty; f = bx * TX + tx; }
    else          { line = bx * TX + tx; f = by * TY + ty; }
    const int nline = DIR == 0 ? p.nj : p.ni, nface = DIR == 0 ? p.ni + 1 : p.nj + 1;
    if (line >= nline || f >= nface) return;
    const int t = DIR == 0 ? tx : ty;  // position of the interface in the tile
    auto atk = [&](int k) { return DIR == 0 ? at(ty, k) : at(k, tx); };
    // this interface's entry of the adjoint's tape (planes of one direction: 10 x 4 gradient
    // entries per stencil point and component, then the 4 face fluxes)
    double* const tape_at = !TAPE ? nullptr
                            : p.tape + (DIR == 0 ? 0 : tape_planes(REC) * (long long)p.nj * (p.ni + 1)) +
                                  fidx<DIR>(p, 0, line, f);
    (void)tape_at;
    [[maybe_unused]] const long long ts = DIR == 0 ? (long long)p.nj * (p.ni + 1) : (long long)(p.nj + 1) * p.ni;
#pragma unroll
    for (int vz = 0; vz < 4 / TZ; ++vz) {
        const int v = tz + vz * TZ;
        double h;
        if constexpr (kStageS) {
            // "+": lf(m) = F+(tile cell t+m), g_m = G+(t+m), substencils centred on t+1, t+2, t+3;
            // "-": lf(m) = F-(tile cell t+5-m), g_m = F-(t+5-m) - F-(t+4-m) = -G-(t+4-m),
            // substencils centred on t+4, t+3, t+2
            constexpr bool Z = REC == DENSE_RECON_WENOZ5;
            const double* Sp = sS + v * NCELL;
            const double* Sm = sS + (4 + v) * NCELL;
            const double* Gp = sG + v * NCELL;
            const double* Gm = sG + (4 + v) * NCELL;
            double gp[4], gm[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                gp[m] = Gp[atk(t + m)];
                gm[m] = -Gm[atk(t + 4 - m)];
            }
            const double lp2 = sF[v * NCELL + atk(t + 2)], lm2 = sF[(4 + v) * NCELL + atk(t + 3)];
            // the value, and for the tape its gradient from the same terms (stencil slot m0:
            // 0 "+", 5 "-")
            auto recon_taped = [&](double lf2, const double gd[4], const double B[3], double d0, double d1,
                                   double d2, int m0) -> double {
                if constexpr (TAPE) {
                    WenoTerms tt;
                    weno_terms<Z>(gd, d0, d1, d2, tt);
                    const double iN = rcp_nr(tt.N);
                    const double num = weno_num(tt);
                    double g[5];
                    weno_grad<Z>(gd, B, d0, d1, d2, tt, num * iN, iN, g);
#pragma unroll
                    for (int m = 0; m < 5; ++m) tape_at[((m0 + m) * 4 + v) * ts] = g[m];
                    return fma(num, iN, lf2);
                } else {
                    (void)m0; (void)B;
                    return weno_from_d<Z>(lf2, gd, d0, d1, d2);
                }
            };
            double d0, d1, d2, B[3];
            betas_staged(gp, Sp[atk(t + 1)], Sp[atk(t + 2)], Sp[atk(t + 3)], d0, d1, d2, B);
            const double hp = recon_taped(lp2, gp, B, d0, d1, d2, 0);
            betas_staged(gm, Sm[atk(t + 4)], Sm[atk(t + 3)], Sm[atk(t + 2)], d0, d1, d2, B);
            const double hm = recon_taped(lm2, gm, B, d0, d1, d2, 5);
            h = hp + hm;
        } else {
            double lp[5], lm[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                // "+": lf(m) = F+(cell f+3+m), smem index t+2+m; "-": lf(m) = F-(cell f+4-m), index t+3-m
                lp[m] = sF[v * NCELL + atk(t + m)];
                lm[m] = sF[(4 + v) * NCELL + atk(t + 5 - m)];
            }
            h = recon5<REC>(lp) + recon5<REC>(lm);
            if constexpr (TAPE && REC != DENSE_RECON_UPWIND5) {
                // the adjoint's tape: the reconstructions' gradients for stencil slots 0 ("+") and 5 ("-")
                double g[5];
                recon_grad<REC>(lp, g);
#pragma unroll
                for (int m = 0; m < 5; ++m) tape_at[(m * 4 + v) * ts] = g[m];
                recon_grad<REC>(lm, g);
#pragma unroll
                for (int m = 0; m < 5; ++m) tape_at[((5 + m) * 4 + v) * ts] = g[m];
            }
        }
        (DIR == 0 ? p.hx : p.he)[fidx<DIR>(p, v, line, f)] = h;
        if constexpr (TAPE) tape_at[(tape_planes(REC) - 4 + v) * ts] = h;
    }
}

// Programmatic dependent launch: in the plain step graph a kernel may be scheduled while the
// one before it drains (its edges are programmatic); every such kernel waits here, before it
// touches memory, until its predecessors have completed and their writes are visible. Launched
// without a programmatic dependency (eagerly, in the batched graphs) it returns at once.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Unknown reconstruction index with a component-wise splitting: the reference leaves h_xi and
// h_eta untouched (scheme_invs_general.f90:4-27); they start at zero (allocate_block).
__global__ void k_flux_noop(Params p, int irk) {
    grid_dependency_wait();
    if (!p.sc->active) return;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        stage_scalars(p, irk);
        atomicOr(&p.sc->status, DENSE_FLAG_RECON_NOOP);
    }
}

// ---------------------------------------------------------------------------------------------
// Characteristic flux kernel: 104 (ADAPT = false) and 105 AdaWENO (ADAPT = true).
// GLF splitting with the stage's global wave speed; Roe averages and eigenvectors once per
// interface for both signs (104; the reference computes them twice) or once per characteristic
// work item (105). AdaWENO takes its cheap smooth branch at most interfaces and the
// characteristic branch at a few percent of them, clustered near shocks. Run per thread, that
// branch would hold whole warps for the sake of one or two lanes; instead each thread does its
// smooth signs and queues its characteristic (interface, sign) items in shared memory, and the
// whole block then works through the queue on full warps.
// Dynamic shared memory of one characteristic sweep block, in doubles: the tile's split fluxes
// sF[8][NL][NC] and primitives sQ[4][NL][NC]; per-cell sqrt(rho) sS (104, fast); and one region
// R that AdaWENO uses three times over: the scalar surrogates sur[2][NL][NC] and, from them,
// the staged indicator terms (fast: second differences D2, ss + 13/12 D2^2 and first differences
// per sign, 6 x [NL][NC]), read by the interfaces; then, after a barrier, the per-sign results
// hbuf[2][4][NT].
template <int DIR, bool ADAPT, int TX, int TY>
struct CharTile {
    // interfaces of a tile along the sweep (KW): a one-row xi tile of TX threads covers TX - 5
    // interfaces, and an eta tile of one or two columns of TY threads TY - 5 per column, so that
    // the tile's cells take one thread each (staging in one pass, with no warp left to stage a
    // second round of halo cells while the others wait at the barrier); other tiles cover one
    // interface per thread
    static constexpr bool kFit = DIR == 0 ? TY == 1 : TX <= 2;
    static constexpr int KW = DIR == 0 ? (kFit ? TX - 5 : TX) : (kFit ? TY - 5 : TY);
    static constexpr int NL = DIR == 0 ? TY : KW + 5;
    static constexpr int NC = DIR == 0 ? KW + 5 : TX;
    static constexpr int NT = TX * TY;
    static constexpr int NCELL = NL * NC;
    static constexpr bool kStageHS = FAST && !ADAPT;
    static constexpr bool kStageInd = FAST && ADAPT;
    static constexpr int kF = 0, kQ = kF + 8 * NCELL, kS = kQ + 4 * NCELL;
    // 104, fast: the forward differences of the split fluxes along the sweep, F(k) - F(k+1)
    static constexpr int kDF = kS + (kStageHS ? NCELL : 0);
    static constexpr int kR = kDF + (kStageHS ? 8 * NCELL : 0);
    static constexpr int kRSize = !ADAPT ? 0
                                  : (kStageInd ? (8 * NCELL > 8 * NT ? 8 * NCELL : 8 * NT)
                                               : (2 * NCELL > 8 * NT ? 2 * NCELL : 8 * NT));
    static constexpr size_t bytes = sizeof(double) * (size_t)(kR + kRSize);
};

template <int DIR, bool ADAPT, int TX, int TY>
__device__ __forceinline__ void flux_char_block(const Params& p, int irk, int bx, int by) {
    if (!p.sc->active) return;
    using L = CharTile<DIR, ADAPT, TX, TY>;
    constexpr int NL = L::NL, NC = L::NC, NT = L::NT, NCELL = L::NCELL;
    constexpr bool kStageHS = L::kStageHS, kStageInd = L::kStageInd;
    extern __shared__ __align__(16) double dsm[];
    double* const sF = dsm + L::kF;
    double* const sQ = dsm + L::kQ;
    double* const sS = dsm + L::kS;
    double* const sR = dsm + L::kR;
    __shared__ int queue[ADAPT ? 2 * NT : 1];
    __shared__ int qn;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + ty * TX;
    const int slot = irk - 1;
    if (DIR == 0 && bx == 0 && by == 0 && tid == 0) stage_scalars(p, irk);
    const double lam = p.sc->maxeig[slot][DIR];
    const int NIp = p.ni + 2 * kB, NJp = p.nj + 2 * kB;
    const double g1 = p.gamma - 1.0, kg = p.gamma / (p.gamma - 1.0);
    if (ADAPT && tid == 0) qn = 0;
    (void)g1; (void)kg; (void)NL;
    // tile cell (r, c) -> offset; k runs along the sweep, (ox, oy) is the interface's tile position
    auto at = [&](int r, int c) { return chk(p, r, NL) * NC + chk(p, c, NC); };
    auto atk = [&](int k, int ox, int oy) { return DIR == 0 ? at(oy, k) : at(k, ox); };

    // phase 1: split fluxes (and primitives) of the tile's cells
    auto cell = [&](int I, int J, int r, int c) {
        const long long o = cidx(p, I, J);
        double U[4], fp[4], fm[4], q[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = p.cons[v * p.plane + o];
#pragma unroll
        for (int v = 0; v < 4; ++v) q[v] = p.prim[v * p.plane + o];
        lf_split<DIR>(U, q[1 + DIR], q[3], lam, fp, fm);
        if constexpr (kStageHS) {
            const double ir = rcp_nr(q[0]);
            q[3] = fma(kg * q[3], ir, 0.5 * fma(q[1], q[1], q[2] * q[2]));
            sS[at(r, c)] = q[0] * rsqrt_nr(q[0]);
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            sF[v * NCELL + at(r, c)] = fp[v];
            sF[(4 + v) * NCELL + at(r, c)] = fm[v];
            sQ[v * NCELL + at(r, c)] = q[v];
        }
        if constexpr (ADAPT) {  // AdaWENO's scalar surrogates rho + F+-(normal momentum)
            sR[at(r, c)] = q[0] + fp[1 + DIR];
            sR[NCELL + at(r, c)] = q[0] + fm[1 + DIR];
        }
    };
    if (DIR == 0) {
        const int f0 = bx * L::KW, j = by * TY + ty;
        if (j < p.nj)
            for (int k = tx; k < L::KW + 5; k += TX) {
                const int I = f0 + 1 + k;
                if (I < NIp) cell(I, j + kB, ty, k);
            }
    } else {
        const int g0 = by * L::KW, i = bx * TX + tx;
        if (i < p.ni)
            for (int k = ty; k < L::KW + 5; k += TY) {
                const int J = g0 + 1 + k;
                if (J < NJp) cell(i + kB, J, k, tx);
            }
    }
    __syncthreads();

    // phase 1b (104, fast): the split fluxes' forward differences along the sweep, once per cell
    // and sign for the cells with a next neighbour in the tile (each serves four interfaces)
    double* const sDF = dsm + L::kDF;
    if constexpr (kStageHS) {
        constexpr int KN = L::KW + 5;
        constexpr int st = DIR == 0 ? 1 : NC;            // neighbour along the sweep
        for (int e = tid; e < 8 * NCELL; e += NT) {
            const int o = e % NCELL;
            const int k = DIR == 0 ? o % NC : o / NC;
            if (k < KN - 1) sDF[e] = sF[e] - sF[e + st];
        }
        __syncthreads();
    }

    // phase 1b (AdaWENO, fast): per cell and sign, the surrogate's second difference
    // A = sur(k-1) + sur(k+1) - 2 sur(k) (symmetric, so the same for both stencil directions),
    // four times the squared-difference term ss + 13/12 A^2 of the smoothness indicators, and
    // the first difference sur(k+1) - sur(k); an interface's indicators then need only their
    // first-order terms. With the factor 4 (exact in binary) the interfaces add B_k^2 in the
    // indicator's FMA with no 1/4 product; the weights and the switch compare homogeneous
    // products of the d_k, which that scale leaves unchanged.
    double* const sD2 = sR + 2 * NCELL;   // [2][NCELL]: A
    double* const sA2 = sR + 4 * NCELL;   // [2][NCELL]: 4 (ss + 13/12 A^2)
    double* const sDl = sR + 6 * NCELL;   // [2][NCELL]: sur(k+1) - sur(k)
    if constexpr (kStageInd) {
        constexpr int KN = L::KW + 5;                    // cells along the sweep
        constexpr int KL = DIR == 0 ? TY : TX;           // lines
        constexpr double k133 = 13.0 / 3.0;
        for (int e = tid; e < KL * (KN - 2); e += NT) {
            const int line = e / (KN - 2), k = 1 + e % (KN - 2);
            const int o = DIR == 0 ? at(line, k) : at(k, line);
            const int om = DIR == 0 ? at(line, k - 1) : at(k - 1, line);
            const int op = DIR == 0 ? at(line, k + 1) : at(k + 1, line);
#pragma unroll
            for (int sg = 0; sg < 2; ++sg) {
                const double* su = sR + sg * NCELL;
                const double a = fma(-2.0, su[o], su[om] + su[op]);
                sD2[sg * NCELL + o] = a;
                sA2[sg * NCELL + o] = fma(k133 * a, a, 4.0 * kSS);
                sDl[sg * NCELL + o] = su[op] - su[o];
            }
        }
        __syncthreads();
    }

    int line, f;
    if (DIR == 0) { line = by * TY + ty; f = bx * L::KW + tx; }
    else          { line = bx * TX + tx; f = by * L::KW + ty; }
    const int nline = DIR == 0 ? p.nj : p.ni, nface = DIR == 0 ? p.ni + 1 : p.nj + 1;
    const bool valid = line < nline && f < nface && (DIR == 0 ? tx : ty) < L::KW;
    auto SF = [&](int q, int k, int ox, int oy) -> double { return sF[q * NCELL + atk(k, ox, oy)]; };
    auto SQ = [&](int q, int k, int ox, int oy) -> double { return sQ[q * NCELL + atk(k, ox, oy)]; };
#if FAST
    using EigT = EigFast;
#else
    using EigT = Eig;
#endif
    // Roe average and eigenvectors of the interface at (ox, oy): cells at tile offsets +2, +3
    auto eig_at = [&](int ox, int oy, EigT& e) {
        const int kl = (DIR == 0 ? ox : oy) + 2, kr = kl + 1;
#if FAST
        double sl, sr, hl, hr;
        if constexpr (kStageHS) {
            sl = sS[atk(kl, ox, oy)];
            sr = sS[atk(kr, ox, oy)];
            hl = SQ(3, kl, ox, oy);
            hr = SQ(3, kr, ox, oy);
        } else {
            const double rl = SQ(0, kl, ox, oy), rr = SQ(0, kr, ox, oy);
            const double ul = SQ(1, kl, ox, oy), ur = SQ(1, kr, ox, oy);
            const double vl = SQ(2, kl, ox, oy), vr = SQ(2, kr, ox, oy);
            hl = fma(kg * SQ(3, kl, ox, oy), rcp_nr(rl), 0.5 * fma(ul, ul, vl * vl));
            hr = fma(kg * SQ(3, kr, ox, oy), rcp_nr(rr), 0.5 * fma(ur, ur, vr * vr));
            sl = rl * rsqrt_nr(rl);
            sr = rr * rsqrt_nr(rr);
        }
        const bool ok = roe_eig_fast<DIR>(g1, sl, sr, SQ(1, kl, ox, oy), SQ(1, kr, ox, oy),
                                          SQ(2, kl, ox, oy), SQ(2, kr, ox, oy), hl, hr, e);
#else
        const bool ok = roe_eig(DIR, p.gamma, SQ(0, kl, ox, oy), SQ(0, kr, ox, oy), SQ(1, kl, ox, oy),
                                SQ(1, kr, ox, oy), SQ(2, kl, ox, oy), SQ(2, kr, ox, oy), SQ(3, kl, ox, oy),
                                SQ(3, kr, ox, oy), e);
#endif
        if (!ok) atomicOr(&p.sc->status, DENSE_FLAG_ROE_IMAG);
    };
    // stencil of sign s: "+" lf(m) = F+(cell f+3+m), tile index t+m; "-" lf(m) = F-(cell f+4-m),
    // tile index t+5-m (m = 0..4 <-> -2..2)
    auto stencil = [&](int ox, int oy, int s, double F[5][4]) {
        const int t0 = DIR == 0 ? ox : oy;
#pragma unroll
        for (int m = 0; m < 5; ++m)
#pragma unroll
            for (int c = 0; c < 4; ++c) F[m][c] = s == 0 ? SF(c, t0 + m, ox, oy) : SF(4 + c, t0 + 5 - m, ox, oy);
    };
    auto char_recon = [&](const EigT& e, const double F[5][4], double h[4]) {
#if FAST
        char_weno_fast<DIR>(e, F, h);
#else
        char_weno(e, F, h);
#endif
    };
    auto store = [&](const double hsum[4]) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            (DIR == 0 ? p.hx : p.he)[fidx<DIR>(p, v, line, f)] = hsum[v];
        }
        if (p.tape) {  // the adjoint's taping recompute: the face fluxes, the last 4 planes a direction
            constexpr int NP = ADAPT ? 5 : 4;
            const long long xs = (long long)p.nj * (p.ni + 1), ts = DIR == 0 ? xs : (long long)(p.nj + 1) * p.ni;
            double* T = p.tape + (DIR == 0 ? 0 : NP * xs) + (NP - 4) * ts + fidx<DIR>(p, 0, line, f);
#pragma unroll
            for (int v = 0; v < 4; ++v) T[v * ts] = hsum[v];
        }
    };
    auto hbuf = [&](int s, int c, int i) -> double& { return sR[(s * 4 + c) * NT + chk(p, i, (int)NT)]; };
    // the indicator of a valid interface and sign into Params::theta (get_theta_*, SC.f90:1-64)
    auto theta_out = [&](int s, double th) {
        const long long xs = (long long)p.nj * (p.ni + 1), es = (long long)(p.nj + 1) * p.ni;
        p.theta[(DIR == 0 ? s * xs : 2 * xs + s * es) + fidx<DIR>(p, 0, line, f)] = th;
    };

    if constexpr (!ADAPT) {
        // 104: every interface takes the characteristic branch for both signs
        if (!valid) return;
        EigT e;
        eig_at(tx, ty, e);
        double hsum[4];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            double h[4];
#if FAST
            // "+": centre F+(t+2), differences F+(t+m) - F+(t+m+1) = DF+(t+m); "-": centre
            // F-(t+3), differences F-(t+5-m) - F-(t+4-m) = -DF-(t+4-m)
            const int t = DIR == 0 ? tx : ty;
            double Fc[4], dF[4][4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                Fc[c] = s == 0 ? SF(c, t + 2, tx, ty) : SF(4 + c, t + 3, tx, ty);
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    dF[m][c] = s == 0 ? sDF[c * NCELL + atk(t + m, tx, ty)]
                                      : -sDF[(4 + c) * NCELL + atk(t + 4 - m, tx, ty)];
            }
            char_weno_fast_g<DIR>(e, Fc, dF, h);
#else
            double F[5][4];
            stencil(tx, ty, s, F);
            char_recon(e, F, h);
#endif
#pragma unroll
            for (int c = 0; c < 4; ++c) hsum[c] = s == 0 ? h[c] : hsum[c] + h[c];
        }
        store(hsum);
    } else {
        // 105, phase 2a: the AdaWENO indicator from the scalar surrogate rho + F+-(normal
        // momentum) (flux_splitting_SC.f90:175-176,206-207; get_theta_*, scheme_weno5th_SC.f90:
        // 1-64,330-393), the smooth branch (SC.f90:110-124), and the queue of the rest
        const int t = DIR == 0 ? tx : ty;
        bool smooth[2] = {true, true};
        double wsur[2][3];
        if (valid) {
#if FAST
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                // "+": substencils centred on cells t+1, t+2, t+3; "-": on t+4, t+3, t+2
                const int c0 = s == 0 ? t + 1 : t + 4, c2 = s == 0 ? t + 3 : t + 2, cm = t + 2;
                const double* D2 = sD2 + s * NCELL;
                const double* A2 = sA2 + s * NCELL;
                const double* Dl = sDl + s * NCELL;
                const double A0 = D2[atk(c0, tx, ty)], A2c = D2[atk(c2, tx, ty)];
                const double dl1 = Dl[atk(s == 0 ? t + 1 : t + 3, tx, ty)];
                const double dl2 = Dl[atk(t + 2, tx, ty)];
                // B0 = lf0 - 4 lf1 + 3 lf2 = A0 +- 2 dl1, B1 = lf1 - lf3 = -+(dl1 + dl2),
                // B2 = 3 lf2 - 4 lf3 + lf4 = A2 -+ 2 dl2 (upper signs "+", lower "-"); d_k here
                // is 4 (ss + beta_k)
                const double B0 = fma(s == 0 ? 2.0 : -2.0, dl1, A0);
                const double B1 = dl1 + dl2;
                const double B2 = fma(s == 0 ? -2.0 : 2.0, dl2, A2c);
                const double d0 = fma(B0, B0, A2[atk(c0, tx, ty)]);
                const double d1 = fma(B1, B1, A2[atk(cm + (s == 0 ? 0 : 1), tx, ty)]);
                const double d2 = fma(B2, B2, A2[atk(c2, tx, ty)]);
                // WENO-Z over the common denominator D = prod d_k^2, P_k = D/d_k^2, T = tau^2:
                // alpha_k D = c_k (D + T P_k); since sum c_k = 1, N = (sum alpha) D = D + T Q with
                // Q = sum c_k P_k, and theta > delta <=> D > theta_c N. Both sides are positive,
                // so the test compares their bit patterns on the integer pipe.
                const double e0 = d0 * d0, e1 = d1 * d1, e2 = d2 * d2;
                const double P0 = e1 * e2, P1 = e0 * e2, P2 = e0 * e1;
                const double D = e0 * P0;
                const double dd = d2 - d0, T = dd * dd;
                const double Q = fma(c31, P1, c30 * P0) + c32 * P2;
                const double N = fma(T, Q, D);
                smooth[s] = __double_as_longlong(D) > __double_as_longlong(p.theta_c * N);
                const double r = rcp_nr(N);
                // u_k = alpha_k / (c_k sum alpha); the weights are w_k = c_k u_k, w1 = 1 - w0 - w2
                wsur[s][0] = fma(T, P0, D) * r;
                wsur[s][2] = fma(T, P2, D) * r;
                if (p.theta) {  // theta = 1/(1 + (sum alpha - 1)^2), sum alpha - 1 = T Q / D
                    const double sm1 = T * Q / D;
                    theta_out(s, 1.0 / (1.0 + sm1 * sm1));
                }
            }
#else
            double lp[5], lm[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                lp[m] = sR[atk(t + m, tx, ty)];
                lm[m] = sR[NCELL + atk(t + 5 - m, tx, ty)];
            }
            double th;
            weno5z_omega_theta(lp, wsur[0][0], wsur[0][1], wsur[0][2], th);
            smooth[0] = th > p.delta;
            if (p.theta) theta_out(0, th);
            weno5z_omega_theta(lm, wsur[1][0], wsur[1][1], wsur[1][2], th);
            smooth[1] = th > p.delta;
            if (p.theta) theta_out(1, th);
#endif
        }
        __syncthreads();  // the staged surrogate terms are consumed; the region takes the results next
        if (p.tape && valid) {
            // the adjoint's taping recompute: the branches taken (1: "+" smooth, 2: "-" smooth)
            // in the first of the direction's 5 planes, so that the reverse follows the same ones
            const long long xs = (long long)p.nj * (p.ni + 1);
            p.tape[(DIR == 0 ? 0 : 5 * xs) + fidx<DIR>(p, 0, line, f)] = (double)((smooth[0] ? 1 : 0) + (smooth[1] ? 2 : 0));
        }
        if (p.count_branches) {
            const int ns = valid ? (int)smooth[0] + (int)smooth[1] : 0;
            const int nc = valid ? 2 - ns : 0;
            const unsigned tot_s = __reduce_add_sync(0xffffffffu, (unsigned)ns);
            const unsigned tot_c = __reduce_add_sync(0xffffffffu, (unsigned)nc);
            const bool any_valid = __any_sync(0xffffffffu, valid);
            const bool any_c = __any_sync(0xffffffffu, nc > 0);
            if ((tid & 31) == 0 && any_valid) {
                atomicAdd(&p.sc->branch_count[4 * DIR + 0], (unsigned long long)tot_s);
                atomicAdd(&p.sc->branch_count[4 * DIR + 1], (unsigned long long)tot_c);
                atomicAdd(&p.sc->branch_count[4 * DIR + 2], 1ull);
                if (any_c) atomicAdd(&p.sc->branch_count[4 * DIR + 3], 1ull);
            }
        }
#if FAST
        // The smooth results are computed by every lane (uniform, no divergence) and kept only
        // where the smooth branch is taken; the lanes past a fitted xi tile's last interface read
        // that interface's stencils. The "-" sign's stencil sum continues the "+" sign's FMA
        // chain, so a lane smooth in both signs has h = h+ + h- with no separate sum; a lane
        // smooth in "-" only keeps (h+ + h-) - h+.
        {
            const int ox = DIR == 0 && tx >= L::KW ? L::KW - 1 : tx;
            const int oy = DIR == 1 && ty >= L::KW ? L::KW - 1 : ty;
            double F[5][4], W[5], hp[4], hs[4];
            stencil(ox, oy, 0, F);
            stencil_from_u(wsur[0][0], wsur[0][2], W);
#pragma unroll
            for (int c = 0; c < 4; ++c)
                hp[c] = fma(W[4], F[4][c], fma(W[3], F[3][c], fma(W[2], F[2][c], fma(W[1], F[1][c], W[0] * F[0][c]))));
            stencil(ox, oy, 1, F);
            stencil_from_u(wsur[1][0], wsur[1][2], W);
#pragma unroll
            for (int c = 0; c < 4; ++c)
                hs[c] = fma(W[4], F[4][c], fma(W[3], F[3][c], fma(W[2], F[2][c], fma(W[1], F[1][c], fma(W[0], F[0][c], hp[c])))));
            if (valid) {
                if (smooth[0] && smooth[1]) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) hbuf(0, c, tid) = hs[c];
                } else {
                    if (smooth[0]) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) hbuf(0, c, tid) = hp[c];
                    } else {
                        queue[chk(p, atomicAdd(&qn, 1), (int)(2 * NT))] = 2 * tid;
                    }
                    if (smooth[1]) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) hbuf(1, c, tid) = hs[c] - hp[c];
                    } else {
                        queue[chk(p, atomicAdd(&qn, 1), (int)(2 * NT))] = 2 * tid + 1;
                    }
                }
            }
        }
#else
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!valid) continue;
            if (smooth[s]) {
                double F[5][4], h[4];
                stencil(tx, ty, s, F);
#if !FAST
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    double lf[5], q0, q1, q2;
#pragma unroll
                    for (int m = 0; m < 5; ++m) lf[m] = F[m][c];
                    candidates(lf, q0, q1, q2);
                    h[c] = wsur[s][0] * q0 + wsur[s][1] * q1 + wsur[s][2] * q2;
                }
#endif
#pragma unroll
                for (int c = 0; c < 4; ++c) hbuf(s, c, tid) = h[c];
            } else {
                queue[chk(p, atomicAdd(&qn, 1), (int)(2 * NT))] = 2 * tid + s;
            }
        }
#endif
        __syncthreads();
        // phase 2b: the block works through the characteristic items (SC.f90:126-163)
        const int nq = qn;
        for (int it = tid; it < nq; it += NT) {
            const int item = queue[it], owner = item >> 1, s = item & 1;
            const int ox = owner % TX, oy = owner / TX;
            EigT e;
            eig_at(ox, oy, e);
            double F[5][4], h[4];
            stencil(ox, oy, s, F);
            char_recon(e, F, h);
#pragma unroll
            for (int c = 0; c < 4; ++c) hbuf(s, c, owner) = h[c];
        }
        __syncthreads();
        // phase 2c: h = h+ + h- (sum_field, field_op.f90:1-21)
        if (valid) {
            double hsum[4];
#if FAST
            const bool both = smooth[0] && smooth[1];
#else
            const bool both = false;
#endif
#pragma unroll
            for (int c = 0; c < 4; ++c) hsum[c] = both ? hbuf(0, c, tid) : hbuf(0, c, tid) + hbuf(1, c, tid);
            store(hsum);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Max of |u|+alpha, |v|+alpha over a block, then one atomicMax per block on the bit pattern
// (non-negative doubles order like their bits; a NaN compares above +inf and propagates).
__device__ __forceinline__ void block_max_atomic(double e1, double e2, double* slot) {
    unsigned long long a = (unsigned long long)__double_as_longlong(e1);
    unsigned long long b = (unsigned long long)__double_as_longlong(e2);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    __shared__ unsigned long long red[2][32];
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((tid & 31) == 0) { red[0][tid >> 5] = a; red[1][tid >> 5] = b; }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < nw; ++w) { a = max(a, red[0][w]); b = max(b, red[1][w]); }
        atomicMax((unsigned long long*)&slot[0], a);
        atomicMax((unsigned long long*)&slot[1], b);
    }
}

// get_primary at one interior cell (get_primary.f90:53-73); returns the two wave speeds and,
// in pv, the primitives it stored.
__device__ __forceinline__ void prim_cell(const Params& p, long long o, const double q[4], double& e1,
                                          double& e2, unsigned& flags, double pv[5]) {
    const double rho = q[0];
#if FAST
    const double ir = rcp_nr(rho);
    const double u = q[1] * ir;
    const double v = q[2] * ir;
#else
    const double u = q[1] / rho;
    const double v = q[2] / rho;
#endif
#if FAST
    // rho (u^2 + v^2) = m_u u + m_v v
    double pr = (p.gamma - 1.0) * fma(-0.5, fma(q[1], u, q[2] * v), q[3]);
#else
    double pr = (p.gamma - 1.0) * (q[3] - 0.5 * rho * (u * u + v * v));
#endif
#if FAST
    // pr < 0 and a2 > 0 tested on the bit patterns (integer pipe, not an FP64 compare): pr < 0
    // is a set sign bit on a nonzero, non-NaN value; a NaN a2 takes either branch to NaN
    const long long pb = __double_as_longlong(pr), pm = pb & 0x7fffffffffffffffLL;
    if (pb < 0 && pm != 0 && pm <= 0x7ff0000000000000LL) { pr = kPFloor; flags |= DENSE_FLAG_P_FLOOR; }
    const double a2 = p.gamma * pr * ir;
    const double alpha = __double_as_longlong(a2) > 0 ? a2 * rsqrt_nr(a2) : sqrt(a2);
#else
    if (pr < 0.0) { pr = kPFloor; flags |= DENSE_FLAG_P_FLOOR; }
    const double alpha = sqrt(p.gamma * pr / rho);
#endif
    p.prim[o] = rho;
    p.prim[p.plane + o] = u;
    p.prim[2 * p.plane + o] = v;
    p.prim[3 * p.plane + o] = pr;
    p.prim[4 * p.plane + o] = alpha;
    pv[0] = rho; pv[1] = u; pv[2] = v; pv[3] = pr; pv[4] = alpha;
    e1 = fabs(u) + alpha;
    e2 = fabs(v) + alpha;
    // numeric checks on the bit patterns (integer pipe): rho <= 0 or NaN, and any NaN
    const long long rb = __double_as_longlong(rho);
    if (rb <= 0 || rb > 0x7ff0000000000000LL) flags |= DENSE_FLAG_NEG_RHO;
    const unsigned long long kAbs = 0x7fffffffffffffffULL, kInf = 0x7ff0000000000000ULL;
    if (((unsigned long long)__double_as_longlong(q[0]) & kAbs) > kInf ||
        ((unsigned long long)__double_as_longlong(q[1]) & kAbs) > kInf ||
        ((unsigned long long)__double_as_longlong(q[2]) & kAbs) > kInf ||
        ((unsigned long long)__double_as_longlong(q[3]) & kAbs) > kInf)
        flags |= DENSE_FLAG_NAN;
}

__device__ __forceinline__ void prim_block(const Params& p, int slot, int bx, int by) {
    const int i = bx * blockDim.x + threadIdx.x, j = by * blockDim.y + threadIdx.y;
    double e1 = 0.0, e2 = 0.0;
    unsigned flags = 0;
    if (i < p.ni && j < p.nj) {
        const long long o = cidx(p, i + kB, j + kB);
        double q[4], pv[5];
#pragma unroll
        for (int v = 0; v < 4; ++v) q[v] = p.cons[v * p.plane + o];
        prim_cell(p, o, q, e1, e2, flags, pv);
    }
    if (flags) atomicOr(&p.sc->status, flags);
    block_max_atomic(e1, e2, p.sc->maxeig[slot]);
}

// time_rk3_general(irk) (time_advance_general.f90:9-267) fused with get_primary of the updated
// state for the next stage. Body force of Rayleigh-Taylor: S = (0, 0, rho, rho v) of the stage
// input (boundary_rt_general.f90:154-155), added after the combine as a separate rounding.
// (i, j): the thread's interior cell.
template <int IRK>
__device__ __forceinline__ void update_block(const Params& p, int i, int j) {
    if (!p.sc->active) return;
    double e1 = 0.0, e2 = 0.0;
    unsigned flags = 0;
    if (i < p.ni && j < p.nj) {
        const Scalars* sc = p.sc;
        const double dtdx = sc->dtdx, dtdy = sc->dtdy, dt = sc->dt;
        const long long o = cidx(p, i + kB, j + kB);
        // the cell's faces: xi left/right, eta bottom/top; planes hxs, hes apart
        const long long hxs = (long long)p.nj * (p.ni + 1), hes = (long long)(p.nj + 1) * p.ni;
        const long long hxl = fidx<0>(p, 0, j, i), hxr = fidx<0>(p, 0, j, i + 1);
        const long long hel = fidx<1>(p, 0, i, j), her = fidx<1>(p, 0, i, j + 1);
        const double rho_in = p.cons[o], rv_in = p.cons[2 * p.plane + o];
#if FAST
        // stage 2: 3/4 q0 + 1/4 (...); stage 3: 1/3 q0 + 2/3 (...)
        const double ka = IRK == 2 ? 3.0 / 4.0 : 1.0 / 3.0, kb = IRK == 2 ? 1.0 / 4.0 : 2.0 / 3.0;
        const double cx = kb * dtdx, cy = kb * dtdy;
        (void)ka; (void)cx; (void)cy;
#endif
        double q[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double dh_dxi = p.hx[v * hxs + hxr] - p.hx[v * hxs + hxl];
            const double dh_deta = p.he[v * hes + her] - p.he[v * hes + hel];
            const double qc = p.cons[v * p.plane + o];
            double qn;
            if (IRK == 1) {
                p.cons0[v * p.plane + o] = qc;
                qn = qc - dtdx * dh_dxi - dtdy * dh_deta;
            } else {
                const double q0 = p.cons0[v * p.plane + o];
#if FAST
                // a q0 + b (qc - (dt/dx dh_xi + dt/dy dh_eta)), b folded into dt/dx and dt/dy
                qn = fma(ka, q0, fma(kb, qc, -fma(cx, dh_dxi, cy * dh_deta)));
#else
                if (IRK == 2) qn = 3.0 / 4.0 * q0 + 1.0 / 4.0 * qc - 1.0 / 4.0 * (dtdx * dh_dxi + dtdy * dh_deta);
                else          qn = 1.0 / 3.0 * q0 + 2.0 / 3.0 * qc - 2.0 / 3.0 * (dtdx * dh_dxi + dtdy * dh_deta);
#endif
            }
            q[v] = qn;
        }
        if (p.bodyforce) {
            const double f = IRK == 1 ? dt : (IRK == 2 ? 1.0 / 4.0 * dt : kTwoThirdsSP * dt);
            q[0] = q[0] + f * 0.0;
            q[1] = q[1] + f * 0.0;
            q[2] = q[2] + f * rho_in;
            q[3] = q[3] + f * rv_in;
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) p.cons[v * p.plane + o] = q[v];
        double pv[5];
        prim_cell(p, o, q, e1, e2, flags, pv);
        if (p.periodic_ghosts) {
            // the cell's periodic images in the ghost layers (the periodic rule of the boundary
            // fill, boundary_ivc_general.f90:37-59): a ghost of layer k copies the interior cell
            // k+1 in from the opposite side; the corner ghosts are never read
            const int I = i + kB, J = j + kB;
            const int Ig = i < kB ? I + p.ni : (i >= p.ni - kB ? I - p.ni : -1);
            const int Jg = j < kB ? J + p.nj : (j >= p.nj - kB ? J - p.nj : -1);
            auto put = [&](long long g) {
#pragma unroll
                for (int v = 0; v < 4; ++v) p.cons[v * p.plane + g] = q[v];
#pragma unroll
                for (int v = 0; v < 5; ++v) p.prim[v * p.plane + g] = pv[v];
            };
            if (Ig >= 0) put(cidx(p, Ig, J));
            if (Jg >= 0) put(cidx(p, I, Jg));
        }
    }
    if (flags) atomicOr(&p.sc->status, flags);
    block_max_atomic(e1, e2, p.sc->maxeig[IRK % 3]);
}

// ---------------------------------------------------------------------------------------------
// Boundary fill (source/boundary/*.f90). One thread per ghost line: a column of the bottom or
// top ghost rows, or a row of the left or right ghost columns; the four ghost layers of a line
// are filled in the reference's order (the extrapolation is recursive outward).
struct Cell {
    double c[4];
    double q[5];
};

__device__ __forceinline__ void state_from(double gamma, double rho, double u, double v, double pr, Cell& g) {
    g.c[0] = rho; g.c[1] = rho * u; g.c[2] = rho * v;
    g.c[3] = pr / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
    g.q[0] = rho; g.q[1] = u; g.q[2] = v; g.q[3] = pr; g.q[4] = sqrt(gamma * pr / rho);
}

__device__ __forceinline__ void load_cell(const Params& p, int I, int J, Cell& g) {
    const long long o = cidx(p, I, J);
#pragma unroll
    for (int v = 0; v < 4; ++v) g.c[v] = p.cons[v * p.plane + o];
#pragma unroll
    for (int v = 0; v < 5; ++v) g.q[v] = p.prim[v * p.plane + o];
}
__device__ __forceinline__ void store_cell(const Params& p, int I, int J, const Cell& g) {
    const long long o = cidx(p, I, J);
#pragma unroll
    for (int v = 0; v < 4; ++v) p.cons[v * p.plane + o] = g.c[v];
#pragma unroll
    for (int v = 0; v < 5; ++v) p.prim[v * p.plane + o] = g.q[v];
}
// Copy with the normal velocity negated (reflective wall): comp = 1 (u, x-walls) or 2 (v, y-walls)
__device__ __forceinline__ void reflect(Cell& g, int comp) {
    // constant indices keep the cell in registers (a run-time index would put it in local memory)
    if (comp == 1) { g.c[1] = -g.c[1]; g.q[1] = -g.q[1]; }
    else           { g.c[2] = -g.c[2]; g.q[2] = -g.q[2]; }
}
// Recursive 4/3, -1/3 extrapolation (boundary_ivc_general.f90:101-119). Strict: the reference's
// two divides; fast: multiplies by the rounded constants (within an ulp, and no serial divides
// in the boundary kernel's dependent chain).
__device__ __forceinline__ double extrap(double near, double far) {
#if FAST
    return fma(near, 4.0 / 3.0, -(far * (1.0 / 3.0)));
#else
    return near * 4.0 / 3.0 - far / 3.0;
#endif
}

enum Side { kBottom = 0, kTop = 1, kLeft = 2, kRight = 3 };
enum Rule { kNone, kPeriodic, kExtrap, kReflect, kDirichletRT, kDMRBottom, kDMRTop, kDMRInflow, kSSLInflow };

__device__ __forceinline__ Rule side_rule(int bench, int side) {
    switch (bench) {
    case DENSE_BENCH_IVC:  // boundary_ivc_general.f90: y periodic, x extrapolated
        return side <= kTop ? kPeriodic : kExtrap;
    case DENSE_BENCH_SEDOV:  // bottom/left reflective, top/right extrapolated
        return (side == kBottom || side == kLeft) ? kReflect : kExtrap;
    case DENSE_BENCH_RT:  // Dirichlet bottom/top, periodic sides
        return side <= kTop ? kDirichletRT : kPeriodic;
    case DENSE_BENCH_RT_REFLECT:
        return side <= kTop ? kDirichletRT : kReflect;
    case DENSE_BENCH_RM: case DENSE_BENCH_SHOCKVORTEX:  // reflective bottom/top, extrapolated sides
        return side <= kTop ? kReflect : kExtrap;
    case DENSE_BENCH_DMR:
        return side == kBottom ? kDMRBottom : side == kTop ? kDMRTop : side == kLeft ? kDMRInflow : kExtrap;
    case DENSE_BENCH_SSL:  // reflective bottom, top untouched, inflow left, extrapolated right
        return side == kBottom ? kReflect : side == kTop ? kNone : side == kLeft ? kSSLInflow : kExtrap;
    case DENSE_BENCH_IVC_PERIODIC: case DENSE_BENCH_RM_PERIODIC:
        return kPeriodic;
    default:
        return kNone;
    }
}

__device__ __forceinline__ void bc_block(const Params& p, int bx) {
    if (!p.sc->active) return;
    const int tid = bx * blockDim.x + threadIdx.x;
    const int ni = p.ni, nj = p.nj;
    int side, line;
    if (tid < ni) { side = kBottom; line = tid; }
    else if (tid < 2 * ni) { side = kTop; line = tid - ni; }
    else if (tid < 2 * ni + nj) { side = kLeft; line = tid - 2 * ni; }
    else if (tid < 2 * ni + 2 * nj) { side = kRight; line = tid - 2 * ni - nj; }
    else return;
    const Rule rule = side_rule(p.benchmark, side);
    if (rule == kNone) return;
    const double gamma = p.gamma;
    const bool vert = side <= kTop;  // ghost rows of an interior column
    const int I = line + kB, J = line + kB;
    // ghost layer k (0 = next to the interior) of this line
    auto ghost = [&](int k, int& gi, int& gj) {
        if (side == kBottom) { gi = I; gj = kB - 1 - k; }
        else if (side == kTop) { gi = I; gj = nj + kB + k; }
        else if (side == kLeft) { gi = kB - 1 - k; gj = J; }
        else { gi = ni + kB + k; gj = J; }
    };
    // interior cell at distance d (1 = adjacent) from the boundary of this line
    auto inner = [&](int d, int& si, int& sj) {
        if (side == kBottom) { si = I; sj = kB - 1 + d; }
        else if (side == kTop) { si = I; sj = nj + kB - d; }
        else if (side == kLeft) { si = kB - 1 + d; sj = J; }
        else { si = ni + kB - d; sj = J; }
    };
    int gi, gj, si, sj;
    switch (rule) {
    case kPeriodic:
    case kReflect: {
        // periodic: ghost k copies the interior cell k+1 in from the opposite side
        // reflect:  ghost k mirrors the interior cell k+1 in from the same side, normal velocity negated
        auto source = [&](int k, int& si_, int& sj_) {
            int gi_, gj_;
            ghost(k, gi_, gj_);
            if (rule == kPeriodic) {
                if (side == kBottom) { si_ = I; sj_ = nj + gj_; }
                else if (side == kTop) { si_ = I; sj_ = gj_ - nj; }
                else if (side == kLeft) { si_ = ni + gi_; sj_ = J; }
                else { si_ = gi_ - ni; sj_ = J; }
            } else {
                inner(k + 1, si_, sj_);
            }
        };
        if ((vert ? nj : ni) >= kB) {
            // the four sources are interior cells: load them all, then store (one round trip
            // of memory latency instead of four; the compiler cannot reorder the loads above
            // the stores itself, not knowing the ghost and interior cells apart)
            Cell g[kB];
#pragma unroll
            for (int k = 0; k < kB; ++k) { source(k, si, sj); load_cell(p, si, sj, g[k]); }
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                if (rule == kReflect) reflect(g[k], vert ? 2 : 1);
                ghost(k, gi, gj);
                store_cell(p, gi, gj, g[k]);
            }
        } else {
            // fewer interior cells (3) than ghost layers: one periodic source is a ghost cell of
            // the same side, so the layers go in the reference's order -- bottom and left from
            // the outermost layer in (the source is read before it is refilled), top and right
            // from the innermost out (boundary_ivc_general.f90:13-35, boundary_rt_general.f90:
            // 129-151). A mirror source there is a ghost of the opposite side, which another
            // thread fills at the same time; the reference leaves such grids undefined too
            // (its result depends on which side its loops reach first).
#pragma unroll
            for (int kk = 0; kk < kB; ++kk) {
                const int k = (side == kBottom || side == kLeft) ? kB - 1 - kk : kk;
                source(k, si, sj);
                Cell g;
                load_cell(p, si, sj, g);
                if (rule == kReflect) reflect(g, vert ? 2 : 1);
                ghost(k, gi, gj);
                store_cell(p, gi, gj, g);
            }
        }
        break;
    }
    case kExtrap: {
        // recursive outward: g = near*4/3 - far/3 with (near, far) = (g_{k-1}, g_{k-2})
        Cell a, b;
        inner(1, si, sj);
        load_cell(p, si, sj, a);
        inner(2, si, sj);
        load_cell(p, si, sj, b);
#pragma unroll
        for (int k = 0; k < kB; ++k) {
            Cell g;
#pragma unroll
            for (int v = 0; v < 4; ++v) g.c[v] = extrap(a.c[v], b.c[v]);
#pragma unroll
            for (int v = 0; v < 5; ++v) g.q[v] = extrap(a.q[v], b.q[v]);
            ghost(k, gi, gj);
            store_cell(p, gi, gj, g);
            b = a;
            a = g;
        }
        break;
    }
    case kDMRBottom: {  // boundary_doublemach_general.f90:14-48
        if (p.xbot[chk(p, line, p.ni)] >= 1.0 / 6.0) {  // reflecting wall
            if (nj >= kB) {  // interior sources: all loads first, as for kReflect
                Cell g[kB];
#pragma unroll
                for (int k = 0; k < kB; ++k) { inner(k + 1, si, sj); load_cell(p, si, sj, g[k]); }
#pragma unroll
                for (int k = 0; k < kB; ++k) { reflect(g[k], 2); ghost(k, gi, gj); store_cell(p, gi, gj, g[k]); }
                break;
            }
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                Cell g;
                inner(k + 1, si, sj);
                load_cell(p, si, sj, g);
                reflect(g, 2);
                ghost(k, gi, gj);
                store_cell(p, gi, gj, g);
            }
            break;
        }
        Cell g;
        state_from(gamma, 8.0, (double)8.25f * sqrt(3.0) * 0.5, -(double)8.25f * 0.5, 116.5, g);
#pragma unroll
        for (int k = 0; k < kB; ++k) { ghost(k, gi, gj); store_cell(p, gi, gj, g); }
        break;
    }
    default: {
        // Dirichlet states: the same state in all four layers
        Cell g;
        if (rule == kDirichletRT) {  // boundary_rt_general.f90:14-57
            if (side == kBottom) state_from(gamma, 2.0, 0.0, 0.0, 1.0, g);
            else state_from(gamma, 1.0, 0.0, 0.0, 2.5, g);
        } else if (rule == kDMRTop) {  // boundary_doublemach_general.f90:51-76, time at the step's start
            if (p.xtop[chk(p, line, p.ni)] < (1.0 / 6.0 + (1.0 + 20.0 * p.sc->t) / sqrt(3.0)))
                state_from(gamma, 8.0, (double)8.25f * sqrt(3.0) * 0.5, -(double)8.25f * 0.5, 116.5, g);
            else
                state_from(gamma, 1.4, 0.0, 0.0, 1.0, g);
        } else if (rule == kDMRInflow) {  // boundary_doublemach_general.f90:79-99
            state_from(gamma, 8.0, (double)8.25f * sqrt(3.0) * 0.5, -(double)8.25f * 0.5, 116.5, g);
        } else if (rule == kSSLInflow) {  // boundary_ssl_general.f90:40-66
            const double yy = p.yleft[chk(p, line, p.nj)];
            const double rho = yy >= 0.0 ? 1.6374 : 0.3626, pr = 0.3327;
            const double pie = 3.141592653589793115997963468544185161590576171875;
            const double t = p.sc->t;
            const double u = 2.5 + 0.5 * tanh(2.0 * yy);
            const double v = 0.05 * cos(2.0 * pie * t / (30.0 / 2.68)) * exp(-(yy * yy) / 10.0)
                           + 0.05 * cos(2.0 * pie * 2.0 * t / (30.0 / 2.68) + pie / 2.0) * exp(-(yy * yy) / 10.0);
            state_from(gamma, rho, u, v, pr, g);
        } else {
            return;
        }
#pragma unroll
        for (int k = 0; k < kB; ++k) { ghost(k, gi, gj); store_cell(p, gi, gj, g); }
        break;
    }
    }
}

// ---------------------------------------------------------------------------------------------
// Kernels of one block (instance) of the solver: block coordinates are the launch's own.
// Resident blocks the register allocation of a characteristic sweep is sized for. AdaWENO's
// blocks stall on the barriers of their work queue, which a third block per SM hides (80
// registers instead of 94, a few bytes spilled: the xi sweep 2 % faster on the 1920 x 480 double
// Mach reflection); the 104 eta sweep lost 4 % that way and keeps its natural 96 registers.
constexpr int char_min_blocks(bool adapt) { return adapt ? 3 : 1; }
template <int DIR, int SPL, int REC, int TX, int TY, bool TAPE = false, int TZ = 1>
__global__ void __launch_bounds__(TX* TY* TZ) k_flux_cw(Params p, int irk) {
    grid_dependency_wait();
    flux_cw_block<DIR, SPL, REC, TX, TY, TAPE, TZ>(p, irk, blockIdx.x, blockIdx.y);
}
template <int DIR, bool ADAPT, int TX, int TY>
__global__ void __launch_bounds__(TX* TY, char_min_blocks(ADAPT)) k_flux_char(Params p, int irk) {
    grid_dependency_wait();
    flux_char_block<DIR, ADAPT, TX, TY>(p, irk, blockIdx.x, blockIdx.y);
}
__global__ void k_prim(Params p, int slot) {
    grid_dependency_wait();
    prim_block(p, slot, blockIdx.x, blockIdx.y);
}
template <int IRK>
__global__ void k_update(Params p) {
    grid_dependency_wait();
    update_block<IRK>(p, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_bc(Params p) {
    grid_dependency_wait();
    bc_block(p, blockIdx.x);
}

// Batched kernels: one launch covers every instance of a batch. Block b works on instance
// map[b].x at block coordinates (map[b].y, map[b].z) of that instance's own grid, with the
// instance's parameters staged in shared memory; the per-block code is the single-instance
// code, so each instance's arithmetic -- and result -- is the same as a plain solve's.
// The instance's parameters to shared memory, 8-byte words in parallel.
__device__ __forceinline__ void load_params(Params& sp, const Params* src) {
    static_assert(sizeof(Params) % sizeof(long long) == 0, "Params copies as 8-byte words");
    const int lt = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    for (int k = lt; k < (int)(sizeof(Params) / sizeof(long long)); k += nt)
        ((long long*)&sp)[k] = ((const long long*)src)[k];
}
#define DENSE_BATCH_PROLOGUE                                                 \
    __shared__ Params sp;                                                    \
    const int3 m = map[blockIdx.x];                                          \
    load_params(sp, tab + m.x);                                              \
    __syncthreads();

template <int DIR, int SPL, int REC, int TX, int TY>
__global__ void __launch_bounds__(TX* TY) kb_flux_cw(const Params* tab, const int3* map, int irk) {
    DENSE_BATCH_PROLOGUE
    flux_cw_block<DIR, SPL, REC, TX, TY>(sp, irk, m.y, m.z);
}
template <int DIR, bool ADAPT, int TX, int TY>
__global__ void __launch_bounds__(TX* TY, char_min_blocks(ADAPT)) kb_flux_char(const Params* tab, const int3* map, int irk) {
    DENSE_BATCH_PROLOGUE
    flux_char_block<DIR, ADAPT, TX, TY>(sp, irk, m.y, m.z);
}
__global__ void kb_prim(const Params* tab, const int3* map, int slot) {
    DENSE_BATCH_PROLOGUE
    prim_block(sp, slot, m.y, m.z);
}
template <int IRK>
__global__ void kb_update(const Params* tab, const int3* map) {
    DENSE_BATCH_PROLOGUE
    update_block<IRK>(sp, m.y * blockDim.x + threadIdx.x, m.z * blockDim.y + threadIdx.y);
}
__global__ void kb_bc(const Params* tab, const int3* map) {
    DENSE_BATCH_PROLOGUE
    bc_block(sp, m.y);
}
#undef DENSE_BATCH_PROLOGUE


// ---------------------------------------------------------------------------------------------
// Step bookkeeping (general_main.f90:23-37): the while-condition at the start of a step and the
// time/step advance at its end.
__device__ __forceinline__ void k_step_begin_body(Scalars* sc) {
    sc->active = (sc->t < sc->t_end) && (sc->step < sc->total_step) && !sc->hold;
}
__device__ __forceinline__ void k_step_end_body(Scalars* sc) {
    if (sc->active) {
        sc->step += 1;
        sc->t = sc->t + sc->dt;
        sc->elasp = sc->elasp + sc->dt;
        // general_main.f90:40: MOD(current_step, save_step) == 0 .or. elasp_time >= dt_save
        if (sc->save_mode && ((sc->save_step > 0 && sc->step % sc->save_step == 0) || sc->elasp >= sc->dt_save))
            sc->hold = 1;
    }
}
__global__ void k_step_begin(Scalars* sc) {
    grid_dependency_wait();
    k_step_begin_body(sc);
}
__global__ void k_step_end(Scalars* sc) {
    grid_dependency_wait();
    k_step_end_body(sc);
}

#define DENSE_PERSIST (FAST && !DENSE_CHECK)
#if DENSE_PERSIST
// ---------------------------------------------------------------------------------------------
// The persistent step of a batch (component-wise schemes). Resident blocks of kPersistThreads
// threads take the step's items (PersistLaunch, internal.h) in list order from one ticket
// counter. An item waits only for its dependency, the phase before it of its own instance (the
// count of that phase's finished items), so one instance's next stage starts while others are
// still in their sweeps: no grid-wide barrier between phases and no idle tail per phase. The list
// is in phase order, so every item an item waits for was handed out before it, to a running
// block: as that block's current item, which waits only for earlier items, or as its next one,
// which it starts once its current, earlier, item is done. So the earliest unfinished item can
// always proceed, and the waits end. They are bounded
// all the same (spin_limit polls); a wait that gives up sets DENSE_FLAG_TIMEOUT in its instance's
// status and the launch's abort word, and every wait after that gives up at once (the step's
// results are then not valid; the host reports DENSE_ERR_TIMEOUT). A finished item publishes
// with a release add after the block's barrier; a waiting block's first thread polls with
// acquire loads before the barrier that releases the others, so the items' writes are visible
// to every thread of the block.
__device__ __forceinline__ unsigned ld_acquire(const unsigned* a) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
    return v;
}
__device__ __forceinline__ void add_release(unsigned* a, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}

// one sweep tile of the item's variant: the batched tile shapes (batch_tile_shape) with
// threads per interface added to make kPersistThreads
template <int DIR, int SPL, int REC, int TX, int TY>
__device__ __noinline__ void persist_tile(const Params& p, int irk, int bx, int by) {
    constexpr int TZ = kPersistThreads / (TX * TY);
    static_assert(TX * TY * TZ == kPersistThreads, "a persistent tile has kPersistThreads threads");
    flux_cw_block<DIR, SPL, REC, TX, TY, false, TZ>(p, irk, bx, by);
}
template <int SPL, int REC>
__device__ __forceinline__ void persist_sweep(const Params& p, int dir, int variant, int irk, int bx, int by) {
    if (dir == 0) {
        switch (variant) {
        case 1: persist_tile<0, SPL, REC, 64, 2>(p, irk, bx, by); break;
        case 2: persist_tile<0, SPL, REC, 32, 8>(p, irk, bx, by); break;
        case 3: persist_tile<0, SPL, REC, 32, 2>(p, irk, bx, by); break;
        default: persist_tile<0, SPL, REC, 32, 4>(p, irk, bx, by); break;
        }
    } else {
        switch (variant) {
        case 1: persist_tile<1, SPL, REC, 8, 16>(p, irk, bx, by); break;
        case 2: persist_tile<1, SPL, REC, 32, 8>(p, irk, bx, by); break;
        case 3: persist_tile<1, SPL, REC, 16, 16>(p, irk, bx, by); break;
        case 4: persist_tile<1, SPL, REC, 4, 64>(p, irk, bx, by); break;
        default: persist_tile<1, SPL, REC, 8, 32>(p, irk, bx, by); break;
        }
    }
}
__device__ __noinline__ void persist_bc(const Params& p, int bx) { bc_block(p, bx); }
template <int IRK>
__device__ __noinline__ void persist_update(const Params& p, int bx, int by) {
    update_block<IRK>(p, bx * 32 + (int)threadIdx.x % 32, by * 8 + (int)threadIdx.x / 32);
}

template <int SPL, int REC>
__global__ void __launch_bounds__(kPersistThreads, SPL == 0 ? 4 : 2)
kb_persist(const Params* tab, PersistLaunch L, int xi_variant, int eta_variant) {
    __shared__ Params sp;
    __shared__ int s_item, s_skip;
    const int lt = threadIdx.x;
    unsigned* const ticket = L.sync;
    unsigned* const abort_w = L.sync + 1;
    unsigned* const done = L.sync + 2;
    const int4* const items = (const int4*)L.items;
    if (lt == 0) s_item = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    int cur = s_item;
    while (cur < L.nitems) {
        // the next ticket is taken now, its value needed only after this item: the block holds
        // two tickets, which keeps the waits finite (an item handed out as a block's next waits
        // only for that block's current item, which is earlier)
        unsigned nxt = 0;
        if (lt == 0) nxt = atomicAdd(ticket, 1u);
        const int4 w = items[cur];
        const int kind = w.x & 15, irk = (w.x >> 4) & 15, ph = (w.x >> 8) & 255, dep = (w.x >> 16) - 1;
        load_params(sp, tab + w.y);
        if (lt == 0) {
            int skip = 0;
            if (dep >= 0) {
                const unsigned* d = done + w.y * kPhases + dep;
                const unsigned want = L.need[w.y * kPhases + dep];
                long long n = 0;
                while (ld_acquire(d) < want) {
                    if (ld_acquire(abort_w)) { skip = 1; break; }
                    if (++n > L.spin_limit) {
                        atomicOr(abort_w, 1u);
                        atomicOr(L.err, 1u);
                        atomicOr(&tab[w.y].sc->status, DENSE_FLAG_TIMEOUT);
                        skip = 1;
                        break;
                    }
                    __nanosleep(64);
                }
            }
            s_skip = skip;
        }
        __syncthreads();
        if (!s_skip) {
            switch (kind) {
            case kItemBegin: if (lt == 0) k_step_begin_body(sp.sc); break;
            case kItemEnd:   if (lt == 0) k_step_end_body(sp.sc); break;
            case kItemBc:    persist_bc(sp, w.z); break;
            case kItemXi:    persist_sweep<SPL, REC>(sp, 0, xi_variant, irk, w.z, w.w); break;
            case kItemEta:   persist_sweep<SPL, REC>(sp, 1, eta_variant, irk, w.z, w.w); break;
            default:
                if (irk == 1) persist_update<1>(sp, w.z, w.w);
                else if (irk == 2) persist_update<2>(sp, w.z, w.w);
                else persist_update<3>(sp, w.z, w.w);
                break;
            }
        }
        __syncthreads();  // the item's writes precede its count; sp and s_item are free again
        if (lt == 0) {
            add_release(done + w.y * kPhases + ph, 1u);
            s_item = (int)nxt;
        }
        __syncthreads();
        cur = s_item;
    }
}
#endif

// ---------------------------------------------------------------------------------------------
// Launchers
// Component-wise sweeps. xi tile: 32 interfaces x 4 rows (32 x 2 on small grids): a tile
// stages (32 + 5)/32 = 1.16 cells per interface whatever its height. eta tile: 8 columns x 32
// interfaces (8 x 8 on small grids): the halo runs along the sweep, so a tall narrow tile stages
// (32 + 5)/32 = 1.16 cells per interface where 32 x 8 staged 1.63 and 32 x 4 2.25 (each staged
// cell costs its split fluxes and eight indicator terms); 8-wide rows still read whole 64-byte
// segments, and the smem rows of a warp (4 rows x 8 columns) stay free of bank conflicts.
constexpr int kXTX = 32, kXTY = 4, kXSTY = 2;   // xi tile; small-grid height
constexpr int kETX = 8, kETY = 32, kESTY = 8;   // eta tile; small-grid height
// characteristic sweeps: eta tiles of 4 columns x 64 interfaces, AdaWENO xi tiles of one row of
// 256 threads (251 interfaces, 256 cells; long lines along the sweep stage fewer halo cells per
// interface: 1.02 in xi and 1.08 in eta against 1.16 and 1.63 for 32 x 4 and 32 x 8; measured on
// the 1920 x 480 double Mach reflection, these shapes took the sweeps from 0.430 / 0.427 to
// 0.385 / 0.374 ms, the eta tile below to 0.355 ms)
constexpr int kCETX = 4, kCETY = 64;
constexpr int kCXTX = 256, kCXTY = 1;
// AdaWENO eta tiles: 2 columns of 128 threads (123 interfaces, 128 cells each): every thread
// stages one cell, and 123-interface columns cover 481 interfaces in 4 tiles with 2 % idle
// lanes against 6 % for 64-interface columns. (The 104 eta sweep, at 102 registers a thread,
// ran 5 % slower on such tiles on the 256 x 1024 Rayleigh-Taylor case and keeps 4 x 64.)
constexpr int kAETX = 2, kAETY = 128;

static inline dim3 grid_xi(const Params& p, int tx, int ty) {
    return dim3((p.ni + 1 + tx - 1) / tx, (p.nj + ty - 1) / ty);
}
static inline dim3 grid_eta(const Params& p, int tx, int ty) {
    return dim3((p.ni + tx - 1) / tx, (p.nj + 1 + ty - 1) / ty);
}

// Streaming multiprocessors of the current device (queried once).
static int sm_count() {
    static const int n = [] {  // thread-safe one-time initialisation
        int dev = 0, m = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || m <= 0)
            m = 152;
        return m;
    }();
    return n;
}

// A component-wise sweep on its tile's dynamic shared memory.
template <int DIR, int SPL, int REC, int TX, int TY, bool TAPE = false, int TZ = 1>
static void cw_launch(dim3 g, const Params& p, int irk, cudaStream_t s) {
    k_flux_cw<DIR, SPL, REC, TX, TY, TAPE, TZ><<<g, dim3(TX, TY, TZ), CwTile<DIR, REC, TX, TY>::bytes, s>>>(p, irk);
}

// On small grids the standard tiles give a sweep only one or two blocks per SM, and the SMs that
// get one more block than the others set the launch's time. Below four blocks per SM the sweep
// runs with shorter tiles, which multiplies the block count, and with four threads per
// interface (one per component: four times the warps to hide the dependent FP64 chains of a
// sweep that is only one wave deep); same arithmetic per interface, so the results do not
// depend on the tile. Measured on the 200 x 200 vortex: 1.925e8 -> 1.976e8 cell-updates/s for
// the four threads; on 512 x 512 and larger grids the standard tiles gain nothing from them.
// The adjoint's taping sweeps keep one thread per interface (no gain measured).
constexpr int cw_small_tz(bool tape) { return tape ? 1 : 4; }
template <int SPL, int REC, bool TAPE = false>
static void launch_cw(const Params& p, int irk, int dir, cudaStream_t s) {
    const unsigned few = 4u * sm_count();
    if (dir == 0) {
        const dim3 g = grid_xi(p, kXTX, kXTY);
        if (g.x * g.y < few) cw_launch<0, SPL, REC, kXTX, kXSTY, TAPE, cw_small_tz(TAPE)>(grid_xi(p, kXTX, kXSTY), p, irk, s);
        else                 cw_launch<0, SPL, REC, kXTX, kXTY, TAPE>(g, p, irk, s);
    } else {
        const dim3 g = grid_eta(p, kETX, kETY);
        if (g.x * g.y < few) cw_launch<1, SPL, REC, kETX, kESTY, TAPE, cw_small_tz(TAPE)>(grid_eta(p, kETX, kESTY), p, irk, s);
        else                 cw_launch<1, SPL, REC, kETX, kETY, TAPE>(g, p, irk, s);
    }
}

static bool recon_known(int r) {
    return r == DENSE_RECON_UPWIND5 || r == DENSE_RECON_WENOJS5 || r == DENSE_RECON_WENOZ5;
}

static void launch_flux(const Params& p, int irk, int dir, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    switch (p.splitting) {
    case DENSE_SPLIT_LLF: case DENSE_SPLIT_GLF: case DENSE_SPLIT_SW: {
        const int spl = p.splitting == DENSE_SPLIT_SW ? 1 : 0;
        if (p.recon == DENSE_RECON_UPWIND5) { spl ? launch_cw<1, 251>(p, irk, dir, s) : launch_cw<0, 251>(p, irk, dir, s); }
        else if (p.recon == DENSE_RECON_WENOJS5) { spl ? launch_cw<1, 253>(p, irk, dir, s) : launch_cw<0, 253>(p, irk, dir, s); }
        else if (p.recon == DENSE_RECON_WENOZ5) { spl ? launch_cw<1, 255>(p, irk, dir, s) : launch_cw<0, 255>(p, irk, dir, s); }
        else if (dir == 0) k_flux_noop<<<1, 32, 0, s>>>(p, irk);
        break;
    }
    case DENSE_SPLIT_CH:
        if (dir == 0) k_flux_char<0, false, kXTX, kXTY><<<grid_xi(p, kXTX, kXTY), dim3(kXTX, kXTY), CharTile<0, false, kXTX, kXTY>::bytes, s>>>(p, irk);
        else          k_flux_char<1, false, kCETX, kCETY><<<grid_eta(p, kCETX, CharTile<1, false, kCETX, kCETY>::KW), dim3(kCETX, kCETY), CharTile<1, false, kCETX, kCETY>::bytes, s>>>(p, irk);
        break;
    case DENSE_SPLIT_SC:
        if (dir == 0) k_flux_char<0, true, kCXTX, kCXTY><<<grid_xi(p, CharTile<0, true, kCXTX, kCXTY>::KW, kCXTY), dim3(kCXTX, kCXTY), CharTile<0, true, kCXTX, kCXTY>::bytes, s>>>(p, irk);
        else          k_flux_char<1, true, kAETX, kAETY><<<grid_eta(p, kAETX, CharTile<1, true, kAETX, kAETY>::KW), dim3(kAETX, kAETY), CharTile<1, true, kAETX, kAETY>::bytes, s>>>(p, irk);
        break;
    default:
        break;
    }
}

// flux(dir) plus the adjoint tape: LLF/GLF with reconstruction 251, 253 or 255 only
static void launch_flux_tape(const Params& p, int irk, int dir, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (p.splitting == DENSE_SPLIT_CH || p.splitting == DENSE_SPLIT_SC) {  // the plain sweep, which tapes too
        launch_flux(p, irk, dir, stream);
        return;
    }
    if (p.splitting != DENSE_SPLIT_LLF && p.splitting != DENSE_SPLIT_GLF && p.splitting != DENSE_SPLIT_SW) return;
    const bool sw = p.splitting == DENSE_SPLIT_SW;
    switch (p.recon) {
    case DENSE_RECON_UPWIND5: sw ? launch_cw<1, 251, true>(p, irk, dir, s) : launch_cw<0, 251, true>(p, irk, dir, s); break;
    case DENSE_RECON_WENOJS5: sw ? launch_cw<1, 253, true>(p, irk, dir, s) : launch_cw<0, 253, true>(p, irk, dir, s); break;
    case DENSE_RECON_WENOZ5:  sw ? launch_cw<1, 255, true>(p, irk, dir, s) : launch_cw<0, 255, true>(p, irk, dir, s); break;
    default:
        break;
    }
}

static int flux_launches(const Params& p, int dir) {
    if (p.splitting >= DENSE_SPLIT_LLF && p.splitting <= DENSE_SPLIT_SW && !recon_known(p.recon))
        return dir == 0 ? 1 : 0;
    return 1;
}

// Cell blocks of 32 x 8; on grids that give fewer than four of them per SM, blocks of 32 x 2
// even out the last wave (one atomic per block: few blocks on those grids either way)
static dim3 cell_block(const Params& p) {
    const unsigned big = (unsigned)((p.ni + 31) / 32) * (unsigned)((p.nj + 7) / 8);
    return big < 4u * sm_count() ? dim3(32, 2) : dim3(32, 8);
}
static void launch_prim(const Params& p, int slot, void* stream) {
    const dim3 b = cell_block(p), g((p.ni + 31) / 32, (p.nj + b.y - 1) / b.y);
    k_prim<<<g, b, 0, (cudaStream_t)stream>>>(p, slot);
}
// One warp per block: a grid's few thousand ghost lines spread over all SMs, so the latency of
// each line's dependent loads and stores overlaps across the whole GPU instead of a few SMs
// (the 200 x 200 vortex's boundary fill 12.4 -> 8.8 us, its step 4 % faster, against 128)
constexpr int kBcThreads = 32;
static void launch_bc(const Params& p, void* stream) {
    const int n = 2 * p.ni + 2 * p.nj;
    k_bc<<<(n + kBcThreads - 1) / kBcThreads, kBcThreads, 0, (cudaStream_t)stream>>>(p);
}
static void launch_update(const Params& p, int irk, void* stream) {
    const dim3 b = cell_block(p), g((p.ni + 31) / 32, (p.nj + b.y - 1) / b.y);
    cudaStream_t s = (cudaStream_t)stream;
    if (irk == 1) k_update<1><<<g, b, 0, s>>>(p);
    else if (irk == 2) k_update<2><<<g, b, 0, s>>>(p);
    else k_update<3><<<g, b, 0, s>>>(p);
}
static void launch_step_begin(const Params& p, void* stream) { k_step_begin<<<1, 1, 0, (cudaStream_t)stream>>>(p.sc); }
static void launch_step_end(const Params& p, void* stream) { k_step_end<<<1, 1, 0, (cudaStream_t)stream>>>(p.sc); }

// ---------------------------------------------------------------------------------------------
// Batched launchers
__global__ void kb_step_begin(const Params* tab, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) k_step_begin_body(tab[i].sc);
}
__global__ void kb_step_end(const Params* tab, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) k_step_end_body(tab[i].sc);
}

static inline const int3* as_map(const void* m) { return (const int3*)m; }

template <int DIR, int SPL, int REC, int TX, int TY>
static void batch_cw(const BatchLaunch& b, int irk, cudaStream_t s) {
    kb_flux_cw<DIR, SPL, REC, TX, TY><<<DIR == 0 ? b.nb_xi : b.nb_eta, dim3(TX, TY), CwTile<DIR, REC, TX, TY>::bytes, s>>>(
        b.tab, as_map(DIR == 0 ? b.map_xi : b.map_eta), irk);
}
// xi tiles: (32,4) (64,2) (32,8) (32,2); eta tiles: (8,32) (8,16) (32,8) (16,16) (4,64)
template <int SPL, int REC>
static void batch_cw_variant(const BatchLaunch& b, int irk, int dir, cudaStream_t s) {
    const int v = dir == 0 ? b.xi_variant : b.eta_variant;
    if (dir == 0) {
        switch (v) {
        case 1: batch_cw<0, SPL, REC, 64, 2>(b, irk, s); break;
        case 2: batch_cw<0, SPL, REC, 32, 8>(b, irk, s); break;
        case 3: batch_cw<0, SPL, REC, 32, 2>(b, irk, s); break;
        default: batch_cw<0, SPL, REC, 32, 4>(b, irk, s); break;
        }
    } else {
        switch (v) {
        case 1: batch_cw<1, SPL, REC, 8, 16>(b, irk, s); break;
        case 2: batch_cw<1, SPL, REC, 32, 8>(b, irk, s); break;
        case 3: batch_cw<1, SPL, REC, 16, 16>(b, irk, s); break;
        case 4: batch_cw<1, SPL, REC, 4, 64>(b, irk, s); break;
        default: batch_cw<1, SPL, REC, 8, 32>(b, irk, s); break;
        }
    }
}

static void batch_flux(const BatchLaunch& b, int irk, int dir, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    switch (b.splitting) {
    case DENSE_SPLIT_LLF: case DENSE_SPLIT_GLF: case DENSE_SPLIT_SW: {
        const int spl = b.splitting == DENSE_SPLIT_SW ? 1 : 0;
        if (b.recon == DENSE_RECON_UPWIND5) { spl ? batch_cw_variant<1, 251>(b, irk, dir, s) : batch_cw_variant<0, 251>(b, irk, dir, s); }
        else if (b.recon == DENSE_RECON_WENOJS5) { spl ? batch_cw_variant<1, 253>(b, irk, dir, s) : batch_cw_variant<0, 253>(b, irk, dir, s); }
        else if (b.recon == DENSE_RECON_WENOZ5) { spl ? batch_cw_variant<1, 255>(b, irk, dir, s) : batch_cw_variant<0, 255>(b, irk, dir, s); }
        break;  // unknown reconstruction: rejected when the batch is created
    }
    case DENSE_SPLIT_CH:
        if (dir == 0) kb_flux_char<0, false, kXTX, kXTY><<<b.nb_xi, dim3(kXTX, kXTY), CharTile<0, false, kXTX, kXTY>::bytes, s>>>(b.tab, as_map(b.map_xi), irk);
        else          kb_flux_char<1, false, kCETX, kCETY><<<b.nb_eta, dim3(kCETX, kCETY), CharTile<1, false, kCETX, kCETY>::bytes, s>>>(b.tab, as_map(b.map_eta), irk);
        break;
    case DENSE_SPLIT_SC:
        if (dir == 0) kb_flux_char<0, true, kCXTX, kCXTY><<<b.nb_xi, dim3(kCXTX, kCXTY), CharTile<0, true, kCXTX, kCXTY>::bytes, s>>>(b.tab, as_map(b.map_xi), irk);
        else          kb_flux_char<1, true, kAETX, kAETY><<<b.nb_eta, dim3(kAETX, kAETY), CharTile<1, true, kAETX, kAETY>::bytes, s>>>(b.tab, as_map(b.map_eta), irk);
        break;
    default:
        break;
    }
}
static void batch_prim(const BatchLaunch& b, int slot, void* stream) {
    kb_prim<<<b.nb_cells, dim3(32, 8), 0, (cudaStream_t)stream>>>(b.tab, as_map(b.map_cells), slot);
}
static void batch_bc(const BatchLaunch& b, void* stream) {
    kb_bc<<<b.nb_bc, 128, 0, (cudaStream_t)stream>>>(b.tab, as_map(b.map_bc));
}
static void batch_update(const BatchLaunch& b, int irk, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (irk == 1) kb_update<1><<<b.nb_cells, dim3(32, 8), 0, s>>>(b.tab, as_map(b.map_cells));
    else if (irk == 2) kb_update<2><<<b.nb_cells, dim3(32, 8), 0, s>>>(b.tab, as_map(b.map_cells));
    else kb_update<3><<<b.nb_cells, dim3(32, 8), 0, s>>>(b.tab, as_map(b.map_cells));
}
static void batch_step_begin(const BatchLaunch& b, void* stream) {
    kb_step_begin<<<(b.n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(b.tab, b.n);
}
static void batch_step_end(const BatchLaunch& b, void* stream) {
    kb_step_end<<<(b.n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(b.tab, b.n);
}

#if DENSE_PERSIST
template <int SPL, int REC>
static void persist_launch(const BatchLaunch& b, const PersistLaunch& L, cudaStream_t s) {
    kb_persist<SPL, REC><<<L.grid, kPersistThreads, L.smem, s>>>(b.tab, L, b.xi_variant, b.eta_variant);
}
template <int SPL, int REC>
static bool persist_dims(PersistLaunch* L, size_t smem) {
    int per_sm = 0;
    if (cudaFuncSetAttribute(kb_persist<SPL, REC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb_persist<SPL, REC>, kPersistThreads, smem) !=
            cudaSuccess ||
        per_sm < 1)
        return false;
    L->grid = per_sm * sm_count();
    L->smem = smem;
    return true;
}
// dynamic shared memory of a batched tile variant
template <int REC>
static size_t cw_tile_bytes(int dir, int variant) {
    if (dir == 0) {
        switch (variant) {
        case 1: return CwTile<0, REC, 64, 2>::bytes;
        case 2: return CwTile<0, REC, 32, 8>::bytes;
        case 3: return CwTile<0, REC, 32, 2>::bytes;
        default: return CwTile<0, REC, 32, 4>::bytes;
        }
    }
    switch (variant) {
    case 1: return CwTile<1, REC, 8, 16>::bytes;
    case 2: return CwTile<1, REC, 32, 8>::bytes;
    case 3: return CwTile<1, REC, 16, 16>::bytes;
    case 4: return CwTile<1, REC, 4, 64>::bytes;
    default: return CwTile<1, REC, 8, 32>::bytes;
    }
}
template <int SPL, int REC>
static bool persist_shape_of(const BatchLaunch& b, PersistLaunch* L) {
    const size_t sx = cw_tile_bytes<REC>(0, b.xi_variant), se = cw_tile_bytes<REC>(1, b.eta_variant);
    const size_t smem = sx > se ? sx : se;
    return persist_dims<SPL, REC>(L, smem);
}
static bool batch_persist_shape(const BatchLaunch& b, PersistLaunch* L) {
    if (b.splitting != DENSE_SPLIT_LLF && b.splitting != DENSE_SPLIT_GLF && b.splitting != DENSE_SPLIT_SW) return false;
    const bool sw = b.splitting == DENSE_SPLIT_SW;
    switch (b.recon) {
    case DENSE_RECON_UPWIND5: return sw ? persist_shape_of<1, 251>(b, L) : persist_shape_of<0, 251>(b, L);
    case DENSE_RECON_WENOJS5: return sw ? persist_shape_of<1, 253>(b, L) : persist_shape_of<0, 253>(b, L);
    case DENSE_RECON_WENOZ5:  return sw ? persist_shape_of<1, 255>(b, L) : persist_shape_of<0, 255>(b, L);
    default: return false;
    }
}
static void batch_persist(const BatchLaunch& b, const PersistLaunch& L, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const bool sw = b.splitting == DENSE_SPLIT_SW;
    switch (b.recon) {
    case DENSE_RECON_UPWIND5: sw ? persist_launch<1, 251>(b, L, s) : persist_launch<0, 251>(b, L, s); break;
    case DENSE_RECON_WENOJS5: sw ? persist_launch<1, 253>(b, L, s) : persist_launch<0, 253>(b, L, s); break;
    default:                  sw ? persist_launch<1, 255>(b, L, s) : persist_launch<0, 255>(b, L, s); break;
    }
}
#endif

// The sweeps take their tile from dynamic shared memory; with the static work queue of the
// characteristic sweeps and the batched kernels' staged parameters, the larger tiles need more
// than the default 48 KB a block may use, which a kernel has to be allowed once (set for every
// tile, whatever its size).
template <class K>
static void allow_smem(K kernel, size_t bytes) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
template <int SPL, int REC>
static void allow_cw_smem() {
    allow_smem(k_flux_cw<0, SPL, REC, kXTX, kXTY>, CwTile<0, REC, kXTX, kXTY>::bytes);
    allow_smem(k_flux_cw<0, SPL, REC, kXTX, kXSTY, false, cw_small_tz(false)>, CwTile<0, REC, kXTX, kXSTY>::bytes);
    allow_smem(k_flux_cw<1, SPL, REC, kETX, kETY>, CwTile<1, REC, kETX, kETY>::bytes);
    allow_smem(k_flux_cw<1, SPL, REC, kETX, kESTY, false, cw_small_tz(false)>, CwTile<1, REC, kETX, kESTY>::bytes);
    // the adjoint's taping sweeps
    allow_smem(k_flux_cw<0, SPL, REC, kXTX, kXTY, true>, CwTile<0, REC, kXTX, kXTY>::bytes);
    allow_smem(k_flux_cw<0, SPL, REC, kXTX, kXSTY, true, cw_small_tz(true)>, CwTile<0, REC, kXTX, kXSTY>::bytes);
    allow_smem(k_flux_cw<1, SPL, REC, kETX, kETY, true>, CwTile<1, REC, kETX, kETY>::bytes);
    allow_smem(k_flux_cw<1, SPL, REC, kETX, kESTY, true, cw_small_tz(true)>, CwTile<1, REC, kETX, kESTY>::bytes);
    // the batched tile variants of batch_cw_variant
    allow_smem(kb_flux_cw<0, SPL, REC, 32, 4>, CwTile<0, REC, 32, 4>::bytes);
    allow_smem(kb_flux_cw<0, SPL, REC, 64, 2>, CwTile<0, REC, 64, 2>::bytes);
    allow_smem(kb_flux_cw<0, SPL, REC, 32, 8>, CwTile<0, REC, 32, 8>::bytes);
    allow_smem(kb_flux_cw<0, SPL, REC, 32, 2>, CwTile<0, REC, 32, 2>::bytes);
    allow_smem(kb_flux_cw<1, SPL, REC, 8, 32>, CwTile<1, REC, 8, 32>::bytes);
    allow_smem(kb_flux_cw<1, SPL, REC, 8, 16>, CwTile<1, REC, 8, 16>::bytes);
    allow_smem(kb_flux_cw<1, SPL, REC, 32, 8>, CwTile<1, REC, 32, 8>::bytes);
    allow_smem(kb_flux_cw<1, SPL, REC, 16, 16>, CwTile<1, REC, 16, 16>::bytes);
    allow_smem(kb_flux_cw<1, SPL, REC, 4, 64>, CwTile<1, REC, 4, 64>::bytes);
}
static bool allow_tile_smem() {
    allow_cw_smem<0, 251>();
    allow_cw_smem<1, 251>();
    allow_cw_smem<0, 253>();
    allow_cw_smem<1, 253>();
    allow_cw_smem<0, 255>();
    allow_cw_smem<1, 255>();
    allow_smem(k_flux_char<0, false, kXTX, kXTY>, CharTile<0, false, kXTX, kXTY>::bytes);
    allow_smem(k_flux_char<1, false, kCETX, kCETY>, CharTile<1, false, kCETX, kCETY>::bytes);
    allow_smem(k_flux_char<0, true, kCXTX, kCXTY>, CharTile<0, true, kCXTX, kCXTY>::bytes);
    allow_smem(k_flux_char<1, true, kAETX, kAETY>, CharTile<1, true, kAETX, kAETY>::bytes);
    allow_smem(kb_flux_char<0, false, kXTX, kXTY>, CharTile<0, false, kXTX, kXTY>::bytes);
    allow_smem(kb_flux_char<1, false, kCETX, kCETY>, CharTile<1, false, kCETX, kCETY>::bytes);
    allow_smem(kb_flux_char<0, true, kCXTX, kCXTY>, CharTile<0, true, kCXTX, kCXTY>::bytes);
    allow_smem(kb_flux_char<1, true, kAETX, kAETY>, CharTile<1, true, kAETX, kAETY>::bytes);
    return true;
}

}  // namespace VNS

#if DENSE_VARIANT_STRICT
const BatchKernelTable* batch_kernels_strict() {
    static const bool smem_ok = VNS::allow_tile_smem();
    (void)smem_ok;
    static const BatchKernelTable t = {VNS::batch_prim, VNS::batch_bc, VNS::batch_flux, VNS::batch_update,
                                       VNS::batch_step_begin, VNS::batch_step_end};
    return &t;
}
#elif DENSE_CHECK
const BatchKernelTable* batch_kernels_checked() {
    static const bool smem_ok = VNS::allow_tile_smem();
    (void)smem_ok;
    static const BatchKernelTable t = {VNS::batch_prim, VNS::batch_bc, VNS::batch_flux, VNS::batch_update,
                                       VNS::batch_step_begin, VNS::batch_step_end};
    return &t;
}
#else
const BatchKernelTable* batch_kernels_fast() {
    static const bool smem_ok = VNS::allow_tile_smem();
    (void)smem_ok;
    static const BatchKernelTable t = {VNS::batch_prim,       VNS::batch_bc,       VNS::batch_flux,
                                       VNS::batch_update,     VNS::batch_step_begin, VNS::batch_step_end,
                                       VNS::batch_persist,    VNS::batch_persist_shape};
    return &t;
}
// Tile shapes of the batched sweeps (the shapes instantiated above).
void batch_tile_shape(int splitting, int dir, int variant, int* tx, int* ty) {
    if (splitting == DENSE_SPLIT_CH || splitting == DENSE_SPLIT_SC) {
        // xi: 32 x 4 for 104, one row of 251 interfaces (256 threads) for AdaWENO; eta: 4 x 64
        // for 104, 2 columns of 123 interfaces (256 threads) for AdaWENO
        const bool sc = splitting == DENSE_SPLIT_SC;
        *tx = dir == 0 ? (sc ? VNS::CharTile<0, true, VNS::kCXTX, VNS::kCXTY>::KW : VNS::kXTX)
                       : (sc ? VNS::kAETX : VNS::kCETX);
        *ty = dir == 0 ? (sc ? VNS::kCXTY : VNS::kXTY)
                       : (sc ? VNS::CharTile<1, true, VNS::kAETX, VNS::kAETY>::KW
                             : VNS::CharTile<1, false, VNS::kCETX, VNS::kCETY>::KW);
        return;
    }
    static const int xi[kXiVariants][2] = {{32, 4}, {64, 2}, {32, 8}, {32, 2}};
    static const int eta[kEtaVariants][2] = {{8, 32}, {8, 16}, {32, 8}, {16, 16}, {4, 64}};
    const int n = dir == 0 ? kXiVariants : kEtaVariants;
    const int v = variant < 0 || variant >= n ? 0 : variant;
    *tx = dir == 0 ? xi[v][0] : eta[v][0];
    *ty = dir == 0 ? xi[v][1] : eta[v][1];
}
#endif

#if DENSE_VARIANT_STRICT
const KernelTable* kernels_strict() {
    static const bool smem_ok = VNS::allow_tile_smem();
    (void)smem_ok;
    static const KernelTable t = {"strict", VNS::launch_prim, VNS::launch_bc, VNS::launch_flux,
                                  VNS::launch_update, VNS::launch_step_begin, VNS::launch_step_end,
                                  VNS::flux_launches, VNS::launch_flux_tape};
    return &t;
}
#elif DENSE_CHECK
const KernelTable* kernels_checked() {
    static const bool smem_ok = VNS::allow_tile_smem();
    (void)smem_ok;
    static const KernelTable t = {"checked", VNS::launch_prim, VNS::launch_bc, VNS::launch_flux,
                                  VNS::launch_update, VNS::launch_step_begin, VNS::launch_step_end,
                                  VNS::flux_launches, VNS::launch_flux_tape};
    return &t;
}
#else
const KernelTable* kernels_fast() {
    static const bool smem_ok = VNS::allow_tile_smem();
    (void)smem_ok;
    static const KernelTable t = {"fast", VNS::launch_prim, VNS::launch_bc, VNS::launch_flux,
                                  VNS::launch_update, VNS::launch_step_begin, VNS::launch_step_end,
                                  VNS::flux_launches, VNS::launch_flux_tape};
    return &t;
}
#endif

}  // namespace dense

#if !DENSE_VARIANT_STRICT && !DENSE_CHECK
// Accuracy check of the fast reciprocal and inverse square root against CUDA's IEEE divide and
// square root: out[4k..4k+3] = (rcp_nr(x), 1/x, rsqrt_nr(x), 1/sqrt(x)) for each x[k].
namespace {
__global__ void k_fastmath(const double* x, double* out, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double v = x[k];
    out[4 * k + 0] = dense::rcp_nr(v);
    out[4 * k + 1] = 1.0 / v;
    out[4 * k + 2] = dense::rsqrt_nr(v);
    out[4 * k + 3] = 1.0 / sqrt(v);
}
}  // namespace

extern "C" int dense_fastmath_check(const double* x, double* out, int n) {
    if (!x || !out || n <= 0) return DENSE_ERR_ARG;
    double *dx = nullptr, *dout = nullptr;
    if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess) return DENSE_ERR_NOMEM;
    if (cudaMalloc(&dout, 4 * (size_t)n * sizeof(double)) != cudaSuccess) { cudaFree(dx); return DENSE_ERR_NOMEM; }
    cudaError_t e = cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_fastmath<<<(n + 255) / 256, 256>>>(dx, dout, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, 4 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dout);
    return e == cudaSuccess ? DENSE_OK : DENSE_ERR_CUDA;
}
#endif
