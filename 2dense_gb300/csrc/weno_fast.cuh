// weno_fast.cuh -- the WENO-JS5 / WENO-Z5 reconstruction terms of the fast kernels and their
// stencil gradient, shared by the sweeps (kernels.cu) and the discrete adjoint's face-level
// reverse (adjoint.cu). Included inside each file's own namespace (both need dense::rcp_nr).
#pragma once

// weno module constants (source/inv_scheme/weno_mod.f90:3-14,37)
constexpr double a300 = 1.0 / 3.0, a301 = -7.0 / 6.0, a302 = 11.0 / 6.0;
constexpr double a310 = -1.0 / 6.0, a311 = 5.0 / 6.0, a312 = 1.0 / 3.0;
constexpr double a320 = 1.0 / 3.0, a321 = 5.0 / 6.0, a322 = -1.0 / 6.0;
constexpr double c30 = 0.1, c31 = 0.6, c32 = 0.3;
constexpr double kSS = (double)1.0e-6f;       // ss = 1.0e-6, a default-real literal (:37)

// The fast WENO reconstructions work from a stencil's centre value lf[2] and its first
// differences g_m = lf[m] - lf[m+1] (m = 0..3): the indicators' second differences A_k =
// g_k - g_{k+1} and first-order combinations B_0 = g_0 - 3 g_1, B_1 = g_1 + g_2, B_2 = 3 g_2 - g_3,
// and the candidates relative to the centre, q_0 - lf2 = g_0/3 - 5 g_1/6, q_1 - lf2 = -g_1/6 -
// g_2/3, q_2 - lf2 = -2 g_2/3 + g_3/6, so that h = lf[2] + sum_k w_k (q_k - lf[2]) (the weights
// sum to one). The indicators are formed four times over, d_k = 4 (ss + beta_k) = 4 ss +
// 13/3 A_k^2 + B_k^2, with no 1/4 products; the weights are ratios of homogeneous products of the
// d_k, which that exact binary scale leaves unchanged.
constexpr double k133 = 13.0 / 3.0;   // 4 x 13/12 (exactly, in binary)

// d_k = 4 (ss + beta_k) from the first differences and the terms s_k = 4 ss + 13/3 A_k^2 (staged
// once per cell by the component-wise sweeps, whose neighbouring interfaces share them); B[k]
// the first-order combinations.
__device__ __forceinline__ void betas_staged(const double g[4], double s0, double s1, double s2, double& d0,
                                             double& d1, double& d2, double B[3]) {
    B[0] = fma(-3.0, g[1], g[0]); B[1] = g[1] + g[2]; B[2] = fma(3.0, g[2], -g[3]);
    d0 = fma(B[0], B[0], s0);
    d1 = fma(B[1], B[1], s1);
    d2 = fma(B[2], B[2], s2);
}
// The same from the first differences alone (a stencil no other interface shares).
__device__ __forceinline__ void betas_g(const double g[4], double& d0, double& d1, double& d2) {
    const double A0 = g[0] - g[1], A1 = g[1] - g[2], A2 = g[2] - g[3];
    const double B0 = fma(-3.0, g[1], g[0]), B1 = g[1] + g[2], B2 = fma(3.0, g[2], -g[3]);
    d0 = fma(k133 * A0, A0, fma(B0, B0, 4.0 * kSS));
    d1 = fma(k133 * A1, A1, fma(B1, B1, 4.0 * kSS));
    d2 = fma(k133 * A2, A2, fma(B2, B2, 4.0 * kSS));
}
__device__ __forceinline__ void first_differences(const double lf[5], double g[4]) {
#pragma unroll
    for (int m = 0; m < 4; ++m) g[m] = lf[m] - lf[m + 1];
}

// Terms of a WENO reconstruction that its value and, in the adjoint's taping sweeps, its gradient
// share: the relative candidates scaled by the linear weights, r_k = c_k (q_k - lf2), e_k = d_k^2,
// P_k = prod_{j != k} e_j, D = prod e_j, tau = |d_2 - d_0| (4 |beta_2 - beta_0|), v_k = alpha_k
// D / c_k -- P_k (JS) or D + tau^2 P_k (Z) -- and N = sum_k c_k v_k = (sum alpha) D.
struct WenoTerms {
    double r[3], P[3], v[3], D, tau, N;
};
template <bool Z>
__device__ __forceinline__ void weno_terms(const double g[4], double d0, double d1, double d2, WenoTerms& t) {
    t.r[0] = fma(c30 / 3.0, g[0], (-5.0 * c30 / 6.0) * g[1]);
    t.r[1] = fma(-c31 / 3.0, g[2], (-c31 / 6.0) * g[1]);
    t.r[2] = fma(c32 / 6.0, g[3], (-2.0 * c32 / 3.0) * g[2]);
    const double e0 = d0 * d0, e1 = d1 * d1, e2 = d2 * d2;
    t.P[0] = e1 * e2; t.P[1] = e0 * e2; t.P[2] = e0 * e1;
    t.D = e0 * t.P[0];
    const double dd = d2 - d0;
    t.tau = fabs(dd);
    const double T = dd * dd;
#pragma unroll
    for (int k = 0; k < 3; ++k) t.v[k] = Z ? fma(T, t.P[k], t.D) : t.P[k];
    t.N = fma(c32, t.v[2], fma(c31, t.v[1], c30 * t.v[0]));
}
// sum_k v_k r_k, the numerator of h - lf2
__device__ __forceinline__ double weno_num(const WenoTerms& t) {
    return fma(t.v[2], t.r[2], fma(t.v[1], t.r[1], t.v[0] * t.r[0]));
}
// h = lf2 + sum_k v_k r_k / N with iN = 1/N. Every operation is an explicit FMA or a product
// feeding one, so no kernel contracts it differently from another (the plain and taping sweeps
// agree bit for bit).
__device__ __forceinline__ double weno_value(const WenoTerms& t, double iN, double lf2) {
    return fma(weno_num(t), iN, lf2);
}
// WENO reconstruction from its centre value, first differences and d_k.
template <bool Z>
__device__ __forceinline__ double weno_from_d(double lf2, const double g[4], double d0, double d1, double d2) {
    WenoTerms t;
    weno_terms<Z>(g, d0, d1, d2, t);
    return weno_value(t, rcp_nr(t.N), lf2);
}

// Gradient of the WENO reconstruction with respect to its stencil, g[m] = dW/dlf[m], for the
// discrete adjoint's tape. W = sum_k w_k q_k with w_k = a_k / sum(a): dW/dq_k = w_k and
// dW/da_k = (q_k - W)/sum(a); a_k depends on lf through beta_k (JS: a_k = c_k/d_k^2, so
// da_k/dbeta_k = -2 a_k/d_k; Z: a_k = c_k (1 + tau^2/d_k^2), so da_k/dbeta_k = -2 c_k tau^2/d_k^3
// and da_k/dtau = 2 c_k tau/d_k^2, tau = |beta_2 - beta_0|; d_k = ss + beta_k), and beta_k =
// 13/12 A_k^2 + 1/4 B_k^2 on the second differences A_k and the first-order combinations B_k.
// Written over the terms the value itself uses (weno_terms: w_k = c_k v_k / N, and c_k (q_k - W)
// = r_k - c_k (W - lf2); the first-order combinations B_k of its indicators), with corr = W -
// lf2 and iN = 1/N as the value computed them, so that the taping sweep evaluates every shared
// term once. The d_k arrive four times ss + beta_k, which scales 1/d_k and the tau terms by 1/4;
// two exact factors of 4 undo it. W(lf + c) = W(lf) + c (the weights see differences only, and
// each candidate's coefficients sum to one), so the five entries sum to one: the centre entry is
// taken as 1 minus the other four.
template <bool Z>
__device__ __forceinline__ void weno_grad(const double gd[4], const double B[3], double d0, double d1, double d2,
                                          const WenoTerms& t, double corr, double iN, double g[5]) {
    constexpr double cs[3] = {c30, c31, c32};
    double E[3], u[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        E[k] = fma(-cs[k], corr, t.r[k]);  // (q_k - W) c_k
        u[k] = t.v[k] * iN;                // w_k / c_k
    }
    const double iD = 4.0 * rcp_nr(t.D);
    const double id0 = d0 * (t.P[0] * iD), id1 = d1 * (t.P[1] * iD), id2 = d2 * (t.P[2] * iD);  // 1/(ss + beta_k)
    const double A0 = gd[0] - gd[1], B0 = B[0];
    const double A1 = gd[1] - gd[2], B1 = B[1];
    const double A2 = gd[2] - gd[3], B2 = B[2];
    // r_k = -1/2 dW/dbeta_k. With dbeta_k/dlf = 13/6 A_k dA_k/dlf + 1/2 B_k dB_k/dlf, beta_k's
    // share of dW/dlf is -13/3 r_k A_k dA_k/dlf - r_k B_k dB_k/dlf.
    double r0, r1, r2;
    if (!Z) {
        // (q_k - W) w_k / d_k = E_k u_k / d_k
        r0 = (E[0] * u[0]) * id0;
        r1 = (E[1] * u[1]) * id1;
        r2 = (E[2] * u[2]) * id2;
    } else {
        // s_k = (q_k - W)/sum(a) * c_k tau / d_k^2 = E_k tau P_k / N (a quarter of it here)
        const double tau = t.tau;
        const double s0 = (E[0] * tau) * (t.P[0] * iN);
        const double s1 = (E[1] * tau) * (t.P[1] * iN);
        const double s2 = (E[2] * tau) * (t.P[2] * iN);
        // dW/dtau = 2 (s0 + s1 + s2); dtau/dbeta_2 = -dtau/dbeta_0 = sign(beta_2 - beta_0)
        const double st = 4.0 * (s0 + s1 + s2);
        const double sh = d2 >= d0 ? st : -st;
        r0 = fma(s0 * tau, id0, sh);
        r1 = s1 * tau * id1;
        r2 = fma(s2 * tau, id2, -sh);
    }
    const double PA0 = r0 * A0, PA1 = r1 * A1, PA2 = r2 * A2;
    const double NB0 = r0 * B0, NB1 = r1 * B1, NB2 = r2 * B2;
    constexpr double k = -13.0 / 3.0;
    // g[m] = sum_k w_k dq_k/dlf[m] (the 5-point stencil of the weights w_k = c_k u_k, the c_k
    // folded into the stencil's constants) + the indicators' shares
    g[0] = fma(c30 * a300, u[0], fma(k, PA0, -NB0));
    g[1] = fma(c30 * a301, u[0], fma(c31 * a310, u[1], fma(-2.0 * k, PA0, fma(k, PA1, fma(4.0, NB0, -NB1)))));
    g[3] = fma(c31 * a312, u[1], fma(c32 * a321, u[2], fma(k, PA1, fma(-2.0 * k, PA2, fma(4.0, NB2, NB1)))));
    g[4] = fma(c32 * a322, u[2], fma(k, PA2, -NB2));
    g[2] = 1.0 - ((g[0] + g[1]) + (g[3] + g[4]));
}

// The weights' share alone of a reconstruction's stencil gradient, for weights computed from one
// stencil (lf, through gd, B, d_k and its weno_terms t, iN = 1/N) and applied to candidates of
// other data: AdaWENO's smooth branch reconstructs every component with the WENO-Z weights of
// its scalar surrogate. With the value sum_k w_k Q_k (Q_k the candidates, already contracted with
// the components' sensitivities) and E_k = c_k (Q_k - sum_j w_j Q_j), g[m] = d(sum_k w_k Q_k)/dlf[m]
// -- weno_grad's indicator terms with its candidate terms left out. The weights see differences
// only, so the five entries sum to zero.
template <bool Z>
__device__ __forceinline__ void weno_weight_grad(const double gd[4], const double B[3], double d0, double d1,
                                                 double d2, const WenoTerms& t, const double E[3], double iN,
                                                 double g[5]) {
    const double iD = 4.0 * rcp_nr(t.D);
    const double id0 = d0 * (t.P[0] * iD), id1 = d1 * (t.P[1] * iD), id2 = d2 * (t.P[2] * iD);  // 1/(ss + beta_k)
    const double A0 = gd[0] - gd[1], A1 = gd[1] - gd[2], A2 = gd[2] - gd[3];
    double r0, r1, r2;
    if (!Z) {
        r0 = (E[0] * (t.v[0] * iN)) * id0;
        r1 = (E[1] * (t.v[1] * iN)) * id1;
        r2 = (E[2] * (t.v[2] * iN)) * id2;
    } else {
        const double tau = t.tau;
        const double s0 = (E[0] * tau) * (t.P[0] * iN);
        const double s1 = (E[1] * tau) * (t.P[1] * iN);
        const double s2 = (E[2] * tau) * (t.P[2] * iN);
        const double st = 4.0 * (s0 + s1 + s2);
        const double sh = d2 >= d0 ? st : -st;
        r0 = fma(s0 * tau, id0, sh);
        r1 = s1 * tau * id1;
        r2 = fma(s2 * tau, id2, -sh);
    }
    const double PA0 = r0 * A0, PA1 = r1 * A1, PA2 = r2 * A2;
    const double NB0 = r0 * B[0], NB1 = r1 * B[1], NB2 = r2 * B[2];
    constexpr double k = -13.0 / 3.0;
    g[0] = fma(k, PA0, -NB0);
    g[1] = fma(-2.0 * k, PA0, fma(k, PA1, fma(4.0, NB0, -NB1)));
    g[3] = fma(k, PA1, fma(-2.0 * k, PA2, fma(4.0, NB2, NB1)));
    g[4] = fma(k, PA2, -NB2);
    g[2] = -((g[0] + g[1]) + (g[3] + g[4]));
}
