// adjoint.cu — the discrete adjoint of the plain solver's time step: LLF splitting (101) with
// upwind5 / WENO-JS5 / WENO-Z5 reconstruction (251/253/255) and TVD-RK3 with the CFL time step,
// on grids periodic in x and y (benchmarks 11 and 14).
//
// The forward step (time_rk3_general, time_advance_general.f90:9-267) applies per stage
//     L(u)_c = -(h_{f+1} - h_f)/dx - (g_{f'+1} - g_{f'})/dy,     cell c between faces f, f+1,
//     h_f = W(F+ of cells f-3..f+1) + W(F- of cells f+2..f-2)    (cells in interior indices,
// ghosts are periodic images), F+- = 0.5((u_n +- lambda) U + P), lambda = |u_n| + alpha of the
// cell (flux_splitting_LLF.f90:67-81), W one of the 5-point reconstructions
// (scheme_weno5js_general.f90, scheme_weno5z_general.f90, scheme_upwind5_general.f90), and
//     u1 = u0 + dt L(u0),  u2 = 3/4 u0 + 1/4 u1 + 1/4 dt L(u1),  u3 = 1/3 u0 + 2/3 u2 + 2/3 dt L(u2)
// with dt = cfl / (max(|u|+alpha)/dx + max(|v|+alpha)/dy) of u0.
//
// The vector-Jacobian product v -> (dL/du)^T v runs in three kernels per stage:
//   k_face (one per direction, one thread per face): hbar_f = (v_right - v_left)/dx, then the
//     reverse mode of the two 5-point reconstructions gives the sensitivities of the stencil's
//     split fluxes; the 5 values per (sign, equation) go to a face buffer G, and the face adds
//     h_f * hbar_f to its block's share of v . L(u) (summation by parts);
//   k_cell (one thread per cell): gathers, in a fixed order, the G entries of every face whose
//     stencils read the cell or one of its periodic images, applies the transposed Jacobian of
//     F+- at the cell for both directions, and applies the reverse of the RK stage;
//   k_dt (one block, once per step): the time step's sensitivity sum_s c_s v_s . L(u_{s-1}),
//     sent through dt(max wave speeds) to the cells where the maxima are attained.
// No atomics: every sum has a fixed order, so the gradient is deterministic.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <string>
#include <vector>

#include "handle.h"

namespace dense {
namespace adj {

constexpr double a300 = 1.0 / 3.0, a301 = -7.0 / 6.0, a302 = 11.0 / 6.0;
constexpr double a310 = -1.0 / 6.0, a311 = 5.0 / 6.0, a312 = 1.0 / 3.0;
constexpr double a320 = 1.0 / 3.0, a321 = 5.0 / 6.0, a322 = -1.0 / 6.0;
constexpr double kSS = (double)1.0e-6f;      // weno_mod.f90:37, a default-real literal
constexpr double kPFloor = (double)1.0e-6f;  // get_primary.f90:58

struct AdjParams {
    int ni, nj;
    long long plane;  // ni * nj: one variable of a compact interior state
    double gamma, dx, dy, inv_dx, inv_dy, cfl;
};

// Reverse mode of one 5-point reconstruction h = W(f): adds hbar * dh/df_m to fbar[m] and
// returns h. For WENO, h = sum_k a_k q_k / S with S = sum_k a_k, so dh/dq_k = a_k/S and
// dh/da_k = (q_k - h)/S; a_k depends on f through the smoothness indicators beta_k
// (JS: a_k = c_k/(eps+beta_k)^2; Z: a_k = c_k (1 + (tau/(eps+beta_k))^2), tau = |beta_2-beta_0|).
template <int REC>
__device__ __forceinline__ double recon_rev(const double f[5], double hbar, double fbar[5]) {
    if (REC == DENSE_RECON_UPWIND5) {
        const double k = hbar / 60.0;
        fbar[0] += 2.0 * k; fbar[1] -= 13.0 * k; fbar[2] += 47.0 * k; fbar[3] += 27.0 * k; fbar[4] -= 3.0 * k;
        return (2.0 * f[0] - 13.0 * f[1] + 47.0 * f[2] + 27.0 * f[3] - 3.0 * f[4]) / 60.0;
    }
    constexpr double c[3] = {0.1, 0.6, 0.3};
    const double q[3] = {a300 * f[0] + a301 * f[1] + a302 * f[2], a310 * f[1] + a311 * f[2] + a312 * f[3],
                         a320 * f[2] + a321 * f[3] + a322 * f[4]};
    const double A[3] = {f[0] - 2.0 * f[1] + f[2], f[1] - 2.0 * f[2] + f[3], f[2] - 2.0 * f[3] + f[4]};
    const double B[3] = {f[0] - 4.0 * f[1] + 3.0 * f[2], f[1] - f[3], 3.0 * f[2] - 4.0 * f[3] + f[4]};
    double beta[3], id[3], a[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        beta[k] = 13.0 / 12.0 * (A[k] * A[k]) + 0.25 * (B[k] * B[k]);
        id[k] = 1.0 / (kSS + beta[k]);
    }
    const double tau = fabs(beta[2] - beta[0]);
#pragma unroll
    for (int k = 0; k < 3; ++k)
        a[k] = REC == DENSE_RECON_WENOJS5 ? c[k] * (id[k] * id[k]) : c[k] * (1.0 + (tau * id[k]) * (tau * id[k]));
    const double iS = 1.0 / (a[0] + a[1] + a[2]);
    const double h = (a[0] * q[0] + a[1] * q[1] + a[2] * q[2]) * iS;
    double qbar[3], bbar[3], taubar = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        qbar[k] = hbar * a[k] * iS;
        const double abar = hbar * (q[k] - h) * iS;
        if (REC == DENSE_RECON_WENOJS5) {
            bbar[k] = -2.0 * abar * a[k] * id[k];                  // da/dbeta = -2 a/(eps+beta)
        } else {
            const double r = tau * id[k];
            bbar[k] = -2.0 * abar * c[k] * r * r * id[k];          // da/dbeta = -2 c r^2/(eps+beta)
            taubar += 2.0 * abar * c[k] * r * id[k];               // da/dtau  =  2 c r/(eps+beta)
        }
    }
    if (REC == DENSE_RECON_WENOZ5) {
        const double sg = beta[2] >= beta[0] ? taubar : -taubar;
        bbar[2] += sg;
        bbar[0] -= sg;
    }
    fbar[0] += qbar[0] * a300;
    fbar[1] += qbar[0] * a301 + qbar[1] * a310;
    fbar[2] += qbar[0] * a302 + qbar[1] * a311 + qbar[2] * a320;
    fbar[3] += qbar[1] * a312 + qbar[2] * a321;
    fbar[4] += qbar[2] * a322;
    // beta_k = 13/12 A_k^2 + 1/4 B_k^2: dbeta/dA = 13/6 A, dbeta/dB = B/2
    double Ab[3], Bb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { Ab[k] = bbar[k] * (13.0 / 6.0) * A[k]; Bb[k] = bbar[k] * 0.5 * B[k]; }
    fbar[0] += Ab[0] + Bb[0];
    fbar[1] += -2.0 * Ab[0] - 4.0 * Bb[0] + Ab[1] + Bb[1];
    fbar[2] += Ab[0] + 3.0 * Bb[0] - 2.0 * Ab[1] + Ab[2] + 3.0 * Bb[2];
    fbar[3] += Ab[1] - Bb[1] - 2.0 * Ab[2] - 4.0 * Bb[2];
    fbar[4] += Ab[2] + Bb[2];
    return h;
}

// get_primary of one cell (get_primary.f90:53-60), with the pressure floor of :58.
struct Prim {
    double u, v, p, a, ir;
    bool floored;
};
__device__ __forceinline__ Prim prim_of(const double U[4], double gamma) {
    Prim q;
    q.ir = 1.0 / U[0];
    q.u = U[1] * q.ir;
    q.v = U[2] * q.ir;
    q.p = (gamma - 1.0) * (U[3] - 0.5 * U[0] * (q.u * q.u + q.v * q.v));
    q.floored = q.p < 0.0;
    if (q.floored) q.p = kPFloor;
    q.a = sqrt(gamma * q.p * q.ir);
    return q;
}

// LLF split fluxes of one cell in direction DIR (flux_splitting_LLF.f90:67-81).
template <int DIR>
__device__ __forceinline__ void llf_fluxes(const double U[4], const Prim& q, double fp[4], double fm[4]) {
    const double un = DIR == 0 ? q.u : q.v;
    const double lam = fabs(un) + q.a;
    const double up = un + lam, um = un - lam;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double add = c == 1 + DIR ? q.p : (c == 3 ? un * q.p : 0.0);
        fp[c] = 0.5 * (up * U[c] + add);
        fm[c] = 0.5 * (um * U[c] + add);
    }
}

// Sensitivities of (u_n, alpha, p) pulled back to the conserved variables of the cell.
template <int DIR>
__device__ __forceinline__ void prim_pullback(const double U[4], const Prim& q, double gamma, double unb,
                                              double ab, double pb, double Ub[4]) {
    // alpha = sqrt(gamma p / rho): dalpha/dp = gamma/(2 alpha rho), dalpha/drho = -alpha/(2 rho)
    double rb = -ab * 0.5 * q.a * q.ir;
    if (!q.floored) pb += ab * gamma * 0.5 / (q.a * U[0]);
    // u_n = m_n / rho
    const double un = DIR == 0 ? q.u : q.v;
    Ub[1 + DIR] += unb * q.ir;
    rb -= unb * un * q.ir;
    // p = (gamma-1)(E - (m1^2 + m2^2)/(2 rho)); constant where floored
    if (!q.floored) {
        const double g1 = gamma - 1.0;
        Ub[3] += g1 * pb;
        Ub[1] -= g1 * q.u * pb;
        Ub[2] -= g1 * q.v * pb;
        rb += g1 * 0.5 * (q.u * q.u + q.v * q.v) * pb;
    }
    Ub[0] += rb;
}

// Ub += (dF+/dU)^T gp + (dF-/dU)^T gm at one cell, direction DIR.
template <int DIR>
__device__ __forceinline__ void llf_vjp(const double U[4], const Prim& q, double gamma, const double gp[4],
                                        const double gm[4], double Ub[4]) {
    const double un = DIR == 0 ? q.u : q.v;
    const double s = un >= 0.0 ? 1.0 : -1.0;
    const double lam = s * un + q.a;
    const double up = un + lam, um = un - lam;
    double Sp = 0.0, Sm = 0.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        Ub[c] += 0.5 * (up * gp[c] + um * gm[c]);
        Sp += gp[c] * U[c];
        Sm += gm[c] * U[c];
    }
    Sp *= 0.5;
    Sm *= 0.5;
    const double g3 = gp[3] + gm[3];
    const double lamb = Sp - Sm;
    const double unb = Sp + Sm + 0.5 * q.p * g3 + s * lamb;
    const double pb = 0.5 * (gp[1 + DIR] + gm[1 + DIR]) + 0.5 * un * g3;
    prim_pullback<DIR>(U, q, gamma, unb, lamb, pb, Ub);
}

// Ub += scale * d(|u_n| + alpha)/dU at one cell.
template <int DIR>
__device__ __forceinline__ void wave_speed_vjp(const double U[4], double gamma, double scale, double Ub[4]) {
    const Prim q = prim_of(U, gamma);
    const double un = DIR == 0 ? q.u : q.v;
    prim_pullback<DIR>(U, q, gamma, (un >= 0.0 ? 1.0 : -1.0) * scale, scale, 0.0, Ub);
}

// Deterministic block sum (fixed lane and warp order); the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double x) {
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __shared__ double red[32];
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((tid & 31) == 0) red[tid >> 5] = x;
    __syncthreads();
    double s = 0.0;
    if (tid == 0)
        for (int w = 0; w < nw; ++w) s += red[w];
    return s;
}

// ---------------------------------------------------------------------------------------------
// Face kernel. xi: TX faces x TY rows per block, the tile's cells f0-3 .. f0+TX+1 staged in
// shared memory; eta: TX columns x TY faces. G[sign][m][eq][...] holds, per face, the
// sensitivity of the m-th stencil value of the (sign, eq) reconstruction; the layout follows
// the forward's face arrays (xi [row][face], eta [face][column]).
template <int DIR, int REC, int TX, int TY>
__global__ void __launch_bounds__(TX * TY) k_face(AdjParams a, const double* __restrict__ u,
                                                  const double* __restrict__ w, double* __restrict__ G,
                                                  double* __restrict__ part) {
    constexpr int NL = DIR == 0 ? TY : TY + 5;
    constexpr int NC = DIR == 0 ? TX + 5 : TX;
    __shared__ double sF[8][NL][NC];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int ni = a.ni, nj = a.nj;
    auto stage_cell = [&](int i, int j, int r, int c) {
        double U[4], fp[4], fm[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = u[v * a.plane + (long long)j * ni + i];
        const Prim q = prim_of(U, a.gamma);
        llf_fluxes<DIR>(U, q, fp, fm);
#pragma unroll
        for (int v = 0; v < 4; ++v) { sF[v][r][c] = fp[v]; sF[4 + v][r][c] = fm[v]; }
    };
    if (DIR == 0) {
        const int f0 = blockIdx.x * TX, j = blockIdx.y * TY + ty;
        if (j < nj)
            for (int k = tx; k < TX + 5; k += TX) {
                int i = f0 - 3 + k;           // cells -3 .. ni+2 are read; the rest of the tile is not
                if (i > ni + 2) break;
                i = i < 0 ? i + ni : (i >= ni ? i - ni : i);
                stage_cell(i, j, ty, k);
            }
    } else {
        const int g0 = blockIdx.y * TY, i = blockIdx.x * TX + tx;
        if (i < ni)
            for (int k = ty; k < TY + 5; k += TY) {
                int j = g0 - 3 + k;
                if (j > nj + 2) break;
                j = j < 0 ? j + nj : (j >= nj ? j - nj : j);
                stage_cell(i, j, k, tx);
            }
    }
    __syncthreads();

    const int line = DIR == 0 ? blockIdx.y * TY + ty : blockIdx.x * TX + tx;
    const int f = DIR == 0 ? blockIdx.x * TX + tx : blockIdx.y * TY + ty;
    const int nline = DIR == 0 ? nj : ni, n = DIR == 0 ? ni : nj;
    double vdl = 0.0;
    if (line < nline && f <= n) {
        const int t = DIR == 0 ? tx : ty;
        const double inv = DIR == 0 ? a.inv_dx : a.inv_dy;
        const long long oR = DIR == 0 ? (long long)line * ni + f : (long long)f * ni + line;
        const long long oL = oR - (DIR == 0 ? 1 : ni);
        const long long gs = DIR == 0 ? (long long)nj * (ni + 1) : (long long)(nj + 1) * ni;
        const long long go = DIR == 0 ? (long long)line * (ni + 1) + f : (long long)f * ni + line;
#pragma unroll 1
        for (int v = 0; v < 4; ++v) {
            const double wr = f < n ? w[v * a.plane + oR] : 0.0;   // face n is the right face of cell n-1 only
            const double wl = f >= 1 ? w[v * a.plane + oL] : 0.0;  // face 0 is the left face of cell 0 only
            const double hb = (wr - wl) * inv;
            double lp[5], lm[5], bp[5] = {0, 0, 0, 0, 0}, bm[5] = {0, 0, 0, 0, 0};
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                if (DIR == 0) { lp[m] = sF[v][ty][t + m]; lm[m] = sF[4 + v][ty][t + 5 - m]; }
                else          { lp[m] = sF[v][t + m][tx]; lm[m] = sF[4 + v][t + 5 - m][tx]; }
            }
            const double h = recon_rev<REC>(lp, hb, bp) + recon_rev<REC>(lm, hb, bm);
            vdl += h * hb;
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                G[((long long)(m * 4 + v)) * gs + go] = bp[m];
                G[((long long)((5 + m) * 4 + v)) * gs + go] = bm[m];
            }
        }
    }
    const double s = block_sum(vdl);
    if (tx == 0 && ty == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// Sum of the G entries that read cell x of a line (faces 0..n), over the cell's periodic
// images: "+" stencils read cell f-3+m, "-" stencils cell f+2-m.
__device__ __forceinline__ void gather_sign(const double* __restrict__ G, long long gs, long long base,
                                            long long stride, int k0, int f, int n, double acc[4]) {
    if (f >= 0 && f <= n) {
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[v] += G[(long long)(k0 + v) * gs + base + f * stride];
    }
    if (f >= n) {  // image x - n, read by face f - n
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[v] += G[(long long)(k0 + v) * gs + base + (f - n) * stride];
    }
    if (f <= 0) {  // image x + n, read by face f + n
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[v] += G[(long long)(k0 + v) * gs + base + (f + n) * stride];
    }
}
__device__ __forceinline__ void gather_line(const double* __restrict__ G, long long gs, long long base,
                                            long long stride, int x, int n, double gp[4], double gm[4]) {
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        gather_sign(G, gs, base, stride, m * 4, x + 3 - m, n, gp);
        gather_sign(G, gs, base, stride, (5 + m) * 4, x - 2 + m, n, gm);
    }
}

// Cell kernel: Ub = (dL/du)^T w at the cell, then the reverse of RK stage STAGE
// (3, 2, 1; 0 = Ub alone). Stage 1 also reduces the wave-speed maxima of its state u0
// (the time step's input) per block, with their cells.
template <int STAGE>
__global__ void __launch_bounds__(256) k_cell(AdjParams a, const double* __restrict__ u,
                                              const double* __restrict__ w, const double* __restrict__ Gx,
                                              const double* __restrict__ Gy, double* __restrict__ acc,
                                              double* __restrict__ out, const double* __restrict__ dtp,
                                              double* __restrict__ mpart) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int ni = a.ni, nj = a.nj;
    double e1 = -1.0, e2 = -1.0;
    long long i1 = LLONG_MAX, i2 = LLONG_MAX;
    if (i < ni && j < nj) {
        const long long o = (long long)j * ni + i;
        double U[4], Ub[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = u[v * a.plane + o];
        const Prim q = prim_of(U, a.gamma);
        {
            double gp[4] = {0, 0, 0, 0}, gm[4] = {0, 0, 0, 0};
            gather_line(Gx, (long long)nj * (ni + 1), (long long)j * (ni + 1), 1, i, ni, gp, gm);
            llf_vjp<0>(U, q, a.gamma, gp, gm, Ub);
        }
        {
            double gp[4] = {0, 0, 0, 0}, gm[4] = {0, 0, 0, 0};
            gather_line(Gy, (long long)(nj + 1) * ni, i, ni, j, nj, gp, gm);
            llf_vjp<1>(U, q, a.gamma, gp, gm, Ub);
        }
        const double dt = STAGE == 0 ? 0.0 : *dtp;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const long long ov = v * a.plane + o;
            if (STAGE == 0) {
                out[ov] = Ub[v];
            } else {
                const double wv = w[ov];
                if (STAGE == 3) {
                    acc[ov] = 1.0 / 3.0 * wv;
                    out[ov] = 2.0 / 3.0 * wv + 2.0 / 3.0 * dt * Ub[v];
                } else if (STAGE == 2) {
                    acc[ov] += 3.0 / 4.0 * wv;
                    out[ov] = 1.0 / 4.0 * wv + 1.0 / 4.0 * dt * Ub[v];
                } else {
                    out[ov] = acc[ov] + wv + dt * Ub[v];
                }
            }
        }
        if (STAGE == 1) {
            e1 = fabs(q.u) + q.a;
            e2 = fabs(q.v) + q.a;
            i1 = i2 = o;
        }
    }
    if (STAGE == 1 && mpart) {
        // block argmax, ties to the lowest cell index
        auto better = [](double ea, long long ia, double eb, long long ib) {
            return ea > eb || (ea == eb && ia < ib);
        };
#pragma unroll
        for (int s = 16; s; s >>= 1) {
            const double oe1 = __shfl_xor_sync(0xffffffffu, e1, s), oe2 = __shfl_xor_sync(0xffffffffu, e2, s);
            const long long oi1 = __shfl_xor_sync(0xffffffffu, i1, s), oi2 = __shfl_xor_sync(0xffffffffu, i2, s);
            if (better(oe1, oi1, e1, i1)) { e1 = oe1; i1 = oi1; }
            if (better(oe2, oi2, e2, i2)) { e2 = oe2; i2 = oi2; }
        }
        __shared__ double se[2][8];
        __shared__ long long si[2][8];
        const int tid = threadIdx.x + threadIdx.y * blockDim.x;
        if ((tid & 31) == 0) { se[0][tid >> 5] = e1; se[1][tid >> 5] = e2; si[0][tid >> 5] = i1; si[1][tid >> 5] = i2; }
        __syncthreads();
        if (tid == 0) {
            const int nw = (blockDim.x * blockDim.y + 31) / 32;
            for (int k = 1; k < nw; ++k) {
                if (better(se[0][k], si[0][k], e1, i1)) { e1 = se[0][k]; i1 = si[0][k]; }
                if (better(se[1][k], si[1][k], e2, i2)) { e2 = se[1][k]; i2 = si[1][k]; }
            }
            double* mp = mpart + 4 * (blockIdx.y * gridDim.x + blockIdx.x);
            mp[0] = e1; mp[1] = (double)i1; mp[2] = e2; mp[3] = (double)i2;
        }
    }
}

// Once per step, after the three stages: dtbar = sum_s c_s part_s (c = 1, 1/4, 2/3 for stages
// 1, 2, 3), then g += dtbar * ddt/dM_x * dM_x/du0 + dtbar * ddt/dM_y * dM_y/du0 at the cells of
// the maxima, with dt = cfl/(M_x/dx + M_y/dy): ddt/dM_x = -dt^2/(cfl dx).
__global__ void __launch_bounds__(256) k_dt(AdjParams a, const double* __restrict__ part, int npart,
                                            const double* __restrict__ mpart, int nm,
                                            const double* __restrict__ u0, double* __restrict__ g,
                                            const double* __restrict__ dtp, int* __restrict__ argmax) {
    const int t = threadIdx.x;
    double s = 0.0;
    for (int k = t; k < 3 * npart; k += blockDim.x) {
        const int st = k / npart;
        s += (st == 0 ? 1.0 : st == 1 ? 0.25 : 2.0 / 3.0) * part[k];
    }
    double e1 = -1.0, e2 = -1.0, i1 = 1e300, i2 = 1e300;
    for (int k = t; k < nm; k += blockDim.x) {
        const double* mp = mpart + 4 * k;
        if (mp[0] > e1 || (mp[0] == e1 && mp[1] < i1)) { e1 = mp[0]; i1 = mp[1]; }
        if (mp[2] > e2 || (mp[2] == e2 && mp[3] < i2)) { e2 = mp[2]; i2 = mp[3]; }
    }
    __shared__ double rs[256], re1[256], re2[256], ri1[256], ri2[256];
    rs[t] = s; re1[t] = e1; re2[t] = e2; ri1[t] = i1; ri2[t] = i2;
    __syncthreads();
    for (int h = blockDim.x / 2; h; h >>= 1) {
        if (t < h) {
            rs[t] += rs[t + h];
            if (re1[t + h] > re1[t] || (re1[t + h] == re1[t] && ri1[t + h] < ri1[t])) { re1[t] = re1[t + h]; ri1[t] = ri1[t + h]; }
            if (re2[t + h] > re2[t] || (re2[t + h] == re2[t] && ri2[t + h] < ri2[t])) { re2[t] = re2[t + h]; ri2[t] = ri2[t + h]; }
        }
        __syncthreads();
    }
    if (t == 0) {
        const double dt = *dtp, dtbar = rs[0];
        // no cell holds a finite maximum (a NaN state): nothing to differentiate
        if (!(ri1[0] >= 0.0 && ri1[0] < (double)a.plane && ri2[0] >= 0.0 && ri2[0] < (double)a.plane)) return;
        const long long c1 = (long long)ri1[0], c2 = (long long)ri2[0];
        argmax[0] = (int)c1;
        argmax[1] = (int)c2;
        const double k1 = -dtbar * dt * dt / (a.cfl * a.dx), k2 = -dtbar * dt * dt / (a.cfl * a.dy);
        double U[4], Ub[4] = {0, 0, 0, 0};
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = u0[v * a.plane + c1];
        wave_speed_vjp<0>(U, a.gamma, k1, Ub);
#pragma unroll
        for (int v = 0; v < 4; ++v) g[v * a.plane + c1] += Ub[v];
#pragma unroll
        for (int v = 0; v < 4; ++v) { U[v] = u0[v * a.plane + c2]; Ub[v] = 0.0; }
        wave_speed_vjp<1>(U, a.gamma, k2, Ub);
#pragma unroll
        for (int v = 0; v < 4; ++v) g[v * a.plane + c2] += Ub[v];
    }
}

__global__ void k_loop(Scalars* sc) {
    sc->t = 0.0;
    sc->step = 0;
    sc->t_end = 1e300;
    sc->total_step = LLONG_MAX;
}

}  // namespace adj
}  // namespace dense

// ---------------------------------------------------------------------------------------------
// Host side
using dense::kB;
using dense::adj::AdjParams;

namespace {

constexpr int kFX = 32, kFY = 4;   // face kernel tiles (xi: faces x rows; eta: columns x faces)
constexpr int kCX = 32, kCY = 8;   // cell kernel blocks

thread_local std::string g_adj_err;

}  // namespace

struct dense_adjoint {
    dense_handle_t* h = nullptr;  // the forward solver: its buffers, kernels and step graph
    dense_config_t cfg{};
    int k = 20;                   // checkpoint every k steps
    int ni = 0, nj = 0;
    size_t state = 0;             // doubles per compact state: 4 ni nj
    AdjParams ap{};
    double* ckpt = nullptr;  int ckpt_cap = 0;  // states at steps 0, k, 2k, ...
    double* dts = nullptr;   int dts_cap = 0;   // dt of every forward step
    int* argmax = nullptr;   int argmax_cap = 0;  // per step: cells of the two maxima
    double* rec = nullptr;                      // k steps x 3 stage states of one segment
    double *g = nullptr, *g1 = nullptr, *g2 = nullptr, *acc = nullptr;
    double *Gx = nullptr, *Gy = nullptr;
    double* part = nullptr;  int npart = 0, nbx = 0;  // per stage: xi then eta face blocks
    double* mpart = nullptr; int nm = 0;
    dim3 gx, gy, gc;
    int nsteps = -1;                            // steps of the last forward
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    long long launches = 0;
    std::string err;
};

namespace {

int aerr(dense_adjoint* a, int code, const std::string& msg) {
    if (a) a->err = msg; else g_adj_err = msg;
    return code;
}

#define ACK(a, call)                                                                             \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return aerr((a), DENSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define AH(a, call)                                                                              \
    do {                                                                                         \
        int r_ = (call);                                                                         \
        if (r_ != DENSE_OK) return aerr((a), r_, std::string("forward solver: ") + dense_last_error((a)->h)); \
    } while (0)

// compact interior state <-> the forward solver's padded cons
int to_solver(dense_adjoint* a, const double* src) {
    dense_handle* h = a->h;
    const size_t plane = (size_t)h->NJp * h->P;
    for (int v = 0; v < 4; ++v)
        ACK(a, cudaMemcpy2DAsync(h->cons + v * plane + (size_t)kB * h->P + kB, (size_t)h->P * sizeof(double),
                                 src + (size_t)v * a->ni * a->nj, (size_t)a->ni * sizeof(double),
                                 (size_t)a->ni * sizeof(double), a->nj, cudaMemcpyDeviceToDevice, h->stream));
    h->uploaded = true;
    h->prim_slot = -1;
    return DENSE_OK;
}
int from_solver(dense_adjoint* a, double* dst) {
    dense_handle* h = a->h;
    const size_t plane = (size_t)h->NJp * h->P;
    for (int v = 0; v < 4; ++v)
        ACK(a, cudaMemcpy2DAsync(dst + (size_t)v * a->ni * a->nj, (size_t)a->ni * sizeof(double),
                                 h->cons + v * plane + (size_t)kB * h->P + kB, (size_t)h->P * sizeof(double),
                                 (size_t)a->ni * sizeof(double), a->nj, cudaMemcpyDeviceToDevice, h->stream));
    return DENSE_OK;
}

int begin(dense_adjoint* a, void* stream) {
    ACK(a, cudaEventRecord(a->ev_in, (cudaStream_t)stream));
    ACK(a, cudaStreamWaitEvent(a->h->stream, a->ev_in, 0));
    return DENSE_OK;
}
int finish(dense_adjoint* a, void* stream) {
    ACK(a, cudaGetLastError());
    ACK(a, cudaEventRecord(a->ev_out, a->h->stream));
    ACK(a, cudaStreamWaitEvent((cudaStream_t)stream, a->ev_out, 0));
    return DENSE_OK;
}

// restart the forward solver from a state: loop bounds open, get_primary of the state
int restart(dense_adjoint* a, const double* state) {
    int rc = to_solver(a, state);
    if (rc) return rc;
    dense::adj::k_loop<<<1, 1, 0, a->h->stream>>>(a->h->sc);
    a->launches += 1;
    AH(a, dense::handle_ensure_prim(a->h, 0));
    a->launches += 1;
    return DENSE_OK;
}

template <int REC>
void launch_vjp(dense_adjoint* a, int stage, const double* u, const double* w, double* out, double* part,
                const double* dtp, cudaStream_t s) {
    using namespace dense::adj;
    const dim3 bf(kFX, kFY), bc(kCX, kCY);
    k_face<0, REC, kFX, kFY><<<a->gx, bf, 0, s>>>(a->ap, u, w, a->Gx, part);
    k_face<1, REC, kFX, kFY><<<a->gy, bf, 0, s>>>(a->ap, u, w, a->Gy, part + a->nbx);
    switch (stage) {
    case 3: k_cell<3><<<a->gc, bc, 0, s>>>(a->ap, u, w, a->Gx, a->Gy, a->acc, out, dtp, nullptr); break;
    case 2: k_cell<2><<<a->gc, bc, 0, s>>>(a->ap, u, w, a->Gx, a->Gy, a->acc, out, dtp, nullptr); break;
    case 1: k_cell<1><<<a->gc, bc, 0, s>>>(a->ap, u, w, a->Gx, a->Gy, a->acc, out, dtp, a->mpart); break;
    default: k_cell<0><<<a->gc, bc, 0, s>>>(a->ap, u, w, a->Gx, a->Gy, nullptr, out, nullptr, nullptr); break;
    }
    a->launches += 3;
}

void vjp(dense_adjoint* a, int stage, const double* u, const double* w, double* out, double* part,
         const double* dtp) {
    cudaStream_t s = a->h->stream;
    switch (a->cfg.recon) {
    case DENSE_RECON_UPWIND5: launch_vjp<DENSE_RECON_UPWIND5>(a, stage, u, w, out, part, dtp, s); break;
    case DENSE_RECON_WENOJS5: launch_vjp<DENSE_RECON_WENOJS5>(a, stage, u, w, out, part, dtp, s); break;
    default:                  launch_vjp<DENSE_RECON_WENOZ5>(a, stage, u, w, out, part, dtp, s); break;
    }
}

// reverse of one step from its three recorded stage states; g holds dJ/du(n+1) on entry and
// dJ/du(n) on return
void reverse_step(dense_adjoint* a, const double* rec_step, int step) {
    const double* dtp = a->dts + step;
    const double* u0 = rec_step;
    const double* u1 = rec_step + a->state;
    const double* u2 = rec_step + 2 * a->state;
    vjp(a, 3, u2, a->g, a->g2, a->part + 2 * a->npart, dtp);
    vjp(a, 2, u1, a->g2, a->g1, a->part + 1 * a->npart, dtp);
    vjp(a, 1, u0, a->g1, a->g, a->part, dtp);
    if (!a->cfg.if_const_dt) {
        dense::adj::k_dt<<<1, 256, 0, a->h->stream>>>(a->ap, a->part, a->npart, a->mpart, a->nm, u0, a->g, dtp,
                                                      a->argmax + 2 * step);
        a->launches += 1;
    }
}

template <class T>
int grow(dense_adjoint* a, T** p, int* cap, int need, size_t unit) {
    if (*cap >= need) return DENSE_OK;
    if (*p) ACK(a, cudaFree(*p));
    *p = nullptr;
    *cap = 0;
    ACK(a, cudaMalloc((void**)p, (size_t)need * unit * sizeof(T)));
    *cap = need;
    return DENSE_OK;
}

}  // namespace

extern "C" {

const char* dense_adjoint_last_error(dense_adjoint_t* a) { return a ? a->err.c_str() : g_adj_err.c_str(); }

long long dense_adjoint_launch_count(dense_adjoint_t* a) { return a ? a->launches : -1; }

void dense_adjoint_destroy(dense_adjoint_t* a) {
    if (!a) return;
    if (a->h) cudaStreamSynchronize(a->h->stream);
    double* bufs[] = {a->ckpt, a->dts, a->rec, a->g, a->g1, a->g2, a->acc, a->Gx, a->Gy, a->part, a->mpart};
    for (double* b : bufs) if (b) cudaFree(b);
    if (a->argmax) cudaFree(a->argmax);
    if (a->ev_in) cudaEventDestroy(a->ev_in);
    if (a->ev_out) cudaEventDestroy(a->ev_out);
    if (a->h) dense_destroy(a->h);
    delete a;
}

int dense_adjoint_create(const dense_config_t* cfg, int checkpoint_every, dense_adjoint_t** out) {
    if (!out || !cfg) return aerr(nullptr, DENSE_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->splitting != DENSE_SPLIT_LLF)
        return aerr(nullptr, DENSE_ERR_ARG, "the adjoint covers the LLF splitting (101) only");
    if (cfg->recon != DENSE_RECON_UPWIND5 && cfg->recon != DENSE_RECON_WENOJS5 && cfg->recon != DENSE_RECON_WENOZ5)
        return aerr(nullptr, DENSE_ERR_ARG, "the adjoint covers reconstructions 251, 253 and 255");
    if (cfg->benchmark != DENSE_BENCH_IVC_PERIODIC && cfg->benchmark != DENSE_BENCH_RM_PERIODIC)
        return aerr(nullptr, DENSE_ERR_ARG, "the adjoint needs a grid periodic in x and y (benchmarks 11, 14)");
    if (cfg->ni < 8 || cfg->nj < 8) return aerr(nullptr, DENSE_ERR_ARG, "the adjoint needs ni, nj >= 8");
    if (checkpoint_every < 1) return aerr(nullptr, DENSE_ERR_ARG, "checkpoint_every must be >= 1");
    auto* a = new dense_adjoint();
    a->cfg = *cfg;
    a->k = checkpoint_every;
    a->ni = cfg->ni;
    a->nj = cfg->nj;
    a->state = (size_t)4 * cfg->ni * cfg->nj;
    int rc = dense_create(cfg, &a->h);
    if (rc) {
        g_adj_err = std::string("forward solver: ") + dense_last_error(nullptr);
        delete a;
        return rc;
    }
    auto fail = [&](int code) {
        g_adj_err = a->err;
        dense_adjoint_destroy(a);
        return code;
    };
    AdjParams& p = a->ap;
    p.ni = cfg->ni; p.nj = cfg->nj; p.plane = (long long)cfg->ni * cfg->nj;
    p.gamma = cfg->gamma; p.dx = cfg->dx; p.dy = cfg->dy; p.inv_dx = 1.0 / cfg->dx; p.inv_dy = 1.0 / cfg->dy;
    p.cfl = cfg->cfl;
    a->gx = dim3((cfg->ni + 1 + kFX - 1) / kFX, (cfg->nj + kFY - 1) / kFY);
    a->gy = dim3((cfg->ni + kFX - 1) / kFX, (cfg->nj + 1 + kFY - 1) / kFY);
    a->gc = dim3((cfg->ni + kCX - 1) / kCX, (cfg->nj + kCY - 1) / kCY);
    a->nbx = (int)(a->gx.x * a->gx.y);
    a->npart = a->nbx + (int)(a->gy.x * a->gy.y);
    a->nm = (int)(a->gc.x * a->gc.y);
    const size_t fx = (size_t)40 * cfg->nj * (cfg->ni + 1), fy = (size_t)40 * (cfg->nj + 1) * cfg->ni;
    struct B { double** p; size_t n; } bufs[] = {
        {&a->g, a->state}, {&a->g1, a->state}, {&a->g2, a->state}, {&a->acc, a->state},
        {&a->Gx, fx}, {&a->Gy, fy}, {&a->part, (size_t)3 * a->npart}, {&a->mpart, (size_t)4 * a->nm},
        {&a->rec, (size_t)3 * a->k * a->state},
    };
    for (auto& b : bufs) {
        cudaError_t e = cudaMalloc((void**)b.p, b.n * sizeof(double));
        if (e != cudaSuccess) { a->err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return fail(DENSE_ERR_NOMEM); }
    }
    if (cudaEventCreateWithFlags(&a->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&a->ev_out, cudaEventDisableTiming) != cudaSuccess) {
        a->err = "cudaEventCreate failed";
        return fail(DENSE_ERR_CUDA);
    }
    *out = a;
    return DENSE_OK;
}

int dense_adjoint_forward(dense_adjoint_t* a, const double* u0, int nsteps, double* uT, void* stream) {
    if (!a || !u0 || !uT) return aerr(a, DENSE_ERR_ARG, "null argument");
    if (nsteps < 0) return aerr(a, DENSE_ERR_ARG, "nsteps < 0");
    const int nseg = (nsteps + a->k - 1) / a->k;
    int rc = grow(a, &a->ckpt, &a->ckpt_cap, nseg > 0 ? nseg : 1, a->state);
    if (!rc) rc = grow(a, &a->dts, &a->dts_cap, nsteps > 0 ? nsteps : 1, 1);
    if (!rc) rc = grow(a, &a->argmax, &a->argmax_cap, nsteps > 0 ? nsteps : 1, 2);
    if (rc) return rc;
    ACK(a, cudaMemsetAsync(a->argmax, 0xff, (size_t)2 * a->argmax_cap * sizeof(int), a->h->stream));
    a->nsteps = -1;
    rc = begin(a, stream);
    if (!rc) rc = restart(a, u0);
    if (rc) return rc;
    AH(a, dense::handle_step_graph(a->h));
    dense_handle* h = a->h;
    for (int s = 0; s < nsteps; ++s) {
        if (s % a->k == 0) {
            rc = from_solver(a, a->ckpt + (size_t)(s / a->k) * a->state);
            if (rc) return rc;
        }
        ACK(a, cudaGraphLaunch(h->step_graph, h->stream));
        a->launches += h->graph_nodes;
        ACK(a, cudaMemcpyAsync(a->dts + s, &h->sc->dt, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    }
    rc = from_solver(a, uT);
    if (rc) return rc;
    a->nsteps = nsteps;
    return finish(a, stream);
}

int dense_adjoint_backward(dense_adjoint_t* a, const double* gT, double* g0, void* stream) {
    if (!a || !gT || !g0) return aerr(a, DENSE_ERR_ARG, "null argument");
    if (a->nsteps < 0) return aerr(a, DENSE_ERR_STATE, "dense_adjoint_backward before dense_adjoint_forward");
    int rc = begin(a, stream);
    if (rc) return rc;
    dense_handle* h = a->h;
    ACK(a, cudaMemcpyAsync(a->g, gT, a->state * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    const int nseg = (a->nsteps + a->k - 1) / a->k;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int s0 = seg * a->k, len = std::min(a->k, a->nsteps - s0);
        rc = restart(a, a->ckpt + (size_t)seg * a->state);
        if (rc) return rc;
        // recompute the segment, recording each stage's input state
        for (int s = 0; s < len; ++s) {
            h->kt->step_begin(h->prm, h->stream);
            for (int irk = 1; irk <= 3; ++irk) {
                rc = from_solver(a, a->rec + ((size_t)s * 3 + irk - 1) * a->state);
                if (rc) return rc;
                h->kt->bc(h->prm, h->stream);
                h->kt->flux(h->prm, irk, 0, h->stream);
                h->kt->flux(h->prm, irk, 1, h->stream);
                h->kt->update(h->prm, irk, h->stream);
            }
            h->kt->step_end(h->prm, h->stream);
            a->launches += 2 + 3 * dense::handle_stage_launches(h);
        }
        for (int s = len - 1; s >= 0; --s) reverse_step(a, a->rec + (size_t)s * 3 * a->state, s0 + s);
    }
    h->prim_slot = -1;
    ACK(a, cudaMemcpyAsync(g0, a->g, a->state * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return finish(a, stream);
}

int dense_adjoint_rhs_vjp(dense_adjoint_t* a, const double* u, const double* v, double* out, double* vdotl,
                          void* stream) {
    if (!a || !u || !v || !out) return aerr(a, DENSE_ERR_ARG, "null argument");
    int rc = begin(a, stream);
    if (rc) return rc;
    vjp(a, 0, u, v, out, a->part, nullptr);
    std::vector<double> part(a->npart);
    ACK(a, cudaMemcpyAsync(part.data(), a->part, a->npart * sizeof(double), cudaMemcpyDeviceToHost, a->h->stream));
    rc = finish(a, stream);
    if (rc) return rc;
    ACK(a, cudaStreamSynchronize(a->h->stream));
    double s = 0.0;
    for (double x : part) s += x;
    if (vdotl) *vdotl = s;
    return DENSE_OK;
}

int dense_adjoint_get_dts(dense_adjoint_t* a, double* dts, int n) {
    if (!a || !dts) return aerr(a, DENSE_ERR_ARG, "null argument");
    if (n < 0 || n > a->nsteps) return aerr(a, DENSE_ERR_ARG, "n exceeds the steps of the last forward");
    if (n == 0) return DENSE_OK;
    ACK(a, cudaMemcpyAsync(dts, a->dts, n * sizeof(double), cudaMemcpyDeviceToHost, a->h->stream));
    ACK(a, cudaStreamSynchronize(a->h->stream));
    return DENSE_OK;
}

int dense_adjoint_get_argmax(dense_adjoint_t* a, int* idx, int n) {
    if (!a || !idx) return aerr(a, DENSE_ERR_ARG, "null argument");
    if (n < 0 || n > a->nsteps) return aerr(a, DENSE_ERR_ARG, "n exceeds the steps of the last forward");
    if (n == 0) return DENSE_OK;
    ACK(a, cudaMemcpyAsync(idx, a->argmax, (size_t)2 * n * sizeof(int), cudaMemcpyDeviceToHost, a->h->stream));
    ACK(a, cudaStreamSynchronize(a->h->stream));
    return DENSE_OK;
}

}  // extern "C"
