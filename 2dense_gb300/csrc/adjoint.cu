// adjoint.cu — the discrete adjoint of the plain solver's time step: LLF, GLF or Steger-Warming
// splitting (101, 102, 103) with upwind5 / WENO-JS5 / WENO-Z5 reconstruction (251/253/255), or
// the characteristic WENO-Z scheme (104, k_char_face) and AdaWENO (105, the same kernel with the
// branches the forward took), and TVD-RK3 with the CFL time step, on
// grids periodic in x and y (benchmarks 11 and 14) or with extrapolated, mirror, fixed-state and
// time-dependent inflow sides (benchmarks 1, 2, 3, 4, 5, 6, 9, 13; wall_terms).
//
// The forward step (time_rk3_general, time_advance_general.f90:9-267) applies per stage
//     L(u)_c = -(h_{f+1} - h_f)/dx - (g_{f'+1} - g_{f'})/dy,     cell c between faces f, f+1,
//     h_f = W(F+ of cells f-3..f+1) + W(F- of cells f+2..f-2)    (cells in interior indices,
// ghosts are periodic images or built by a wall rule), F+- = 0.5((u_n +- lambda) U + P),
// lambda = |u_n| + alpha of the cell (flux_splitting_LLF.f90:67-81), W one of the 5-point
// reconstructions
// (scheme_weno5js_general.f90, scheme_weno5z_general.f90, scheme_upwind5_general.f90), and
//     u1 = u0 + dt L(u0),  u2 = 3/4 u0 + 1/4 u1 + 1/4 dt L(u1),  u3 = 1/3 u0 + 2/3 u2 + 2/3 dt L(u2)
// with dt = cfl / (max(|u|+alpha)/dx + max(|v|+alpha)/dy) of u0.
//
// FP64 is the scarce resource on GB300 (about 1.3 TFLOP/s against 7.9 TB/s of HBM), so the
// reverse sweep does not re-evaluate the reconstructions: when a segment is recomputed from its
// checkpoint, the flux sweeps run in their taping form (flux_tape of the kernel table), which
// writes, per face, the gradient g[m] = dW/dlf[m] of each of its 8 reconstructions and the
// fluxes h -- 352 bytes per face and direction, read back once. The vector-Jacobian product
// v -> (dL/du)^T v of a stage is then two light kernels:
//   k_hbar (one thread per face, both directions): hbar_f = (v_right - v_left)/dx, and the
//     face's share h_f . hbar_f of v . L(u) (summation by parts), summed per block;
//   k_rev (one thread per cell): for every face whose stencils read the cell or one of its
//     periodic images, hbar_f g[m] accumulated in a fixed order into the sensitivities of the
//     cell's F+ and F-; the transposed Jacobian of F+- at the cell (both directions); the
//     reverse of the RK stage;
// and once per step k_dt (one block): the time step's sensitivity sum_s c_s v_s . L(u_{s-1}),
// sent through dt(max wave speeds) to the cells where the maxima are attained.
// GLF (flux_splitting_GLF.f90:13-70) splits with the stage's global lambda = max over the cells
// of |u_n| + alpha of the stage input instead of the cell's own: k_maxarg / k_maxred find that
// maximum and its cell before the stage's reverse, k_rev uses it as a constant and sums the
// sensitivity of lambda over all cells per block, and k_lamg sends the total through lambda to
// the cell of the maximum (the gradient of a max flows to its argmax, ties to the lowest cell).
// Steger-Warming (flux_splitting_SW.f90:14-168) splits each cell's flux with the three eigenvalues
// u_n, u_n -+ alpha of the cell alone; its transposed Jacobian is taken exactly in forward mode:
// the split, written once over a dual-number type, is evaluated with each conserved variable of
// the cell seeded in turn (four passes), and the sensitivities of F+ and F- contract the columns.
// No atomics: every sum has a fixed order, so the gradient is deterministic.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fastmath.cuh"
#include "handle.h"
#include "nvtx.h"

namespace dense {
namespace adj {

#include "weno_fast.cuh"
constexpr double kPFloor = (double)1.0e-6f;  // get_primary.f90:58

struct AdjParams {
    int ni, nj;
    long long plane;  // ni * nj: one variable of a compact interior state
    long long xs, ys; // face planes: xi nj (ni+1), eta (nj+1) ni
    int np;           // tape planes per direction (tape_planes; 4 for 104, the fluxes alone)
    int gnp;          // planes per direction of what the cell kernel gathers: the tape (np), or
                      // the characteristic scheme's face sensitivities of the split fluxes (40)
    double gamma, dx, dy, inv_dx, inv_dy, cfl;
    int rule[4];      // ghost rule of each side (bottom, top, left, right): kRulePeriodic, ...
    // Rayleigh-Taylor's body force: each stage adds f_s (0, 0, rho, rho v) of its input, f_s =
    // dt, dt/4, (2/3 in single precision) dt (time_advance_general.f90:79,160,242); the
    // stages' per-block sums of w . (0, 0, rho, rho v) for the time step's sensitivity go to
    // bpart[(s - 1) nm + block]
    int bodyforce;
    double* bpart;
    int bench;        // the benchmark (its fixed ghost states: fixed_state)
    // characteristic WENO-Z (104, 105): k_char_face writes each face's split-flux sensitivities
    // (what the cell kernel gathers, kRecFaceSens) and, per face, the sensitivities of the
    // primitives (rho, u, v, p) of its left and right cells through the Roe eigenvectors:
    // rbar[8][face plane] a direction (left cell 0..3, right cell 4..7), xi then eta
    int charac;
    double* rbar;
    // AdaWENO (105): the smooth branch's surrogate rho + F(normal momentum) adds the density
    // sensitivities of its stencil cells, planes 40 + s*5 + m of the gathered face array
    int adapt;
    // the shock / shear layer (6): the rows' cell-centre y (the inflow's profile); the stages'
    // per-block sums of the inflow ghosts' time sensitivity (tpart[(s - 1) nm + block]); tacc[0]
    // the running sum, over the steps already reversed, of the loss's sensitivity to their start
    // times, which every earlier time step moves
    int ssl;
    const double* yleft;
    double* tpart;
    double* tacc;
};
// Ghost rules of the benchmarks the adjoint covers (boundary_*_general.f90): a periodic copy,
// the recursive 4/3, -1/3 extrapolation of the two cells next to the side, the mirror of the
// four cells next to it with the normal velocity negated -- applied to the conserved variables
// and, separately, to the primitives -- or a fixed state (Rayleigh-Taylor's Dirichlet bottom and
// top, boundary_rt_general.f90:14-57), which no interior cell feeds.
constexpr int kRulePeriodic = 0, kRuleExtrap = 1, kRuleReflect = 2, kRuleFixed = 3;
// the double Mach reflection's bottom: the mirror where the column's centre x >= 1/6, the fixed
// post-shock state before it (boundary_doublemach_general.f90:14-48)
constexpr int kRuleDMRBottom = 4;
// the shock / shear layer's left inflow (boundary_ssl_general.f90:40-66): a state per row that
// oscillates in the step's start time, which the time steps make a function of the state
constexpr int kRuleSSLInflow = 5;
constexpr double kTwoThirdsSingle = (double)(2.0f / 3.0f);  // time_advance_general.f90:242

// get_primary of one cell (get_primary.f90:53-60), with the pressure floor of :58; rs = 1/alpha'
// with alpha'^2 = gamma p / rho, so that alpha = alpha'^2 rs and dalpha/dp = gamma/(2 rho) rs.
struct Prim {
    double u, v, p, a, ir, rs;
    bool floored;
};
__device__ __forceinline__ Prim prim_of(const double U[4], double gamma) {
    Prim q;
    q.ir = rcp_nr(U[0]);
    q.u = U[1] * q.ir;
    q.v = U[2] * q.ir;
    q.p = (gamma - 1.0) * (U[3] - 0.5 * U[0] * (q.u * q.u + q.v * q.v));
    q.floored = q.p < 0.0;
    if (q.floored) q.p = kPFloor;
    const double a2 = gamma * q.p * q.ir;
    q.rs = rsqrt_nr(a2);
    q.a = a2 * q.rs;
    return q;
}

// Sensitivities of all primitives (rho, u, v, p, alpha) pulled back to the conserved variables.
__device__ __forceinline__ void prim_pullback_all(const double U[4], const Prim& q, double gamma, double rhob,
                                                  double ub, double vb, double pb, double ab, double Ub[4]) {
    double rb = rhob - ab * 0.5 * q.a * q.ir;
    if (!q.floored) pb += ab * (0.5 * gamma) * q.ir * q.rs;
    Ub[1] += ub * q.ir;
    Ub[2] += vb * q.ir;
    rb -= (ub * q.u + vb * q.v) * q.ir;
    if (!q.floored) {
        const double g1 = gamma - 1.0;
        Ub[3] += g1 * pb;
        Ub[1] -= g1 * q.u * pb;
        Ub[2] -= g1 * q.v * pb;
        rb += g1 * 0.5 * (q.u * q.u + q.v * q.v) * pb;
    }
    Ub[0] += rb;
}

// Sensitivities of (u_n, alpha, p) pulled back to the conserved variables of the cell.
template <int DIR>
__device__ __forceinline__ void prim_pullback(const double U[4], const Prim& q, double gamma, double unb,
                                              double ab, double pb, double Ub[4]) {
    // alpha = sqrt(gamma p / rho): dalpha/dp = gamma/(2 alpha rho), dalpha/drho = -alpha/(2 rho)
    double rb = -ab * 0.5 * q.a * q.ir;
    if (!q.floored) pb += ab * (0.5 * gamma) * q.ir * q.rs;
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

// Ub += (dF+/dU)^T gp + (dF-/dU)^T gm at one cell, direction DIR, with F+- = 0.5((u_n +- lambda)
// U + P): LLF's lambda = |u_n| + alpha of the cell is pulled back here; GLF's lambda (lam_g, the
// global maximum) is a constant at the cell, and its sensitivity is returned for the caller to
// send to the cell of the maximum.
// The split's sensitivities at one cell in terms of its own U and primitives (u_n, p, alpha),
// as a ghost cell holds them (its primitives come from the ghost rule, not from its U): Ub +=
// dF/dU^T g, and unb, pb, ab; returns lambda's sensitivity (GLF).
template <int DIR, bool GLF>
__device__ __forceinline__ double llf_bar(const double U[4], double un, double p, double alpha, const double gp[4],
                                          const double gm[4], double lam_g, double Ub[4], double& unb, double& pb,
                                          double& ab) {
    const double s = un >= 0.0 ? 1.0 : -1.0;
    const double lam = GLF ? lam_g : s * un + alpha;
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
    unb = Sp + Sm + 0.5 * p * g3 + (GLF ? 0.0 : s * lamb);
    pb = 0.5 * (gp[1 + DIR] + gm[1 + DIR]) + 0.5 * un * g3;
    ab = GLF ? 0.0 : lamb;
    return lamb;
}

template <int DIR, bool GLF>
__device__ __forceinline__ double llf_vjp(const double U[4], const Prim& q, double gamma, const double gp[4],
                                          const double gm[4], double lam_g, double Ub[4]) {
    const double un = DIR == 0 ? q.u : q.v;
    const double s = un >= 0.0 ? 1.0 : -1.0;
    const double lam = GLF ? lam_g : s * un + q.a;
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
    const double unb = Sp + Sm + 0.5 * q.p * g3 + (GLF ? 0.0 : s * lamb);
    const double pb = 0.5 * (gp[1 + DIR] + gm[1 + DIR]) + 0.5 * un * g3;
    prim_pullback<DIR>(U, q, gamma, unb, GLF ? 0.0 : lamb, pb, Ub);
    return lamb;
}

// ---- Steger-Warming: exact Jacobian columns in forward mode ---------------------------------
// A value and its derivative along one seed direction.
struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, fma(a.d, b.v, a.v * b.d)}; }
__device__ __forceinline__ Dual operator*(double c, Dual a) { return {c * a.v, c * a.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double r = rcp_nr(b.v), q = a.v * r;
    return {q, (a.d - q * b.d) * r};
}
__device__ __forceinline__ Dual operator/(Dual a, double c) { return {a.v / c, a.d / c}; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
    const double rs = rsqrt_nr(a.v), s = a.v * rs;
    return {s, 0.5 * a.d * rs};
}

// The Steger-Warming split of one cell in direction DIR from its conserved variables: get_primary
// (get_primary.f90:53-60, with the pressure floor of :58), then flux_splitting_SW.f90:42-91 (xi)
// / :110-160 (eta) -- eigenvalues l1 = u_n, l2 = u_n - alpha, l3 = u_n + alpha split as
// (l +- sqrt(l^2 + eps^2))/2 with eps = 0.125.
template <int DIR>
__device__ __forceinline__ void sw_split_prim_dual(Dual rho, Dual u, Dual v, Dual a, double gamma, Dual fp[4],
                                                   Dual fm[4]) {
    const Dual uu2 = u * u + v * v;
    const double eps2 = 0.125 * 0.125, g1 = gamma - 1.0, c2g = 1.0 / (2.0 * gamma);
    const Dual un = DIR == 0 ? u : v, ut = DIR == 0 ? v : u;
    const Dual l1 = un, l2 = un - a, l3 = un + a;
    const Dual e{eps2, 0.0};
    const Dual s1 = dsqrt(l1 * l1 + e), s2 = dsqrt(l2 * l2 + e), s3 = dsqrt(l3 * l3 + e);
    const Dual q2 = l2 * l2 + ut * ut, q3 = l3 * l3 + ut * ut;
    const Dual crho = c2g * rho;
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
        const Dual p1 = 0.5 * (sg == 0 ? l1 + s1 : l1 - s1);
        const Dual p2 = 0.5 * (sg == 0 ? l2 + s2 : l2 - s2);
        const Dual p3 = 0.5 * (sg == 0 ? l3 + s3 : l3 - s3);
        const Dual wii = ((3.0 - gamma) / (2.0 * g1)) * ((p2 + p3) * (a * a));
        const Dual A = (2.0 * g1) * p1;
        Dual* f = sg == 0 ? fp : fm;
        f[0] = (A + p2 + p3) * crho;
        f[1 + DIR] = (A * un + p2 * l2 + p3 * l3) * crho;
        f[2 - DIR] = ((A + p2 + p3) * ut) * crho;
        f[3] = (g1 * (p1 * uu2) + 0.5 * (p2 * q2) + 0.5 * (p3 * q3) + wii) * crho;
    }
}
template <int DIR>
__device__ __forceinline__ void sw_split_dual(const Dual U[4], double gamma, Dual fp[4], Dual fm[4]) {
    const Dual rho = U[0];
    const Dual u = U[1] / rho, v = U[2] / rho;
    Dual p = (gamma - 1.0) * (U[3] - 0.5 * (rho * (u * u + v * v)));
    if (p.v < 0.0) p = Dual{kPFloor, 0.0};
    const Dual a = dsqrt((gamma * p) / rho);
    sw_split_prim_dual<DIR>(rho, u, v, a, gamma, fp, fm);
}

// The Steger-Warming split's sensitivities at a ghost cell with respect to its primitives
// (rho, u, v, alpha; the split does not read U): pr += dF/dprim^T g, one forward pass each.
template <int DIR>
__device__ __forceinline__ void sw_prim_bar(const double pv[4], double gamma, const double gp[4], const double gm[4],
                                            double pr[4]) {
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        Dual q[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) q[c] = Dual{pv[c], c == k ? 1.0 : 0.0};
        Dual fp[4], fm[4];
        sw_split_prim_dual<DIR>(q[0], q[1], q[2], q[3], gamma, fp, fm);
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) acc = fma(gp[c], fp[c].d, fma(gm[c], fm[c].d, acc));
        pr[k] += acc;
    }
}

// Ub += (dF+/dU)^T gp + (dF-/dU)^T gm of the Steger-Warming split in both directions at one cell
// (g[d] the sensitivities of direction d's F+ then F-): one forward pass per conserved variable.
__device__ __forceinline__ void sw_vjp(const double U[4], double gamma, const double gpx[4], const double gmx[4],
                                       const double gpy[4], const double gmy[4], double Ub[4]) {
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        Dual Ud[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) Ud[c] = Dual{U[c], c == k ? 1.0 : 0.0};
        Dual fp[4], fm[4];
        double acc = 0.0;
        sw_split_dual<0>(Ud, gamma, fp, fm);
#pragma unroll
        for (int c = 0; c < 4; ++c) acc = fma(gpx[c], fp[c].d, fma(gmx[c], fm[c].d, acc));
        sw_split_dual<1>(Ud, gamma, fp, fm);
#pragma unroll
        for (int c = 0; c < 4; ++c) acc = fma(gpy[c], fp[c].d, fma(gmy[c], fm[c].d, acc));
        Ub[k] += acc;
    }
}

// Ub += scale * d(|u_n| + alpha)/dU at one cell.
template <int DIR>
__device__ __forceinline__ void wave_speed_vjp(const double U[4], double gamma, double scale, double Ub[4]) {
    const Prim q = prim_of(U, gamma);
    const double un = DIR == 0 ? q.u : q.v;
    prim_pullback<DIR>(U, q, gamma, (un >= 0.0 ? 1.0 : -1.0) * scale, scale, 0.0, Ub);
}

// Block-wide (max, lowest index) of two (value, cell) pairs; the result is valid in thread 0.
__device__ __forceinline__ bool argmax_better(double ea, long long ia, double eb, long long ib) {
    return ea > eb || (ea == eb && ia < ib);
}
__device__ __forceinline__ void block_argmax(double& e1, long long& i1, double& e2, long long& i2) {
#pragma unroll
    for (int s = 16; s; s >>= 1) {
        const double oe1 = __shfl_xor_sync(0xffffffffu, e1, s), oe2 = __shfl_xor_sync(0xffffffffu, e2, s);
        const long long oi1 = __shfl_xor_sync(0xffffffffu, i1, s), oi2 = __shfl_xor_sync(0xffffffffu, i2, s);
        if (argmax_better(oe1, oi1, e1, i1)) { e1 = oe1; i1 = oi1; }
        if (argmax_better(oe2, oi2, e2, i2)) { e2 = oe2; i2 = oi2; }
    }
    __shared__ double se[2][32];
    __shared__ long long si[2][32];
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if ((tid & 31) == 0) { se[0][tid >> 5] = e1; se[1][tid >> 5] = e2; si[0][tid >> 5] = i1; si[1][tid >> 5] = i2; }
    __syncthreads();
    if (tid == 0) {
        const int nw = (blockDim.x * blockDim.y + 31) / 32;
        for (int k = 1; k < nw; ++k) {
            if (argmax_better(se[0][k], si[0][k], e1, i1)) { e1 = se[0][k]; i1 = si[0][k]; }
            if (argmax_better(se[1][k], si[1][k], e2, i2)) { e2 = se[1][k]; i2 = si[1][k]; }
        }
    }
}

// Deterministic block sum of two values (fixed lane and warp order); valid in thread 0.
__device__ __forceinline__ void block_sum2(double& x, double& y) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    __shared__ double red2[2][32];
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((tid & 31) == 0) { red2[0][tid >> 5] = x; red2[1][tid >> 5] = y; }
    __syncthreads();
    if (tid == 0) {
        x = 0.0;
        y = 0.0;
        for (int w = 0; w < nw; ++w) { x += red2[0][w]; y += red2[1][w]; }
    }
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
// Face kernel, both directions (blockIdx.z): hbar per face and equation, and the block's share
// of v . L(u). Tape and hbar arrays follow the forward's face arrays: xi [nj][ni+1] planes, then
// eta [nj+1][ni] planes.
__global__ void __launch_bounds__(256) k_hbar(AdjParams a, const double* __restrict__ w,
                                              const double* __restrict__ tape, double* __restrict__ hb,
                                              double* __restrict__ part) {
    const int dir = blockIdx.z;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int ni = a.ni, nj = a.nj;
    const int line = dir == 0 ? y : x, f = dir == 0 ? x : y;
    const int nline = dir == 0 ? nj : ni, n = dir == 0 ? ni : nj;
    double vdl = 0.0;
    if (line < nline && f <= n) {
        const double inv = dir == 0 ? a.inv_dx : a.inv_dy;
        const long long oR = dir == 0 ? (long long)line * ni + f : (long long)f * ni + line;
        const long long oL = oR - (dir == 0 ? 1 : ni);
        const long long ts = dir == 0 ? a.xs : a.ys;
        const long long to = dir == 0 ? (long long)line * (ni + 1) + f : (long long)f * ni + line;
        const double* H = tape + (dir == 0 ? 0 : a.np * a.xs) + (long long)(a.np - 4) * ts + to;
        double* HB = hb + (dir == 0 ? 0 : 4 * a.xs) + to;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double wr = f < n ? w[v * a.plane + oR] : 0.0;   // face n is the right face of cell n-1 only
            const double wl = f >= 1 ? w[v * a.plane + oL] : 0.0;  // face 0 is the left face of cell 0 only
            const double hbv = (wr - wl) * inv;
            HB[v * ts] = hbv;
            vdl = fma(hbv, H[v * ts], vdl);
        }
    }
    const double s = block_sum(vdl);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
}

// Sensitivities of the F+ and F- values of cell x of a line (faces 0..n of the line, at offset
// base + f*stride of their planes): sum over the faces whose "+" stencil reads the cell
// (face x+3-m reads it as its m-th value) or whose "-" stencil does (face x-2+m), including the
// faces that read it through a periodic image (x -+ n). REC = kRecFaceSens: T holds the split
// fluxes' sensitivities themselves (the characteristic schemes' face kernel wrote them with the
// faces' hbar already applied), and H is not read.
constexpr int kRecFaceSens = 0;
template <int REC>
__device__ __forceinline__ void add_face(const double* __restrict__ T, const double* __restrict__ H, long long ts,
                                         long long off, int s, int m, double acc[4]) {
    constexpr double cu[5] = {2.0 / 60.0, -13.0 / 60.0, 47.0 / 60.0, 27.0 / 60.0, -3.0 / 60.0};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        if (REC == kRecFaceSens) {
            acc[v] += T[(long long)((s * 5 + m) * 4 + v) * ts + off];
        } else {
            const double g = REC == DENSE_RECON_UPWIND5 ? cu[m] : T[(long long)((s * 5 + m) * 4 + v) * ts + off];
            acc[v] = fma(g, H[v * ts + off], acc[v]);
        }
    }
}
template <int REC>
__device__ __forceinline__ void gather_line(const double* __restrict__ T, const double* __restrict__ H, long long ts,
                                            long long base, long long stride, int x, int n, bool periodic,
                                            double gp[4], double gm[4]) {
    if (x >= 3 && x <= n - 4) {  // every reading face inside 1..n-1: no images
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            add_face<REC>(T, H, ts, base + (long long)(x + 3 - m) * stride, 0, m, gp);
            add_face<REC>(T, H, ts, base + (long long)(x - 2 + m) * stride, 1, m, gm);
        }
        return;
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) {
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int f = s == 0 ? x + 3 - m : x - 2 + m;
            double* acc = s == 0 ? gp : gm;
            if (f >= 0 && f <= n) add_face<REC>(T, H, ts, base + (long long)f * stride, s, m, acc);
            if (!periodic) continue;
            if (f >= n) add_face<REC>(T, H, ts, base + (long long)(f - n) * stride, s, m, acc);  // image x - n
            if (f <= 0) add_face<REC>(T, H, ts, base + (long long)(f + n) * stride, s, m, acc);  // image x + n
        }
    }
}

// AdaWENO: the density sensitivity of cell x of a line (faces as gather_line) from the faces
// whose surrogate stencils read it, periodic images included.
__device__ __forceinline__ double gather_rho_line(const double* __restrict__ T, long long ts, long long base,
                                                  long long stride, int x, int n, bool periodic) {
    double acc = 0.0;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int f = s == 0 ? x + 3 - m : x - 2 + m;
            const double* R = T + (long long)(40 + s * 5 + m) * ts + base;
            if (f >= 0 && f <= n) acc += R[(long long)f * stride];
            if (!periodic) continue;
            if (f >= n) acc += R[(long long)(f - n) * stride];
            if (f <= 0) acc += R[(long long)(f + n) * stride];
        }
    }
    return acc;
}

// The ghost cells of a side with a wall rule that the interior cell (i, j) feeds, in direction
// DIR (0: the left and right sides of row j, 1: the bottom and top of column i): for each such
// ghost, its state rebuilt from the interior state by the rule, the sensitivities of its F+ and
// F- gathered from the faces whose stencils read it, the split's sensitivities in terms of the
// ghost's U and primitives (a ghost's primitives come from the rule, not from its U), and these
// sent back through the rule: into Ub directly, into pbar (rho, u, v, p, alpha of the cell) for
// the caller to pull back through get_primary. A mirror ghost k copies the cell k+1 in from the
// side (normal velocity negated); an extrapolated ghost k is w1_k c1 + w2_k c2 of the two cells
// next to the side (the recursion g = 4/3 near - 1/3 far unrolled), so both of those cells
// rebuild all four ghosts and take their shares. GLF: a ghost's lambda sensitivity goes to the
// global lambda once (lb, by the cell next to the side or the mirrored cell).
// Conserved variables of the fixed ghost state of side `side` of direction DIR at line `line`
// (a column for the bottom and top, a row for the sides), at the step's start time t:
// Rayleigh-Taylor's bottom (2, 0, 0, 1) and top (1, 0, 0, 2.5) (boundary_rt_general.f90:14-57);
// the double Mach reflection's inflow and bottom-before-the-wall post-shock state, and its top,
// post-shock ahead of the moving shock x < 1/6 + (1 + 20 t)/sqrt(3), pre-shock behind it
// (boundary_doublemach_general.f90:51-99). Same formulas as the boundary fill's state_from.
// The shear layer's inflow at row `line` and time t (boundary_ssl_general.f90:40-66: the same
// formulas as the boundary fill), and dv/dt, the only component that moves with t.
__device__ __forceinline__ void ssl_inflow(const AdjParams& a, int line, double t, double& rho, double& u, double& v,
                                           double& pr, double& dv) {
    const double yy = a.yleft[line];
    const double pie = 3.141592653589793115997963468544185161590576171875;
    rho = yy >= 0.0 ? 1.6374 : 0.3626;
    pr = 0.3327;
    u = 2.5 + 0.5 * tanh(2.0 * yy);
    const double e = exp(-(yy * yy) / 10.0), om = 2.0 * pie / (30.0 / 2.68);
    const double a1 = 2.0 * pie * t / (30.0 / 2.68), a2 = 2.0 * pie * 2.0 * t / (30.0 / 2.68) + pie / 2.0;
    v = 0.05 * cos(a1) * e + 0.05 * cos(a2) * e;
    dv = -0.05 * e * (om * sin(a1) + 2.0 * om * sin(a2));
}
__device__ __forceinline__ void fixed_state(const AdjParams& a, int dir, int side, int line, double t, double Ug[4],
                                            double* qg = nullptr) {
    double rho, u = 0.0, v = 0.0, pr;
    if (a.bench == DENSE_BENCH_SSL) {
        if (dir == 1) {  // the top: the setup's post-shock state, never refilled
            rho = 2.1101; u = 2.9709; v = -0.1367; pr = (double)0.4754f;
        } else {         // the left inflow at time t
            double dv;
            ssl_inflow(a, line, t, rho, u, v, pr, dv);
        }
    } else if (a.bench == DENSE_BENCH_DMR) {
        const double x = ((double)(line + 1) - 0.5) * a.dx;  // the column's centre (init centres)
        const bool post = !(dir == 1 && side == 1) || x < (1.0 / 6.0 + (1.0 + 20.0 * t) / sqrt(3.0));
        if (post) { rho = 8.0; u = (double)8.25f * sqrt(3.0) * 0.5; v = -(double)8.25f * 0.5; pr = 116.5; }
        else      { rho = 1.4; pr = 1.0; }
    } else {
        const bool bottom = side == 0;
        rho = bottom ? 2.0 : 1.0;
        pr = bottom ? 1.0 : 2.5;
    }
    Ug[0] = rho; Ug[1] = rho * u; Ug[2] = rho * v;
    Ug[3] = pr / (a.gamma - 1.0) + 0.5 * rho * (u * u + v * v);
    if (qg) { qg[0] = rho; qg[1] = u; qg[2] = v; qg[3] = pr; qg[4] = sqrt(a.gamma * pr / rho); }
}

template <int DIR, int SPL, int REC>
__device__ __forceinline__ void wall_terms(const AdjParams& a, const double* __restrict__ u,
                                           const double* __restrict__ tape, const double* __restrict__ hb, int i,
                                           int j, const Prim& q, const double U[4], double lam_g, double t,
                                           double Ub[4], double pbar[5], double& lb, double& tl) {
    const int n = DIR == 0 ? a.ni : a.nj, x = DIR == 0 ? i : j;
    const long long ts = DIR == 0 ? a.xs : a.ys;
    const double* T = DIR == 0 ? tape : tape + a.gnp * a.xs;
    const double* H = DIR == 0 ? hb : hb + 4 * a.xs;
    const long long base = DIR == 0 ? (long long)j * (a.ni + 1) : i;
    const long long stride = DIR == 0 ? 1 : a.ni;
    constexpr double we[2][4] = {{4.0 / 3.0, 13.0 / 9.0, 40.0 / 27.0, 121.0 / 81.0},
                                 {-1.0 / 3.0, -4.0 / 9.0, -13.0 / 27.0, -40.0 / 81.0}};
#pragma unroll 1
    for (int side = 0; side < 2; ++side) {
        int rule = a.rule[DIR == 0 ? 2 + side : side];
        if (rule == kRulePeriodic) continue;
        const int line = DIR == 0 ? j : i;
        if (rule == kRuleDMRBottom) rule = ((double)(i + 1) - 0.5) * a.dx >= 1.0 / 6.0 ? kRuleReflect : kRuleFixed;
        const int dist = side == 0 ? x + 1 : n - x;  // 1 = next to the side
        if (rule == kRuleFixed || rule == kRuleSSLInflow) {
            // a fixed ghost state depends on no cell; only GLF's global lambda enters its
            // split, dF+-/dlambda = +-U/2, whose sensitivity the cell next to the side takes for
            // the line's four ghosts. The shear layer's inflow moves with the step's start time:
            // the same cell takes its ghosts' time sensitivity, (dL/dghost)^T w . dghost/dt
            // with only v moving (dU/dt = (0, 0, rho, rho v) v', dprim/dt = (0, 0, v', 0, 0)),
            // and, for the characteristic schemes, the boundary face's Roe share of ghost 0.
            const bool moving = rule == kRuleSSLInflow;
            if (dist != 1 || (SPL != 1 && !moving)) continue;
            double Ug[4], qg[5];
            fixed_state(a, DIR, side, line, t, Ug, qg);
            double dv = 0.0;
            if (moving) {
                double r_, u_, v_, p_;
                ssl_inflow(a, line, t, r_, u_, v_, p_, dv);
            }
#pragma unroll 1
            for (int k = 0; k < 4; ++k) {
                double gp[4] = {0, 0, 0, 0}, gm[4] = {0, 0, 0, 0};
                gather_line<REC>(T, H, ts, base, stride, side == 0 ? -1 - k : n + k, n, false, gp, gm);
                if (SPL == 1) {
                    double s = 0.0;
#pragma unroll
                    for (int c = 0; c < 4; ++c) s = fma(gp[c] - gm[c], Ug[c], s);
                    lb += 0.5 * s;
                }
                if (!moving) continue;
                if (SPL == 2) {
                    const double pv[4] = {qg[0], qg[1], qg[2], qg[4]};
                    double pr4[4] = {0, 0, 0, 0};
                    sw_prim_bar<DIR>(pv, a.gamma, gp, gm, pr4);
                    tl = fma(pr4[2], dv, tl);
                } else {
                    // U of the ghost and its primitives (rho, u, v, p, alpha)
                    const double g[9] = {Ug[0], Ug[1], Ug[2], Ug[3], qg[0], qg[1], qg[2], qg[3], qg[4]};
                    double Ubg[4] = {0, 0, 0, 0}, unb, pb, ab;
                    llf_bar<DIR, SPL == 1>(g, g[5 + DIR], g[7], g[8], gp, gm, lam_g, Ubg, unb, pb, ab);
                    // the normal velocity (u on the left side) does not move; v does
                    tl = fma(Ubg[2] * qg[0] + Ubg[3] * (qg[0] * qg[2]), dv, tl);
                    if (DIR == 1) tl = fma(unb, dv, tl);
                }
                if (a.charac && k == 0) {
                    const double* RB = a.rbar + (DIR == 0 ? 0 : 8 * a.xs) + base + (long long)(side == 0 ? 0 : n) * stride;
                    tl = fma(RB[(side == 0 ? 2 : 6) * ts], dv, tl);
                }
            }
            continue;
        }
        if (dist > (rule == kRuleReflect ? 4 : 2)) continue;
        // extrapolation: conserved variables and primitives (rho, u, v, p, alpha) of the two
        // cells next to the side
        double c1[9], c2[9];
        if (rule == kRuleExtrap) {
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const int xx = side == 0 ? d : n - 1 - d;
                const long long o = DIR == 0 ? (long long)j * a.ni + xx : (long long)xx * a.ni + i;
                double* c = d == 0 ? c1 : c2;
#pragma unroll
                for (int v = 0; v < 4; ++v) c[v] = u[v * a.plane + o];
                const Prim qq = prim_of(c, a.gamma);
                c[4] = c[0]; c[5] = qq.u; c[6] = qq.v; c[7] = qq.p; c[8] = qq.a;
            }
        }
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            double w;
            if (rule == kRuleReflect) {
                if (dist != k + 1) continue;
                w = 1.0;
            } else {
                w = we[dist - 1][k];
            }
            double g[9];  // the ghost's U (0..3) and primitives (4..8)
            if (rule == kRuleReflect) {
#pragma unroll
                for (int v = 0; v < 4; ++v) g[v] = U[v];
                g[4] = U[0]; g[5] = q.u; g[6] = q.v; g[7] = q.p; g[8] = q.a;
                g[1 + DIR] = -g[1 + DIR];
                g[5 + DIR] = -g[5 + DIR];
            } else {
#pragma unroll
                for (int v = 0; v < 9; ++v) {
                    double na = c1[v], fa = c2[v], gv = 0.0;
                    for (int l = 0; l <= k; ++l) {
                        gv = fma(na, 4.0 / 3.0, -(fa * (1.0 / 3.0)));
                        fa = na;
                        na = gv;
                    }
                    g[v] = gv;
                }
            }
            double gp[4] = {0, 0, 0, 0}, gm[4] = {0, 0, 0, 0};
            gather_line<REC>(T, H, ts, base, stride, side == 0 ? -1 - k : n + k, n, false, gp, gm);
            double Ubg[4] = {0, 0, 0, 0}, prb[5] = {0, 0, 0, 0, 0};
            if (SPL == 2) {
                const double pv[4] = {g[4], g[5], g[6], g[8]};
                double pr4[4] = {0, 0, 0, 0};
                sw_prim_bar<DIR>(pv, a.gamma, gp, gm, pr4);
                prb[0] = pr4[0]; prb[1] = pr4[1]; prb[2] = pr4[2]; prb[4] = pr4[3];
            } else {
                double unb, pb, ab;
                const double lamb = llf_bar<DIR, SPL == 1>(g, g[5 + DIR], g[7], g[8], gp, gm, lam_g, Ubg, unb, pb, ab);
                prb[1 + DIR] = unb;
                prb[3] = pb;
                prb[4] = ab;
                if (SPL == 1 && (rule == kRuleReflect || dist == 1)) lb += lamb;
            }
            if (a.adapt)  // the ghost's density in the surrogate stencils that read it
                prb[0] += gather_rho_line(T, ts, base, stride, side == 0 ? -1 - k : n + k, n, false);
            if (a.charac && k == 0) {
                // the ghost next to the side is a Roe cell of the boundary face: the left cell of
                // face 0, the right cell of face n
                const double* RB = a.rbar + (DIR == 0 ? 0 : 8 * a.xs) + base + (long long)(side == 0 ? 0 : n) * stride;
#pragma unroll
                for (int v = 0; v < 4; ++v) prb[v] += RB[(side == 0 ? v : 4 + v) * ts];
            }
            const double sn = rule == kRuleReflect ? -1.0 : 1.0;
#pragma unroll
            for (int v = 0; v < 4; ++v) Ub[v] += (v == 1 + DIR ? sn * w : w) * Ubg[v];
#pragma unroll
            for (int v = 0; v < 5; ++v) pbar[v] += (v == 1 + DIR ? sn * w : w) * prb[v];
        }
    }
}

// ---- characteristic WENO-Z (104): the face-level reverse ------------------------------------
// Conserved variables (c[0..3]) and primitives (rho, u, v, p, alpha: c[4..8]) of cell x (interior
// index along DIR, a ghost when outside 0..n-1) of line `line`, by the side rules as the forward's
// boundary fill builds them: a periodic image, the mirror of cell k for ghost k (normal velocity
// and momentum negated), the recursive extrapolation of the two cells next to the side (cons and
// primitives each), or a fixed state.
__device__ __forceinline__ void cell_state(const AdjParams& a, const double* __restrict__ u, long long o,
                                           double c[9]) {
#pragma unroll
    for (int v = 0; v < 4; ++v) c[v] = u[v * a.plane + o];
    const Prim q = prim_of(c, a.gamma);
    c[4] = c[0]; c[5] = q.u; c[6] = q.v; c[7] = q.p; c[8] = q.a;
}
template <int DIR>
__device__ __forceinline__ void fetch_cell(const AdjParams& a, const double* __restrict__ u, int line, int x,
                                           double t, double c[9]) {
    const int n = DIR == 0 ? a.ni : a.nj;
    auto off = [&](int xx) { return DIR == 0 ? (long long)line * a.ni + xx : (long long)xx * a.ni + line; };
    if (x >= 0 && x < n) { cell_state(a, u, off(x), c); return; }
    const int side = x < 0 ? 0 : 1, k = x < 0 ? -1 - x : x - n;  // ghost layer k (0: next to the side)
    int rule = a.rule[DIR == 0 ? 2 + side : side];
    if (rule == kRuleDMRBottom) rule = ((double)(line + 1) - 0.5) * a.dx >= 1.0 / 6.0 ? kRuleReflect : kRuleFixed;
    if (rule == kRulePeriodic) {
        cell_state(a, u, off(side == 0 ? x + n : x - n), c);
    } else if (rule == kRuleReflect) {
        cell_state(a, u, off(side == 0 ? k : n - 1 - k), c);
        c[1 + DIR] = -c[1 + DIR];
        c[5 + DIR] = -c[5 + DIR];
    } else if (rule == kRuleExtrap) {
        double c1[9], c2[9];
        cell_state(a, u, off(side == 0 ? 0 : n - 1), c1);
        cell_state(a, u, off(side == 0 ? 1 : n - 2), c2);
#pragma unroll
        for (int v = 0; v < 9; ++v) {
            double na = c1[v], fa = c2[v], gv = 0.0;
            for (int l = 0; l <= k; ++l) {
                gv = fma(na, 4.0 / 3.0, -(fa * (1.0 / 3.0)));
                fa = na;
                na = gv;
            }
            c[v] = gv;
        }
    } else {  // a fixed state at the step's start time t
        fixed_state(a, DIR, side, line, t, c, c + 4);
    }
}

// Per face of direction DIR, two threads (adjacent lanes, one per sign): the characteristic
// reconstruction recomputed from the stage input u -- the GLF split fluxes of the stencil cells
// (the stage's global lambda), the Roe average of the face's two cells and its eigenvectors
// (roe_eig_fast's formulas), the sign's five split fluxes projected on the characteristic
// fields and WENO-Z per field with its stencil gradient (weno_grad) -- and its reverse for the
// face's hbar: the back-projection's transpose gives each field's value sensitivity, times the
// field's stencil gradient the sensitivities of the projected values, the transposed
// projection those of the split fluxes, written per (sign, stencil point, component) as the
// cell kernel's gather reads them (kRecFaceSens); and the eigenvectors'
// sensitivities -- from the projections (sum over the stencil of the projected-value
// sensitivities times the split fluxes) and the back-projection, the two signs' shares summed
// across the lane pair -- sent through the eigenvectors' formulas and the Roe average to the
// primitives (rho, u, v, p) of the face's two cells (rbar: the "+" lane writes the left cell's,
// the "-" lane the right cell's).
// A block of 32 x 4 threads takes 16 faces x 4 lines (xi) or 16 lines x 4 faces (eta); its
// cells' split fluxes and primitives are staged once in shared memory (each cell's get_primary
// and split computed once, not once per reading face), and each thread parks its projected-value
// sensitivities there too, which keeps the field loop's live registers down.
template <int DIR>
__global__ void __launch_bounds__(128, 3) k_char_face(AdjParams a, const double* __restrict__ u,
                                                  const double* __restrict__ hb, const double* __restrict__ lamv,
                                                  const double* __restrict__ tp, const double* __restrict__ flags,
                                                  double* __restrict__ fbar) {
    constexpr int FA = DIR == 0 ? 16 : 4;  // faces of a block along the direction
    constexpr int NB = DIR == 0 ? 4 : 16;  // lines of a block
    constexpr int NA = FA + 5;             // cells staged along a line: f0-3 .. f0+FA+1
    __shared__ double sC[12][NB][NA];      // F+ (0..3), F- (4..7), rho, u, v, p (8..11)
    __shared__ double sL[20][128];         // per thread: cb[k] g_k[m] of its sign, row k*5+m
    const int ni = a.ni, nj = a.nj;
    const int n = DIR == 0 ? ni : nj, nline = DIR == 0 ? nj : ni;
    const int tid = threadIdx.x + 32 * threadIdx.y;
    const int f0 = (DIR == 0 ? blockIdx.x : blockIdx.y) * FA, l0 = (DIR == 0 ? blockIdx.y : blockIdx.x) * NB;
    const double lam = lamv[DIR];
    {
        const double t = tp ? *tp : 0.0;
        for (int idx = tid; idx < NA * NB; idx += 128) {
            const int ai = idx % NA, bi = idx / NA;
            const int x = f0 - 3 + ai, line = l0 + bi;  // x >= -3; faces <= n read cells <= n+2
            if (line >= nline || x > n + 2) continue;
            double c[9];
            fetch_cell<DIR>(a, u, line, x, t, c);
            const double un = c[5 + DIR], pr = c[7];
            const double P[4] = {0.0, DIR == 0 ? pr : 0.0, DIR == 1 ? pr : 0.0, un * pr};
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                sC[v][bi][ai] = 0.5 * fma(un + lam, c[v], P[v]);
                sC[4 + v][bi][ai] = 0.5 * fma(un - lam, c[v], P[v]);
                sC[8 + v][bi][ai] = c[4 + v];
            }
        }
    }
    __syncthreads();
    const int sg = threadIdx.x & 1, fl = threadIdx.x >> 1;
    const int fa = DIR == 0 ? fl : (int)threadIdx.y, bi = DIR == 0 ? (int)threadIdx.y : fl;
    const int f = f0 + fa, line = l0 + bi;
    const bool valid = f <= n && line < nline;  // the same for both lanes of a face
    const long long ts = DIR == 0 ? a.xs : a.ys;
    const long long to = DIR == 0 ? (long long)line * (ni + 1) + f : (long long)f * ni + line;
    const double g1 = a.gamma - 1.0, kg = a.gamma / g1;
    // AdaWENO (flags): the branches the forward took at this face, bit 0 "+" smooth, bit 1 "-"
    int fbits = 0;
    if (flags && valid) fbits = (int)flags[(DIR == 0 ? 0 : 5 * a.xs) + to];
    const bool smooth = (fbits >> sg) & 1, any_char = fbits != 3;
    // this sign's split flux of stencil point m, component cc (F+ of cells f-3..f+1, F- of
    // cells f+2..f-2), and the cell's density
    auto am = [&](int m) { return fa + (sg ? 5 - m : m); };
    auto F = [&](int m, int cc) { return sC[sg * 4 + cc][bi][am(m)]; };
    // the eigen quantities' sensitivities (this lane's sign; summed across the pair below)
    double un0b = 0, ut0b = 0, a0b = 0, h0b = 0, uu0b = 0, a0un0b = 0;
    double A0[4] = {0, 0, 0, 0}, A1[4] = {0, 0, 0, 0}, A3[4] = {0, 0, 0, 0}, A20 = 0;  // A[k][cc]
    // the Roe average's inputs of this lane's cell (the "+" lane the left cell, the "-" lane the
    // right), exchanged across the pair: sqrt(rho) and the total enthalpy
    const int ac = fa + 2 + sg;
    const double rs = valid ? sC[8][bi][ac] : 1.0, us = valid ? sC[9][bi][ac] : 0.0;
    const double vs = valid ? sC[10][bi][ac] : 0.0, ps = valid ? sC[11][bi][ac] : 1.0;
    const double irs = 1.0 / rs, ss = sqrt(rs), hs = fma(kg * ps, irs, 0.5 * (us * us + vs * vs));
    const double ss_o = __shfl_xor_sync(0xffffffffu, ss, 1), hs_o = __shfl_xor_sync(0xffffffffu, hs, 1);
    const double us_o = __shfl_xor_sync(0xffffffffu, us, 1), vs_o = __shfl_xor_sync(0xffffffffu, vs, 1);
    const double sl = sg ? ss_o : ss, sr = sg ? ss : ss_o, hl = sg ? hs_o : hs, hr = sg ? hs : hs_o;
    const double ul = sg ? us_o : us, ur = sg ? us : us_o, vl = sg ? vs_o : vs, vr = sg ? vs : vs_o;
    double r = 0.5, u0 = 0, v0 = 0, h0 = 0, uu0 = 0, c2 = 1, ia = 1, a0 = 1;
    double ihh = 0, un0 = 0, ut0 = 0;
    if (valid) {
        double* const FB = fbar + (DIR == 0 ? 0 : a.gnp * a.xs) + to;
        double HB[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) HB[v] = hb[(DIR == 0 ? 0 : 4 * a.xs) + v * ts + to];
        if (any_char) {  // a face whose signs are both smooth never forms its Roe average
            r = 1.0 / (sl + sr);
            u0 = (sr * ur + sl * ul) * r; v0 = (sr * vr + sl * vl) * r; h0 = (sr * hr + sl * hl) * r;
            uu0 = 0.5 * (u0 * u0 + v0 * v0);
            c2 = g1 * (h0 - uu0);
            ia = 1.0 / sqrt(c2); a0 = c2 * ia; ihh = g1 * ia * ia;
            un0 = DIR == 0 ? u0 : v0; ut0 = DIR == 0 ? v0 : u0;
        }
        if (!smooth) {
            const double a0un0 = a0 * un0;
            const double hu = 0.5 * uu0 * ihh, nu = 0.5 * un0 * ia, ia5 = 0.5 * ia;
            const double pn = 0.5 * un0 * ihh, pt = 0.5 * ut0 * ihh, ih = 0.5 * ihh;
            const double ln0 = -pn - ia5, ln3 = -pn + ia5;
            // M[cc][k]: the coefficient of split-flux component cc in characteristic field k
            double M[4][4];
            M[0][0] = hu + nu; M[3][0] = ih;
            M[0][3] = hu - nu; M[3][3] = ih;
            if (DIR == 0) { M[1][0] = ln0; M[2][0] = -pt; M[1][3] = ln3; M[2][3] = -pt; }
            else          { M[1][0] = -pt; M[2][0] = ln0; M[1][3] = -pt; M[2][3] = ln3; }
            M[0][1] = 1.0 - uu0 * ihh; M[1][1] = u0 * ihh; M[2][1] = v0 * ihh; M[3][1] = -ihh;
            M[0][2] = -ut0; M[1][2] = DIR == 1 ? 1.0 : 0.0; M[2][2] = DIR == 0 ? 1.0 : 0.0; M[3][2] = 0.0;
            const double hn = HB[1 + DIR], ht = HB[2 - DIR];
            // the back-projection's transpose: each field value's sensitivity
            const double sb = HB[0] + un0 * hn + ut0 * ht, db = a0 * hn + a0un0 * HB[3];
            const double cb[4] = {sb - db + h0 * HB[3], sb + uu0 * HB[3], ht + ut0 * HB[3], sb + db + h0 * HB[3]};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                double lf[5];
#pragma unroll
                for (int m = 0; m < 5; ++m)
                    lf[m] = fma(M[0][k], F(m, 0), fma(M[1][k], F(m, 1), fma(M[2][k], F(m, 2), M[3][k] * F(m, 3))));
                double gd[4], d0, d1, d2;
                first_differences(lf, gd);
                betas_g(gd, d0, d1, d2);
                const double B[3] = {fma(-3.0, gd[1], gd[0]), gd[1] + gd[2], fma(3.0, gd[2], -gd[3])};
                WenoTerms wt;
                weno_terms<true>(gd, d0, d1, d2, wt);
                const double iN = rcp_nr(wt.N), num = weno_num(wt);
                const double cv = fma(num, iN, lf[2]);
                double G[5];
                weno_grad<true>(gd, B, d0, d1, d2, wt, num * iN, iN, G);
#pragma unroll
                for (int m = 0; m < 5; ++m) sL[k * 5 + m][tid] = cb[k] * G[m];
                // the back-projection's own sensitivities, linear in the field values: with
                // s = cv0 + cv1 + cv3 and d = cv3 - cv0, un0 takes s hn, a0 d hn, ut0 s ht + cv2 h3,
                // h0 (cv0 + cv3) h3, a0 un0 d h3, uu0 cv1 h3
                if (k != 2) { un0b = fma(cv, hn, un0b); ut0b = fma(cv, ht, ut0b); }
                if (k == 0) { a0b = fma(-cv, hn, a0b); h0b = fma(cv, HB[3], h0b); a0un0b = fma(-cv, HB[3], a0un0b); }
                if (k == 3) { a0b = fma(cv, hn, a0b); h0b = fma(cv, HB[3], h0b); a0un0b = fma(cv, HB[3], a0un0b); }
                if (k == 1) uu0b = fma(cv, HB[3], uu0b);
                if (k == 2) ut0b = fma(cv, HB[3], ut0b);
            }
            // the split fluxes' sensitivities (the transposed projection) and the projection
            // coefficients' (sum over the stencil of the projected values' times the split fluxes)
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                const double l0_ = sL[m][tid], l1_ = sL[5 + m][tid], l2_ = sL[10 + m][tid], l3_ = sL[15 + m][tid];
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) {
                    const double Fm = F(m, cc);
                    FB[(long long)((sg * 5 + m) * 4 + cc) * ts] =
                        fma(M[cc][0], l0_, fma(M[cc][1], l1_, fma(M[cc][2], l2_, M[cc][3] * l3_)));
                    A0[cc] = fma(l0_, Fm, A0[cc]);
                    A1[cc] = fma(l1_, Fm, A1[cc]);
                    A3[cc] = fma(l3_, Fm, A3[cc]);
                    if (cc == 0) A20 = fma(l2_, Fm, A20);
                }
                if (flags) FB[(long long)(40 + sg * 5 + m) * ts] = 0.0;  // no density share
            }
        } else {
            // AdaWENO's smooth branch (scheme_weno5th_SC.f90:110-124): every component
            // reconstructed from its own candidates with the WENO-Z weights w_k of the scalar
            // surrogate sur = rho + F(normal momentum). Its reverse: dh_v/dF_v[m] = sum_k w_k
            // a_k,m, the same for the four components; the weights' sensitivities Q_k =
            // sum_v hbar_v q_k(F_v) = q_k(phi), phi[m] = sum_v hbar_v F_v[m], sent through the
            // surrogate's weights to its five values, and from each to the cell's density and
            // normal-momentum split flux.
            double phi[5], sur[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                phi[m] = fma(HB[0], F(m, 0), fma(HB[1], F(m, 1), fma(HB[2], F(m, 2), HB[3] * F(m, 3))));
                sur[m] = sC[8][bi][am(m)] + F(m, 1 + DIR);
            }
            double gd[4], d0, d1, d2;
            first_differences(sur, gd);
            betas_g(gd, d0, d1, d2);
            const double B[3] = {fma(-3.0, gd[1], gd[0]), gd[1] + gd[2], fma(3.0, gd[2], -gd[3])};
            WenoTerms wt;
            weno_terms<true>(gd, d0, d1, d2, wt);
            const double iN = rcp_nr(wt.N);
            const double w0 = c30 * wt.v[0] * iN, w1 = c31 * wt.v[1] * iN, w2 = c32 * wt.v[2] * iN;
            const double Q0 = fma(a300, phi[0], fma(a301, phi[1], a302 * phi[2]));
            const double Q1 = fma(a310, phi[1], fma(a311, phi[2], a312 * phi[3]));
            const double Q2 = fma(a320, phi[2], fma(a321, phi[3], a322 * phi[4]));
            const double Wq = fma(w0, Q0, fma(w1, Q1, w2 * Q2));
            const double E[3] = {c30 * (Q0 - Wq), c31 * (Q1 - Wq), c32 * (Q2 - Wq)};
            double gw[5];
            weno_weight_grad<true>(gd, B, d0, d1, d2, wt, E, iN, gw);
            const double gc[5] = {w0 * a300, fma(w0, a301, w1 * a310), fma(w0, a302, fma(w1, a311, w2 * a320)),
                                  fma(w1, a312, w2 * a321), w2 * a322};
#pragma unroll
            for (int m = 0; m < 5; ++m) {
#pragma unroll
                for (int cc = 0; cc < 4; ++cc)
                    FB[(long long)((sg * 5 + m) * 4 + cc) * ts] = cc == 1 + DIR ? fma(HB[cc], gc[m], gw[m]) : HB[cc] * gc[m];
                FB[(long long)(40 + sg * 5 + m) * ts] = gw[m];
            }
        }
    }
    // the two signs' shares (both lanes of a pair are valid or neither; every lane shuffles)
    auto pair_sum = [](double& v) { v += __shfl_xor_sync(0xffffffffu, v, 1); };
    pair_sum(un0b); pair_sum(ut0b); pair_sum(a0b); pair_sum(h0b); pair_sum(uu0b); pair_sum(a0un0b);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) { pair_sum(A0[cc]); pair_sum(A1[cc]); pair_sum(A3[cc]); }
    pair_sum(A20);
    if (!valid) return;
    double* const RB = a.rbar + (DIR == 0 ? 0 : 8 * a.xs) + to + (long long)(4 * sg) * ts;
    if (!any_char) {  // no Roe average at this face
#pragma unroll
        for (int v = 0; v < 4; ++v) RB[v * ts] = 0.0;
        return;
    }
    // the eigenvector entries' sensitivities back to the Roe quantities
    const double l00b = A0[0], l03b = A3[0];
    const double l10b = A0[1], l13b = A3[1], l20b = A0[2], l23b = A3[2];
    const double l30b = A0[3] + A3[3];
    const double l01b = A1[0], l11b = A1[1], l21b = A1[2], l31b = A1[3];
    ut0b -= A20;
    const double hub = l00b + l03b, nub = l00b - l03b;
    const double nrm0 = DIR == 0 ? l10b : l20b, nrm3 = DIR == 0 ? l13b : l23b;  // the ln0, ln3 entries
    const double tg0 = DIR == 0 ? l20b : l10b, tg3 = DIR == 0 ? l23b : l13b;    // the -pt entries
    const double pnb = -nrm0 - nrm3, ia5b = -nrm0 + nrm3, ptb = -tg0 - tg3, ihb = l30b;
    double ihhb = 0.0, iab = 0.0, u0b = 0.0, v0b = 0.0;
    uu0b += -ihh * l01b + 0.5 * ihh * hub;
    ihhb += -uu0 * l01b + u0 * l11b + v0 * l21b - l31b + 0.5 * uu0 * hub + 0.5 * un0 * pnb + 0.5 * ut0 * ptb +
            0.5 * ihb;
    u0b += ihh * l11b;
    v0b += ihh * l21b;
    un0b += 0.5 * ia * nub + 0.5 * ihh * pnb + a0 * a0un0b;
    ut0b += 0.5 * ihh * ptb;
    iab += 0.5 * un0 * nub + 0.5 * ia5b;
    a0b += un0 * a0un0b;
    if (DIR == 0) { u0b += un0b; v0b += ut0b; }
    else          { v0b += un0b; u0b += ut0b; }
    iab += 2.0 * g1 * ia * ihhb;  // ihh = g1 ia^2
    double c2b = ia * a0b;        // a0 = c2 ia
    iab += c2 * a0b;
    c2b += -0.5 * ia * ia * ia * iab;  // ia = c2^-1/2
    h0b += g1 * c2b;
    uu0b += -g1 * c2b;
    u0b += u0 * uu0b;
    v0b += v0 * uu0b;
    // the Roe average's inputs, then this lane's cell's primitives (the "+" lane the left cell's,
    // rbar planes 0..3; the "-" lane the right cell's, 4..7): d sqrt(rho), d h, d u, d v of the
    // average, then rho and p through sqrt(rho) and h = kg p / rho + (u^2 + v^2)/2
    const double sbar = r * ((us - u0) * u0b + (vs - v0) * v0b + (hs - h0) * h0b);
    const double sr_ = ss * r, kgir = kg * irs;
    const double hbar = sr_ * h0b;
    RB[0 * ts] = fma(0.5 * ss * irs, sbar, -(kgir * ps * irs * hbar));  // d sqrt(rho)/d rho = 1/(2 sqrt(rho))
    RB[1 * ts] = fma(us, hbar, sr_ * u0b);
    RB[2 * ts] = fma(vs, hbar, sr_ * v0b);
    RB[3 * ts] = kgir * hbar;
}

// Cell kernel: Ub = (dL/du)^T w at the cell from the stage's tape and hbar, then the reverse of
// RK stage STAGE (3, 2, 1; 0 = Ub alone; a kernel argument, uniform over the grid). Stage 1
// also reduces the wave-speed maxima of its state u0 (the time step's input) per block, with
// their cells. WALLS: the grid has wall sides (wall_terms). SPL: 0 LLF, 1 GLF, 2 SW. GLF:
// lamv holds the stage's global lambda of both directions; the sensitivities of lambda are summed
// per block into lpart.
template <int REC, int SPL, bool WALLS>
__global__ void __launch_bounds__(128) k_rev(AdjParams a, const double* __restrict__ u,
                                             const double* __restrict__ w, const double* __restrict__ tape,
                                             const double* __restrict__ hb, double* __restrict__ acc,
                                             double* __restrict__ out, const double* __restrict__ dtp,
                                             const double* __restrict__ tp, double* __restrict__ mpart,
                                             const double* __restrict__ lamv, double* __restrict__ lpart,
                                             int STAGE) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int ni = a.ni, nj = a.nj;
    double e1 = -1.0, e2 = -1.0;
    long long i1 = LLONG_MAX, i2 = LLONG_MAX;
    double lbx = 0.0, lby = 0.0;
    double bsum = 0.0, Ub_bf0 = 0.0, Ub_bf2 = 0.0;  // the body force's terms (a.bodyforce)
    double tsl = 0.0;                                 // the inflow ghosts' time sensitivity (a.ssl)
    if (i < ni && j < nj) {
        const long long o = (long long)j * ni + i;
        double U[4], Ub[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = u[v * a.plane + o];
        constexpr bool GLF = SPL == 1;
        const Prim q = prim_of(U, a.gamma);
        double gpx[4] = {0, 0, 0, 0}, gmx[4] = {0, 0, 0, 0}, gpy[4] = {0, 0, 0, 0}, gmy[4] = {0, 0, 0, 0};
        const bool px = a.rule[2] == kRulePeriodic, py = a.rule[0] == kRulePeriodic;
        gather_line<REC>(tape, hb, a.xs, (long long)j * (ni + 1), 1, i, ni, px, gpx, gmx);
        // LF splittings pull each direction back before gathering the next (fewer live
        // registers); Steger-Warming seeds each variable once for both directions
        if (SPL != 2) lbx = llf_vjp<0, GLF>(U, q, a.gamma, gpx, gmx, GLF ? lamv[0] : 0.0, Ub);
        gather_line<REC>(tape + a.gnp * a.xs, hb + 4 * a.xs, a.ys, i, ni, j, nj, py, gpy, gmy);
        if (SPL != 2) lby = llf_vjp<1, GLF>(U, q, a.gamma, gpy, gmy, GLF ? lamv[1] : 0.0, Ub);
        else          sw_vjp(U, a.gamma, gpx, gmx, gpy, gmy, Ub);
        if (a.charac) {
            // the Roe averages of the faces this cell is a side of: the left cell of face x+1 and
            // the right cell of face x in each direction (and, on periodic lines, the right cell
            // of face n from cell 0 and the left cell of face 0 from cell n-1, their images)
            double rb[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
            for (int D = 0; D < 2; ++D) {
                const int n = D == 0 ? ni : nj, x = D == 0 ? i : j;
                const long long ts = D == 0 ? a.xs : a.ys;
                const double* RB = a.rbar + (D == 0 ? 0 : 8 * a.xs);
                auto face = [&](int f) { return D == 0 ? (long long)j * (ni + 1) + f : (long long)f * ni + i; };
                auto add = [&](int f, int q0) {
#pragma unroll
                    for (int v = 0; v < 4; ++v) rb[v] += RB[(q0 + v) * ts + face(f)];
                };
                add(x + 1, 0);
                add(x, 4);
                if (D == 0 ? px : py) {
                    if (x == n - 1) add(0, 0);
                    if (x == 0) add(n, 4);
                }
            }
            prim_pullback_all(U, q, a.gamma, rb[0], rb[1], rb[2], rb[3], 0.0, Ub);
        }
        if (a.adapt)  // the surrogate stencils' density sensitivities (rho = U[0])
            Ub[0] += gather_rho_line(tape, a.xs, (long long)j * (ni + 1), 1, i, ni, px) +
                     gather_rho_line(tape + a.gnp * a.xs, a.ys, i, ni, j, nj, py);
        if (WALLS && (!px || !py)) {  // the ghost cells of wall sides that this cell feeds
            // (a separate instantiation: the periodic kernels keep their registers)
            double pbar[5] = {0, 0, 0, 0, 0};
            const double t = tp ? *tp : 0.0;  // the step's start time (the moving shock's ghosts)
            if (!px) wall_terms<0, SPL, REC>(a, u, tape, hb, i, j, q, U, GLF ? lamv[0] : 0.0, t, Ub, pbar, lbx, tsl);
            if (!py) wall_terms<1, SPL, REC>(a, u, tape, hb, i, j, q, U, GLF ? lamv[1] : 0.0, t, Ub, pbar, lby, tsl);
            prim_pullback_all(U, q, a.gamma, pbar[0], pbar[1], pbar[2], pbar[3], pbar[4], Ub);
        }
        const double dt = STAGE == 0 ? 0.0 : *dtp;
        if (STAGE != 0 && a.bodyforce) {
            // the stage's body force f_s (0, 0, rho, rho v) of its input u: (df/du)^T w sends
            // f_s w[2] to rho and f_s w[3] to rho v; its dt-part w . S for the time step
            const double w2 = w[2 * a.plane + o], w3 = w[3 * a.plane + o];
            const double f = (STAGE == 1 ? 1.0 : STAGE == 2 ? 0.25 : kTwoThirdsSingle) * dt;
            bsum = fma(w2, U[0], w3 * U[2]);
            Ub_bf0 = f * w2;
            Ub_bf2 = f * w3;
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const long long ov = v * a.plane + o;
            if (STAGE == 0) {
                out[ov] = Ub[v];
            } else {
                const double wv = w[ov];
                const double bf = v == 0 ? Ub_bf0 : v == 2 ? Ub_bf2 : 0.0;
                if (STAGE == 3) {
                    acc[ov] = 1.0 / 3.0 * wv;
                    out[ov] = 2.0 / 3.0 * wv + 2.0 / 3.0 * dt * Ub[v] + bf;
                } else if (STAGE == 2) {
                    acc[ov] += 3.0 / 4.0 * wv;
                    out[ov] = 1.0 / 4.0 * wv + 1.0 / 4.0 * dt * Ub[v] + bf;
                } else {
                    out[ov] = acc[ov] + wv + dt * Ub[v] + bf;
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
        block_argmax(e1, i1, e2, i2);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double* mp = mpart + 4 * (blockIdx.y * gridDim.x + blockIdx.x);
            mp[0] = e1; mp[1] = (double)i1; mp[2] = e2; mp[3] = (double)i2;
        }
    }
    if (SPL == 1) {
        __syncthreads();  // the argmax reduction's shared arrays are read before the next sum
        block_sum2(lbx, lby);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double* lp = lpart + 2 * (blockIdx.y * gridDim.x + blockIdx.x);
            lp[0] = lbx;
            lp[1] = lby;
        }
    }
    if (STAGE != 0 && (a.bodyforce || a.ssl)) {  // uniform over the grid
        __syncthreads();  // the shared arrays of the reductions above are free again
        block_sum2(bsum, tsl);
        const int blk = (STAGE - 1) * (gridDim.x * gridDim.y) + blockIdx.y * gridDim.x + blockIdx.x;
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (a.bodyforce) a.bpart[blk] = bsum;
            if (a.ssl) a.tpart[blk] = tsl;
        }
    }
}

// GLF: per block, the maxima of |u|+alpha and |v|+alpha over the stage input's cells and their
// cells (the stage's global lambda, max_eig_i/j of get_primary.f90:69-73).
__global__ void __launch_bounds__(128) k_maxarg(AdjParams a, const double* __restrict__ u,
                                                double* __restrict__ mpart) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    double e1 = -1.0, e2 = -1.0;
    long long i1 = LLONG_MAX, i2 = LLONG_MAX;
    if (i < a.ni && j < a.nj) {
        const long long o = (long long)j * a.ni + i;
        double U[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = u[v * a.plane + o];
        const Prim q = prim_of(U, a.gamma);
        e1 = fabs(q.u) + q.a;
        e2 = fabs(q.v) + q.a;
        i1 = i2 = o;
    }
    block_argmax(e1, i1, e2, i2);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double* mp = mpart + 4 * (blockIdx.y * gridDim.x + blockIdx.x);
        mp[0] = e1; mp[1] = (double)i1; mp[2] = e2; mp[3] = (double)i2;
    }
}

// GLF: the block maxima reduced to lamv = (lambda_x, lambda_y, cell of lambda_x, cell of
// lambda_y), ties to the lowest cell. One block of 256 threads.
__global__ void __launch_bounds__(256) k_maxred(const double* __restrict__ mpart, int nm, double* __restrict__ lamv) {
    const int t = threadIdx.x;
    double e1 = -1.0, e2 = -1.0;
    long long i1 = LLONG_MAX, i2 = LLONG_MAX;
    for (int k = t; k < nm; k += blockDim.x) {
        const double* mp = mpart + 4 * k;
        if (argmax_better(mp[0], (long long)mp[1], e1, i1)) { e1 = mp[0]; i1 = (long long)mp[1]; }
        if (argmax_better(mp[2], (long long)mp[3], e2, i2)) { e2 = mp[2]; i2 = (long long)mp[3]; }
    }
    block_argmax(e1, i1, e2, i2);
    if (t == 0) { lamv[0] = e1; lamv[1] = e2; lamv[2] = (double)i1; lamv[3] = (double)i2; }
}

// GLF: the stage's total sensitivity of lambda_x and lambda_y (the block sums of k_rev, in a
// fixed order) sent through |u_n| + alpha at the cells of the maxima into the stage's output,
// with the stage's coefficient of L(u) (1 for STAGE 0, dt, dt/4, 2 dt/3 for stages 1, 2, 3).
template <int STAGE>
__global__ void __launch_bounds__(256) k_lamg(AdjParams a, const double* __restrict__ lpart, int nb,
                                              const double* __restrict__ lamv, const double* __restrict__ u,
                                              const double* __restrict__ dtp, double* __restrict__ out) {
    const int t = threadIdx.x;
    double sx = 0.0, sy = 0.0;
    for (int k = t; k < nb; k += blockDim.x) { sx += lpart[2 * k]; sy += lpart[2 * k + 1]; }
    block_sum2(sx, sy);
    if (t != 0) return;
    const double dt = STAGE == 0 ? 1.0 : *dtp;
    const double c = STAGE == 0 ? 1.0 : STAGE == 1 ? dt : STAGE == 2 ? 0.25 * dt : 2.0 / 3.0 * dt;
    const double cell[2] = {lamv[2], lamv[3]};
    const double sens[2] = {sx, sy};
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        // no cell holds a finite maximum (a NaN state): nothing to differentiate
        if (!(cell[d] >= 0.0 && cell[d] < (double)a.plane)) continue;
        const long long o = (long long)cell[d];
        double U[4], Ub[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = u[v * a.plane + o];
        if (d == 0) wave_speed_vjp<0>(U, a.gamma, c * sens[d], Ub);
        else        wave_speed_vjp<1>(U, a.gamma, c * sens[d], Ub);
#pragma unroll
        for (int v = 0; v < 4; ++v) out[v * a.plane + o] += Ub[v];
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
    if (a.bodyforce)  // the stages' body-force terms w . S, with their own stage-3 factor
        for (int k = t; k < 3 * nm; k += blockDim.x) {
            const int st = k / nm;
            s += (st == 0 ? 1.0 : st == 1 ? 0.25 : kTwoThirdsSingle) * a.bpart[k];
        }
    double ts_ = 0.0;  // the shear layer: the stages' time sensitivities, with L's stage factors
    if (a.ssl)
        for (int k = t; k < 3 * nm; k += blockDim.x) {
            const int st = k / nm;
            ts_ += (st == 0 ? 1.0 : st == 1 ? 0.25 : 2.0 / 3.0) * a.tpart[k];
        }
    double e1 = -1.0, e2 = -1.0, i1 = 1e300, i2 = 1e300;
    for (int k = t; k < nm; k += blockDim.x) {
        const double* mp = mpart + 4 * k;
        if (mp[0] > e1 || (mp[0] == e1 && mp[1] < i1)) { e1 = mp[0]; i1 = mp[1]; }
        if (mp[2] > e2 || (mp[2] == e2 && mp[3] < i2)) { e2 = mp[2]; i2 = mp[3]; }
    }
    __shared__ double rs[256], re1[256], re2[256], ri1[256], ri2[256], rt[256];
    rs[t] = s; re1[t] = e1; re2[t] = e2; ri1[t] = i1; ri2[t] = i2; rt[t] = ts_;
    __syncthreads();
    for (int h = blockDim.x / 2; h; h >>= 1) {
        if (t < h) {
            rs[t] += rs[t + h];
            rt[t] += rt[t + h];
            if (re1[t + h] > re1[t] || (re1[t + h] == re1[t] && ri1[t + h] < ri1[t])) { re1[t] = re1[t + h]; ri1[t] = ri1[t + h]; }
            if (re2[t + h] > re2[t] || (re2[t + h] == re2[t] && ri2[t + h] < ri2[t])) { re2[t] = re2[t + h]; ri2[t] = ri2[t + h]; }
        }
        __syncthreads();
    }
    if (t == 0) {
        const double dt = *dtp;
        double dtbar = rs[0];
        if (a.ssl) {
            // this step's dt moves the start time of every later step: it takes the sensitivities
            // to their start times summed so far; then this step's own joins the sum
            const double S = a.tacc[0];
            dtbar += S;
            a.tacc[0] = fma(dt, rt[0], S);
        }
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

constexpr int kCX = 32, kCY = 4;   // cell kernel blocks
constexpr int kHX = 32, kHY = 8;   // face kernel blocks

thread_local std::string g_adj_err;

}  // namespace

struct dense_adjoint {
    dense_handle_t* h = nullptr;  // the forward solver: its buffers, kernels and step graph
    dense_config_t cfg{};
    int k = 20;                   // checkpoint every k steps
    int ni = 0, nj = 0;
    size_t state = 0;             // doubles per compact state: 4 ni nj
    size_t tape_stage = 0;        // doubles of one stage's tape (both directions)
    AdjParams ap{};
    double* ckpt = nullptr;  int ckpt_cap = 0;    // states at steps 0, k, 2k, ...
    double* dts = nullptr;   int dts_cap = 0;     // dt of every forward step, then (from dts_cap
                                                  // on) each step's start time
    int* argmax = nullptr;   int argmax_cap = 0;  // per step: cells of the two maxima
    double* rec = nullptr;                        // k steps x 3 stage states of one segment
    double* tape = nullptr;                       // k steps x 3 stage tapes of one segment
    double *g = nullptr, *g1 = nullptr, *g2 = nullptr, *acc = nullptr, *hb = nullptr;
    double* part = nullptr;  int npart = 0;       // per stage: k_hbar blocks
    double* mpart = nullptr; int nm = 0;
    // GLF: the stage's (lambda_x, lambda_y, their cells), block maxima, block sums of lambda's
    // sensitivity
    double *lamv = nullptr, *lmp = nullptr, *lpart = nullptr;
    // the characteristic schemes (104, 105): the faces' split-flux sensitivities (40 planes a
    // direction; 50 with AdaWENO's densities) the cell kernel gathers
    double* fbar = nullptr;
    dim3 gh, gc, gfx, gfy;
    int nsteps = -1;                              // steps of the last forward
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    long long launches = 0;
    std::string err;
    // A full segment's recompute and reverse as CUDA graphs, the same for every segment: they
    // read and write the segment buffers (rec, tape) and the segment's slices of the time steps
    // and maxima cells, copied into seg_dts / out of seg_argmax around the reverse.
    cudaGraphExec_t rec_exec = nullptr, rev_exec = nullptr;
    long long rec_nodes = 0, rev_nodes = 0;
    dense::Params rec_prm{};                      // the solver parameters rec_exec was built with
    double* seg_dts = nullptr;
    int* seg_argmax = nullptr;
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

// one stage of the forward solver with taping sweeps: boundary, flux_tape xi and eta, update.
// Launched eagerly, directly on the solver's stream: forking the eta sweep onto a second stream
// made the eagerly launched backward 34 % slower (the fork pays inside a graph: graph_stage).
int taped_stage(dense_adjoint* a, int irk, double* tape) {
    dense_handle* h = a->h;
    dense::Params p = h->prm;
    p.tape = tape;
    h->kt->bc(h->prm, h->stream);
    h->kt->flux_tape(p, irk, 0, h->stream);
    h->kt->flux_tape(p, irk, 1, h->stream);
    h->kt->update(h->prm, irk, h->stream);
    a->launches += 4;
    return DENSE_OK;
}
// The same stage as graph nodes (under stream capture), like the step graph's stage: the eta
// taping sweep a branch beside the xi sweep, and on grids periodic in x and y no boundary fill
// in stages 2 and 3 (the previous update wrote the ghost layers).
cudaError_t graph_stage(dense_adjoint* a, int irk, double* tape) {
    dense_handle* h = a->h;
    dense::Params p = h->prm;
    p.tape = tape;
    if (irk == 1 || !h->prm.periodic_ghosts) {
        h->kt->bc(h->prm, h->stream);
        a->launches += 1;
    }
    cudaError_t e = cudaEventRecord(h->ev_fork, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->side, h->ev_fork, 0);
    if (e != cudaSuccess) return e;
    h->kt->flux_tape(p, irk, 1, h->side);
    h->kt->flux_tape(p, irk, 0, h->stream);
    e = cudaEventRecord(h->ev_join, h->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, h->ev_join, 0);
    if (e != cudaSuccess) return e;
    h->kt->update(h->prm, irk, h->stream);
    a->launches += 3;
    return cudaSuccess;
}

template <int REC, int SPL, bool WALLS>
void launch_rev_w(dense_adjoint* a, int stage, const double* u, const double* tape, const double* w, double* out,
                  const double* dtp, const double* tp, cudaStream_t s) {
    using namespace dense::adj;
    const dim3 bc(kCX, kCY);
    double* const lv = a->lamv;
    double* const lp = a->lpart;
    const double* hb = a->hb;
    if (stage == 0)
        k_rev<REC, SPL, WALLS><<<a->gc, bc, 0, s>>>(a->ap, u, w, tape, hb, nullptr, out, nullptr, tp, nullptr,
                                                    lv, lp, 0);
    else
        k_rev<REC, SPL, WALLS><<<a->gc, bc, 0, s>>>(a->ap, u, w, tape, hb, a->acc, out, dtp, tp,
                                                    stage == 1 ? a->mpart : nullptr, lv, lp, stage);
}
template <int REC, int SPL>
void launch_rev(dense_adjoint* a, int stage, const double* u, const double* tape, const double* w, double* out,
                const double* dtp, const double* tp, cudaStream_t s) {
    const int* r = a->ap.rule;
    const bool walls = r[0] != dense::adj::kRulePeriodic || r[2] != dense::adj::kRulePeriodic;
    if (walls) launch_rev_w<REC, SPL, true>(a, stage, u, tape, w, out, dtp, tp, s);
    else       launch_rev_w<REC, SPL, false>(a, stage, u, tape, w, out, dtp, tp, s);
}
template <int SPL>
void launch_rev_recon(dense_adjoint* a, int stage, const double* u, const double* tape, const double* w,
                      double* out, const double* dtp, const double* tp, cudaStream_t s) {
    switch (a->cfg.recon) {
    case DENSE_RECON_UPWIND5: launch_rev<DENSE_RECON_UPWIND5, SPL>(a, stage, u, tape, w, out, dtp, tp, s); break;
    case DENSE_RECON_WENOJS5: launch_rev<DENSE_RECON_WENOJS5, SPL>(a, stage, u, tape, w, out, dtp, tp, s); break;
    default:                  launch_rev<DENSE_RECON_WENOZ5, SPL>(a, stage, u, tape, w, out, dtp, tp, s); break;
    }
}

// the reverse of one stage: hbar of w on every face (and w . L(u) per block into part), then
// the cells; GLF (and the characteristic scheme, which splits by GLF) first finds the stage's
// global lambda and its cells, and last sends lambda's sensitivity to those cells; the
// characteristic scheme takes each face's reverse (k_char_face) before the cells gather it
void vjp(dense_adjoint* a, int stage, const double* u, const double* tape, const double* w, double* out,
         double* part, const double* dtp, const double* tp) {
    using namespace dense::adj;
    cudaStream_t s = a->h->stream;
    const bool charac = a->ap.charac != 0;
    const bool glf = a->cfg.splitting == DENSE_SPLIT_GLF || charac;
    if (glf) {
        k_maxarg<<<a->gc, dim3(kCX, kCY), 0, s>>>(a->ap, u, a->lmp);
        k_maxred<<<1, 256, 0, s>>>(a->lmp, a->nm, a->lamv);
        a->launches += 2;
    }
    k_hbar<<<a->gh, dim3(kHX, kHY), 0, s>>>(a->ap, w, tape, a->hb, part);
    if (charac) {
        const double* flags = a->ap.adapt ? tape : nullptr;  // the branches taken, first plane a direction
        k_char_face<0><<<a->gfx, dim3(kCX, kCY), 0, s>>>(a->ap, u, a->hb, a->lamv, tp, flags, a->fbar);
        k_char_face<1><<<a->gfy, dim3(kCX, kCY), 0, s>>>(a->ap, u, a->hb, a->lamv, tp, flags, a->fbar);
        a->launches += 2;
        launch_rev<dense::adj::kRecFaceSens, 1>(a, stage, u, a->fbar, w, out, dtp, tp, s);  // the faces' own sensitivities
    } else if (glf) launch_rev_recon<1>(a, stage, u, tape, w, out, dtp, tp, s);
    else if (a->cfg.splitting == DENSE_SPLIT_SW) launch_rev_recon<2>(a, stage, u, tape, w, out, dtp, tp, s);
    else launch_rev_recon<0>(a, stage, u, tape, w, out, dtp, tp, s);
    a->launches += 2;
    if (glf) {
        switch (stage) {
        case 3: k_lamg<3><<<1, 256, 0, s>>>(a->ap, a->lpart, a->nm, a->lamv, u, dtp, out); break;
        case 2: k_lamg<2><<<1, 256, 0, s>>>(a->ap, a->lpart, a->nm, a->lamv, u, dtp, out); break;
        case 1: k_lamg<1><<<1, 256, 0, s>>>(a->ap, a->lpart, a->nm, a->lamv, u, dtp, out); break;
        default: k_lamg<0><<<1, 256, 0, s>>>(a->ap, a->lpart, a->nm, a->lamv, u, dtp, out); break;
        }
        a->launches += 1;
    }
}

// reverse of one step from its three recorded stage states and tapes, its time step *dtp, its
// start time *tp and the slot of its maxima cells; g holds dJ/du(n+1) on entry and dJ/du(n) on
// return
void reverse_step(dense_adjoint* a, const double* rec_step, const double* tape_step, const double* dtp,
                  const double* tp, int* argmax) {
    const double* u[3] = {rec_step, rec_step + a->state, rec_step + 2 * a->state};
    const double* t[3] = {tape_step, tape_step + a->tape_stage, tape_step + 2 * a->tape_stage};
    vjp(a, 3, u[2], t[2], a->g, a->g2, a->part + 2 * a->npart, dtp, tp);
    vjp(a, 2, u[1], t[1], a->g2, a->g1, a->part + 1 * a->npart, dtp, tp);
    vjp(a, 1, u[0], t[0], a->g1, a->g, a->part, dtp, tp);
    if (!a->cfg.if_const_dt) {
        dense::adj::k_dt<<<1, 256, 0, a->h->stream>>>(a->ap, a->part, a->npart, a->mpart, a->nm, u[0], a->g, dtp,
                                                      argmax);
        a->launches += 1;
    }
}

// record the stage inputs of a segment's step s and recompute it with taping sweeps
int recompute_step(dense_adjoint* a, int s, bool graph) {
    dense_handle* h = a->h;
    h->kt->step_begin(h->prm, h->stream);
    for (int irk = 1; irk <= 3; ++irk) {
        int rc = from_solver(a, a->rec + ((size_t)s * 3 + irk - 1) * a->state);
        if (rc) return rc;
        double* tape = a->tape + ((size_t)s * 3 + irk - 1) * a->tape_stage;
        if (graph) {
            const cudaError_t e = graph_stage(a, irk, tape);
            if (e != cudaSuccess) return aerr(a, DENSE_ERR_CUDA, std::string("segment graph: ") + cudaGetErrorString(e));
        } else {
            rc = taped_stage(a, irk, tape);
            if (rc) return rc;
        }
    }
    h->kt->step_end(h->prm, h->stream);
    a->launches += 2;
    return DENSE_OK;
}

// Capture `body` (launches on the solver's stream) as a graph; *nodes = the kernels it launched.
template <class F>
int capture(dense_adjoint* a, F body, cudaGraphExec_t* exec, long long* nodes) {
    dense_handle* h = a->h;
    if (*exec) cudaGraphExecDestroy(*exec);
    *exec = nullptr;
    const long long l0 = a->launches;
    ACK(a, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = body();
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    *nodes = a->launches - l0;
    a->launches = l0;
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return aerr(a, DENSE_ERR_CUDA, std::string("segment capture: ") + cudaGetErrorString(e));
    const cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return aerr(a, DENSE_ERR_CUDA, std::string("segment graph: ") + cudaGetErrorString(ie));
    return DENSE_OK;
}

// the graphs of a full segment (k steps), built on first use and again when the solver's
// parameters have changed since
int segment_graphs(dense_adjoint* a) {
    dense_handle* h = a->h;
    if (!a->rec_exec || std::memcmp(&a->rec_prm, &h->prm, sizeof(h->prm)) != 0) {
        AH(a, dense::handle_ensure_side(h));
        int rc = capture(a, [&] {
            for (int s = 0; s < a->k; ++s) {
                const int r = recompute_step(a, s, true);
                if (r) return r;
            }
            return (int)DENSE_OK;
        }, &a->rec_exec, &a->rec_nodes);
        if (rc) return rc;
        a->rec_prm = h->prm;
    }
    if (!a->rev_exec) {
        int rc = capture(a, [&] {
            for (int s = a->k - 1; s >= 0; --s)
                reverse_step(a, a->rec + (size_t)s * 3 * a->state, a->tape + (size_t)s * 3 * a->tape_stage,
                             a->seg_dts + s, a->seg_dts + a->k + s, a->seg_argmax + 2 * s);
            return (int)DENSE_OK;
        }, &a->rev_exec, &a->rev_nodes);
        if (rc) return rc;
    }
    return DENSE_OK;
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

int dense_adjoint_get_solver(dense_adjoint_t* a, dense_handle_t** h) {
    if (!a || !h) return aerr(a, DENSE_ERR_ARG, "null argument");
    *h = a->h;
    return DENSE_OK;
}

void dense_adjoint_destroy(dense_adjoint_t* a) {
    if (!a) return;
    if (a->h) cudaStreamSynchronize(a->h->stream);
    double* bufs[] = {a->ckpt, a->dts, a->rec, a->tape, a->g, a->g1, a->g2, a->acc, a->hb, a->part, a->mpart,
                      a->lamv, a->lmp, a->lpart, a->seg_dts, a->ap.bpart, a->fbar, a->ap.rbar,
                      a->ap.tpart, a->ap.tacc};
    for (double* b : bufs) if (b) cudaFree(b);
    if (a->argmax) cudaFree(a->argmax);
    if (a->seg_argmax) cudaFree(a->seg_argmax);
    if (a->rec_exec) cudaGraphExecDestroy(a->rec_exec);
    if (a->rev_exec) cudaGraphExecDestroy(a->rev_exec);
    if (a->ev_in) cudaEventDestroy(a->ev_in);
    if (a->ev_out) cudaEventDestroy(a->ev_out);
    if (a->h) dense_destroy(a->h);
    delete a;
}

int dense_adjoint_create(const dense_config_t* cfg, int checkpoint_every, dense_adjoint_t** out) {
    if (!out || !cfg) return aerr(nullptr, DENSE_ERR_ARG, "null argument");
    *out = nullptr;
    const bool adapt = cfg->splitting == DENSE_SPLIT_SC;
    const bool charac = cfg->splitting == DENSE_SPLIT_CH || adapt;
    if (cfg->splitting != DENSE_SPLIT_LLF && cfg->splitting != DENSE_SPLIT_GLF && cfg->splitting != DENSE_SPLIT_SW &&
        !charac)
        return aerr(nullptr, DENSE_ERR_ARG,
                    "the adjoint covers the LLF, GLF and Steger-Warming splittings (101-103), the characteristic "
                    "WENO-Z (104) and AdaWENO (105)");
    // the characteristic schemes reconstruct by their own WENO-Z; the recon field is not read
    if (!charac && cfg->recon != DENSE_RECON_UPWIND5 && cfg->recon != DENSE_RECON_WENOJS5 &&
        cfg->recon != DENSE_RECON_WENOZ5)
        return aerr(nullptr, DENSE_ERR_ARG, "the adjoint covers reconstructions 251, 253 and 255");
    // ghost rules (bottom, top, left, right) of the benchmarks covered: periodic, the
    // extrapolation, the mirror and fixed states (boundary_ivc/sedov/rm/shockvortex/rt_general.f90)
    int rules[4];
    switch (cfg->benchmark) {
    case DENSE_BENCH_IVC_PERIODIC: case DENSE_BENCH_RM_PERIODIC:
        rules[0] = rules[1] = rules[2] = rules[3] = dense::adj::kRulePeriodic; break;
    case DENSE_BENCH_IVC:  // y periodic, x extrapolated
        rules[0] = rules[1] = dense::adj::kRulePeriodic; rules[2] = rules[3] = dense::adj::kRuleExtrap; break;
    case DENSE_BENCH_SEDOV:  // mirror bottom and left, extrapolation top and right
        rules[0] = rules[2] = dense::adj::kRuleReflect; rules[1] = rules[3] = dense::adj::kRuleExtrap; break;
    case DENSE_BENCH_RM: case DENSE_BENCH_SHOCKVORTEX:  // mirror bottom and top, extrapolated sides
        rules[0] = rules[1] = dense::adj::kRuleReflect; rules[2] = rules[3] = dense::adj::kRuleExtrap; break;
    case DENSE_BENCH_RT:  // fixed bottom and top states, periodic sides
        rules[0] = rules[1] = dense::adj::kRuleFixed; rules[2] = rules[3] = dense::adj::kRulePeriodic; break;
    case DENSE_BENCH_RT_REFLECT:  // fixed bottom and top states, mirror sides
        rules[0] = rules[1] = dense::adj::kRuleFixed; rules[2] = rules[3] = dense::adj::kRuleReflect; break;
    case DENSE_BENCH_DMR:  // wall from x = 1/6 on, moving-shock top, inflow left, extrapolated right
        rules[0] = dense::adj::kRuleDMRBottom; rules[1] = rules[2] = dense::adj::kRuleFixed;
        rules[3] = dense::adj::kRuleExtrap; break;
    case DENSE_BENCH_SSL:  // mirror bottom, the setup's top ghosts, oscillating inflow, extrapolated right
        rules[0] = dense::adj::kRuleReflect; rules[1] = dense::adj::kRuleFixed;
        rules[2] = dense::adj::kRuleSSLInflow; rules[3] = dense::adj::kRuleExtrap; break;
    default:
        return aerr(nullptr, DENSE_ERR_ARG,
                    "the adjoint covers the benchmarks 1, 2, 3, 4, 5, 6, 9, 11, 13 and 14");
    }
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
    if (cfg->benchmark == DENSE_BENCH_DMR) {
        // the forward solver's boundary rows of the cell centres x = (i - 1/2) dx (init centres):
        // the bottom wall starts at x = 1/6, the top state follows the shock
        std::vector<double> xs(cfg->ni);
        for (int i = 0; i < cfg->ni; ++i) xs[i] = ((double)(i + 1) - 0.5) * cfg->dx;
        if (cudaMemcpy(a->h->xbot, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(a->h->xtop, xs.data(), xs.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
            a->err = "cudaMemcpy of the boundary rows failed";
            return fail(DENSE_ERR_CUDA);
        }
    }
    if (cfg->benchmark == DENSE_BENCH_SSL) {
        // the setup's state once, for what the restarts (interior only) do not write: the top
        // ghost rows, which the shear layer's rule never refills, and the rows' y of the inflow
        dense_config_t c2 = *cfg;
        long long nc = 0, np_ = 0, nxy = 0;
        if (dense_array_sizes(&c2, &nc, &np_, &nxy) != DENSE_OK) {
            a->err = "dense_array_sizes failed";
            return fail(DENSE_ERR_ARG);
        }
        std::vector<double> cons((size_t)nc), prim((size_t)np_), xs((size_t)nxy), ys((size_t)nxy);
        if (dense_init_setup(&c2, cons.data(), prim.data(), xs.data(), ys.data()) != DENSE_OK ||
            dense_upload(a->h, cons.data(), prim.data(), xs.data(), ys.data()) != DENSE_OK ||
            cudaStreamSynchronize(a->h->stream) != cudaSuccess) {
            a->err = std::string("the shear layer's setup state: ") + dense_last_error(a->h);
            return fail(DENSE_ERR_CUDA);
        }
    }
    AdjParams& p = a->ap;
    p.ni = cfg->ni; p.nj = cfg->nj; p.plane = (long long)cfg->ni * cfg->nj;
    p.xs = (long long)cfg->nj * (cfg->ni + 1);
    p.ys = (long long)(cfg->nj + 1) * cfg->ni;
    p.np = adapt ? 5 : charac ? 4 : dense::tape_planes(cfg->recon);
    p.gnp = adapt ? 50 : charac ? 40 : p.np;
    p.charac = charac ? 1 : 0;
    p.adapt = adapt ? 1 : 0;
    p.gamma = cfg->gamma; p.dx = cfg->dx; p.dy = cfg->dy; p.inv_dx = 1.0 / cfg->dx; p.inv_dy = 1.0 / cfg->dy;
    p.cfl = cfg->cfl;
    for (int k = 0; k < 4; ++k) p.rule[k] = rules[k];
    // the forward solver applies the body force on the same condition (fill_params)
    p.bodyforce = cfg->if_bodyforce &&
                  (cfg->benchmark == DENSE_BENCH_RT || cfg->benchmark == DENSE_BENCH_RT_REFLECT);
    p.bench = cfg->benchmark;
    p.ssl = cfg->benchmark == DENSE_BENCH_SSL ? 1 : 0;
    p.yleft = a->h->yleft;
    a->tape_stage = (size_t)p.np * (size_t)(p.xs + p.ys);
    a->gh = dim3((cfg->ni + 1 + kHX - 1) / kHX, (cfg->nj + 1 + kHY - 1) / kHY, 2);
    a->gc = dim3((cfg->ni + kCX - 1) / kCX, (cfg->nj + kCY - 1) / kCY);
    // k_char_face blocks: 16 faces x 4 lines (xi), 16 lines x 4 faces (eta), two threads a face
    a->gfx = dim3((cfg->ni + 1 + 15) / 16, (cfg->nj + 3) / 4);
    a->gfy = dim3((cfg->ni + 15) / 16, (cfg->nj + 1 + 3) / 4);
    a->npart = (int)(a->gh.x * a->gh.y * a->gh.z);
    a->nm = (int)(a->gc.x * a->gc.y);
    struct B { double** p; size_t n; } bufs[] = {
        {&a->g, a->state}, {&a->g1, a->state}, {&a->g2, a->state}, {&a->acc, a->state},
        {&a->hb, (size_t)4 * (p.xs + p.ys)}, {&a->part, (size_t)3 * a->npart}, {&a->mpart, (size_t)4 * a->nm},
        {&a->rec, (size_t)3 * a->k * a->state}, {&a->tape, (size_t)3 * a->k * a->tape_stage},
        {&a->lamv, 4}, {&a->lmp, (size_t)4 * a->nm}, {&a->lpart, (size_t)2 * a->nm}, {&a->seg_dts, (size_t)2 * a->k},
        {&p.bpart, (size_t)3 * a->nm}, {&p.tpart, (size_t)3 * a->nm}, {&p.tacc, 1},
    };
    for (auto& b : bufs) {
        cudaError_t e = cudaMalloc((void**)b.p, b.n * sizeof(double));
        if (e != cudaSuccess) { a->err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return fail(DENSE_ERR_NOMEM); }
    }
    if (charac) {
        const size_t fp = (size_t)(p.xs + p.ys);
        struct B2 { double** p; size_t n; } cb[] = {{&a->fbar, (size_t)p.gnp * fp}, {&p.rbar, 8 * fp}};
        for (auto& b : cb) {
            cudaError_t e = cudaMalloc((void**)b.p, b.n * sizeof(double));
            if (e != cudaSuccess) { a->err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return fail(DENSE_ERR_NOMEM); }
        }
    }
    if (cudaMalloc((void**)&a->seg_argmax, (size_t)2 * a->k * sizeof(int)) != cudaSuccess) {
        a->err = "cudaMalloc of the segment's maxima cells failed";
        return fail(DENSE_ERR_NOMEM);
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
    dense::NvtxRange nvtx_("dense_adjoint_forward");
    if (!a || !u0 || !uT) return aerr(a, DENSE_ERR_ARG, "null argument");
    if (nsteps < 0) return aerr(a, DENSE_ERR_ARG, "nsteps < 0");
    const int nseg = (nsteps + a->k - 1) / a->k;
    int rc = grow(a, &a->ckpt, &a->ckpt_cap, nseg > 0 ? nseg : 1, a->state);
    if (!rc) rc = grow(a, &a->dts, &a->dts_cap, nsteps > 0 ? nsteps : 1, 2);
    if (!rc) rc = grow(a, &a->argmax, &a->argmax_cap, nsteps > 0 ? nsteps : 1, 2);
    if (rc) return rc;
    a->nsteps = -1;
    rc = begin(a, stream);
    if (rc) return rc;
    ACK(a, cudaMemsetAsync(a->argmax, 0xff, (size_t)2 * a->argmax_cap * sizeof(int), a->h->stream));
    rc = restart(a, u0);
    if (rc) return rc;
    AH(a, dense::handle_step_graph(a->h));
    dense_handle* h = a->h;
    for (int s = 0; s < nsteps; ++s) {
        if (s % a->k == 0) {
            rc = from_solver(a, a->ckpt + (size_t)(s / a->k) * a->state);
            if (rc) return rc;
        }
        ACK(a, cudaMemcpyAsync(a->dts + a->dts_cap + s, &h->sc->t, sizeof(double), cudaMemcpyDeviceToDevice,
                               h->stream));
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
    dense::NvtxRange nvtx_("dense_adjoint_backward");
    if (!a || !gT || !g0) return aerr(a, DENSE_ERR_ARG, "null argument");
    if (a->nsteps < 0) return aerr(a, DENSE_ERR_STATE, "dense_adjoint_backward before dense_adjoint_forward");
    int rc = begin(a, stream);
    if (rc) return rc;
    dense_handle* h = a->h;
    ACK(a, cudaMemcpyAsync(a->g, gT, a->state * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    if (a->ap.ssl) ACK(a, cudaMemsetAsync(a->ap.tacc, 0, sizeof(double), h->stream));  // no later step yet
    const int nseg = (a->nsteps + a->k - 1) / a->k;
    if (a->nsteps >= a->k) {
        rc = segment_graphs(a);
        if (rc) return rc;
    }
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int s0 = seg * a->k, len = std::min(a->k, a->nsteps - s0);
        rc = restart(a, a->ckpt + (size_t)seg * a->state);
        if (rc) return rc;
        // the segment's start time (the double Mach reflection's top ghosts move with it)
        ACK(a, cudaMemcpyAsync(&h->sc->t, a->dts + a->dts_cap + s0, sizeof(double), cudaMemcpyDeviceToDevice,
                               h->stream));
        if (len == a->k) {
            // a full segment: its recompute (recording each stage's input state, taping the
            // sweeps) and its reverse as the segment graphs
            ACK(a, cudaGraphLaunch(a->rec_exec, h->stream));
            ACK(a, cudaMemcpyAsync(a->seg_dts, a->dts + s0, (size_t)a->k * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
            ACK(a, cudaMemcpyAsync(a->seg_dts + a->k, a->dts + a->dts_cap + s0, (size_t)a->k * sizeof(double),
                                   cudaMemcpyDeviceToDevice, h->stream));
            ACK(a, cudaGraphLaunch(a->rev_exec, h->stream));
            ACK(a, cudaMemcpyAsync(a->argmax + 2 * (size_t)s0, a->seg_argmax, (size_t)2 * a->k * sizeof(int),
                                   cudaMemcpyDeviceToDevice, h->stream));
            a->launches += a->rec_nodes + a->rev_nodes;
            continue;
        }
        for (int s = 0; s < len; ++s) {
            rc = recompute_step(a, s, false);
            if (rc) return rc;
        }
        for (int s = len - 1; s >= 0; --s)
            reverse_step(a, a->rec + (size_t)s * 3 * a->state, a->tape + (size_t)s * 3 * a->tape_stage,
                         a->dts + s0 + s, a->dts + a->dts_cap + s0 + s, a->argmax + 2 * (s0 + s));
    }
    h->prim_slot = -1;
    ACK(a, cudaMemcpyAsync(g0, a->g, a->state * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return finish(a, stream);
}

int dense_adjoint_rhs_vjp(dense_adjoint_t* a, const double* u, const double* v, double* out, double* vdotl,
                          void* stream) {
    dense::NvtxRange nvtx_("dense_adjoint_rhs_vjp");
    if (!a || !u || !v || !out) return aerr(a, DENSE_ERR_ARG, "null argument");
    int rc = begin(a, stream);
    if (!rc) rc = restart(a, u);
    if (rc) return rc;
    // the first stage's sweeps at u tape its reconstructions and fluxes (the update's result is
    // not used); step_begin opens the stage (the loop bounds are open after restart)
    a->h->kt->step_begin(a->h->prm, a->h->stream);
    a->launches += 1;
    rc = taped_stage(a, 1, a->tape);
    if (rc) return rc;
    a->h->prim_slot = -1;
    vjp(a, 0, u, a->tape, v, out, a->part, nullptr, nullptr);
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
