// dense_oracle.cpp — TEST INFRASTRUCTURE ONLY: the CPU oracle for the 2DENSE hot path.
//
// A line-faithful C++ restatement of the reference Fortran solver's per-stage path (primitive
// recovery, boundary fill, flux splitting, reconstruction, TVD-RK3) and its initial setups.
// It exists to check the GPU kernels and to time a CPU baseline; nothing in the product links,
// imports or calls it. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// may load it.
//
// Fidelity rules (the reference is built with `gfortran -O2`, source/CMakeLists.txt:12):
//  * statement order and left-to-right evaluation as written in the Fortran;
//  * `x**2` -> x*x, `x**2.5d0` / `rho**gamma` -> pow();
//  * default-real (single) literals are promoted from float: 1.0e-6 -> (double)1.0e-6f;
//  * compile with -ffp-contract=off so no FMA is formed (gfortran -O2 on generic x86-64 forms
//    none); IEEE divide and sqrt.
// Common subexpressions that gfortran would evaluate once (sqrt(rho) in the Roe average,
// u+lambda in a splitting) are hoisted into locals; this does not change any result bit.
//
// Parity status: the reference Fortran cannot be compiled here (no Fortran compiler), so this
// restatement is pinned by mathematical known answers (free-stream preservation, polynomial
// exactness, L*R = I, symmetries, conservation), not by reference outputs.
//
// The scalar type T is `double` for results and timing, or `Counted` to count the floating
// point operations the reference executes on field values (FLOPs per cell-update).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>
#if defined(_OPENMP)
#include <omp.h>
#endif

#include "../include/dense2d.h"

namespace oracle {

// ---------------------------------------------------------------------------------------------
// Operation counter
struct OpCount {
    long long add = 0, mul = 0, div = 0, sqrt = 0, transc = 0;
};
static OpCount g_ops;

struct Counted {
    double v;
    Counted() : v(0.0) {}
    Counted(double x) : v(x) {}  // NOLINT: implicit on purpose (literals and scalars)
};
inline Counted operator+(Counted a, Counted b) { g_ops.add++; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { g_ops.add++; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { g_ops.mul++; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { g_ops.div++; return Counted(a.v / b.v); }
inline Counted operator-(Counted a) { return Counted(-a.v); }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { return a.v >= b.v; }
inline Counted sqrt(Counted a) { g_ops.sqrt++; return Counted(std::sqrt(a.v)); }
inline Counted fabs(Counted a) { return Counted(std::fabs(a.v)); }
inline Counted exp(Counted a) { g_ops.transc++; return Counted(std::exp(a.v)); }
inline Counted log(Counted a) { g_ops.transc++; return Counted(std::log(a.v)); }
inline Counted cos(Counted a) { g_ops.transc++; return Counted(std::cos(a.v)); }
inline Counted sin(Counted a) { g_ops.transc++; return Counted(std::sin(a.v)); }
inline Counted tanh(Counted a) { g_ops.transc++; return Counted(std::tanh(a.v)); }
inline Counted pow(Counted a, Counted b) { g_ops.transc++; return Counted(std::pow(a.v, b.v)); }
inline Counted fmax(Counted a, Counted b) { return Counted(std::fmax(a.v, b.v)); }
inline double val(Counted a) { return a.v; }
inline double val(double a) { return a; }

using std::sqrt; using std::fabs; using std::exp; using std::log; using std::cos; using std::sin;
using std::tanh; using std::pow; using std::fmax;

// Fortran default-real literal promoted to double precision.
static inline double SP(float f) { return (double)f; }

// weno module constants (source/inv_scheme/weno_mod.f90:3-14,37)
static const double a300 = 1.0 / 3.0, a301 = -7.0 / 6.0, a302 = 11.0 / 6.0;
static const double a310 = -1.0 / 6.0, a311 = 5.0 / 6.0, a312 = 1.0 / 3.0;
static const double a320 = 1.0 / 3.0, a321 = 5.0 / 6.0, a322 = -1.0 / 6.0;
static const double c30 = 0.1, c31 = 0.6, c32 = 0.3;
static const double ss = (double)1.0e-6f;  // weno_mod.f90:37, a default-real literal
static const double pie = 3.141592653589793115997963468544185161590576171875;  // atan(1d0)*4d0

template <class T> static inline T sq(T x) { return x * x; }

// weno5js_stencil_alpha (weno_mod.f90:146-165)
template <class T>
static inline void weno5js_alpha(const T lf[5], T& aa0, T& aa1, T& aa2) {
    T is0 = T(13.0) * sq(lf[0] - T(2.0) * lf[1] + lf[2]) / T(12.0)
          + sq(lf[0] - T(4.0) * lf[1] + T(3.0) * lf[2]) / T(4.0);
    T is1 = T(13.0) * sq(lf[1] - T(2.0) * lf[2] + lf[3]) / T(12.0)
          + sq(lf[1] - lf[3]) / T(4.0);
    T is2 = T(13.0) * sq(lf[2] - T(2.0) * lf[3] + lf[4]) / T(12.0)
          + sq(T(3.0) * lf[2] - T(4.0) * lf[3] + lf[4]) / T(4.0);
    aa0 = T(c30) / sq(T(ss) + is0);
    aa1 = T(c31) / sq(T(ss) + is1);
    aa2 = T(c32) / sq(T(ss) + is2);
}

// weno5z_stencil_alpha (weno_mod.f90:168-189)
template <class T>
static inline void weno5z_alpha(const T lf[5], T& aa0, T& aa1, T& aa2) {
    T is0 = T(13.0) * sq(lf[0] - T(2.0) * lf[1] + lf[2]) / T(12.0)
          + sq(lf[0] - T(4.0) * lf[1] + T(3.0) * lf[2]) / T(4.0);
    T is1 = T(13.0) * sq(lf[1] - T(2.0) * lf[2] + lf[3]) / T(12.0)
          + sq(lf[1] - lf[3]) / T(4.0);
    T is2 = T(13.0) * sq(lf[2] - T(2.0) * lf[3] + lf[4]) / T(12.0)
          + sq(T(3.0) * lf[2] - T(4.0) * lf[3] + lf[4]) / T(4.0);
    T tau5 = fabs(is2 - is0);
    aa0 = T(c30) * (T(1.0) + sq(tau5 / (T(ss) + is0)));
    aa1 = T(c31) * (T(1.0) + sq(tau5 / (T(ss) + is1)));
    aa2 = T(c32) * (T(1.0) + sq(tau5 / (T(ss) + is2)));
}

// The three third-order candidate values (weno_mod.f90:57-59).
template <class T>
static inline void candidates(const T lf[5], T& q30, T& q31, T& q32) {
    q30 = T(a300) * lf[0] + T(a301) * lf[1] + T(a302) * lf[2];
    q31 = T(a310) * lf[1] + T(a311) * lf[2] + T(a312) * lf[3];
    q32 = T(a320) * lf[2] + T(a321) * lf[3] + T(a322) * lf[4];
}

// weno5js_stencil (weno_mod.f90:98-112) with omega_only (:115-127)
template <class T> static inline T weno5js(const T lf[5]) {
    T q30, q31, q32, aa0, aa1, aa2;
    candidates(lf, q30, q31, q32);
    weno5js_alpha(lf, aa0, aa1, aa2);
    T s = aa0 + aa1 + aa2;
    T w0 = aa0 / s, w1 = aa1 / s, w2 = aa2 / s;
    return w0 * q30 + w1 * q31 + w2 * q32;
}

// weno5z_stencil (weno_mod.f90:50-64) with omega_only (:67-79)
template <class T> static inline T weno5z(const T lf[5]) {
    T q30, q31, q32, aa0, aa1, aa2;
    candidates(lf, q30, q31, q32);
    weno5z_alpha(lf, aa0, aa1, aa2);
    T s = aa0 + aa1 + aa2;
    T w0 = aa0 / s, w1 = aa1 / s, w2 = aa2 / s;
    return w0 * q30 + w1 * q31 + w2 * q32;
}

// weno5z_stencil_omega_theta (weno_mod.f90:82-95)
template <class T>
static inline void weno5z_omega_theta(const T lf[5], T& w0, T& w1, T& w2, T& theta) {
    T aa0, aa1, aa2;
    weno5z_alpha(lf, aa0, aa1, aa2);
    T s = aa0 + aa1 + aa2;
    w0 = aa0 / s; w1 = aa1 / s; w2 = aa2 / s;
    theta = T(1.0) / (T(1.0) + sq(s - T(1.0)));
}

// upwind5 (scheme_upwind5_general.f90:86-90)
template <class T> static inline T upwind5(const T lf[5]) {
    return (T(2.0) * lf[0] - T(13.0) * lf[1] + T(47.0) * lf[2] + T(27.0) * lf[3]
            - T(3.0) * lf[4]) / T(60.0);
}

#if defined(_OPENMP)
#define OMP_FOR _Pragma("omp parallel for schedule(static) if(kPar)")
#else
#define OMP_FOR
#endif

// ---------------------------------------------------------------------------------------------
template <class T> struct Solver {
    static constexpr bool kPar = std::is_same<T, double>::value;

    dense_config_t cfg;
    int ni, nj, b, NIp, NJp;
    double gamma, cfl, delta;
    double dx, dy;                  // block geometry (init_*_general.f90)
    double dt;                      // flow_general::dt
    double current_time = 0.0, elasp_time = 0.0;
    int current_step = 0;
    T max_eig_i = 0.0, max_eig_j = 0.0;
    bool bodyforce_alloc = false;   // allocate_block allocated bodyforce (if_bodyforce at init)
    bool recon_noop = false;

    std::vector<T> cons, prim, cons_temp, bodyforce;
    std::vector<T> flux_xi, flux_eta, flux_xip, flux_xin, flux_etap, flux_etan;
    std::vector<T> h_xip, h_xin, h_etap, h_etan, h_xi, h_eta;
    std::vector<T> theta_xip, theta_xin, theta_etap, theta_etan;
    std::vector<double> x, y;

    static long long ops_now() { return g_ops.add + g_ops.mul + g_ops.div + g_ops.sqrt; }

    explicit Solver(const dense_config_t& c) : cfg(c) {
        ni = c.ni; nj = c.nj; b = 4; NIp = ni + 2 * b; NJp = nj + 2 * b;
        gamma = c.gamma; cfl = c.cfl; delta = c.delta; dt = c.dt;
        dx = c.dx; dy = c.dy;
        size_t P = (size_t)NIp * NJp;
        cons.assign(P * 4, T(0.0)); prim.assign(P * 6, T(0.0)); cons_temp.assign(P * 4, T(0.0));
        bodyforce.assign(P * 4, T(0.0));
        flux_xi.assign((size_t)NIp * nj * 4, T(0.0)); flux_eta.assign((size_t)NJp * ni * 4, T(0.0));
        flux_xip.assign((size_t)NIp * nj * 4, T(0.0)); flux_xin.assign((size_t)NIp * nj * 4, T(0.0));
        flux_etap.assign((size_t)NJp * ni * 4, T(0.0)); flux_etan.assign((size_t)NJp * ni * 4, T(0.0));
        size_t HX = (size_t)(ni + 1) * nj * 4, HE = (size_t)(nj + 1) * ni * 4;
        h_xip.assign(HX, T(0.0)); h_xin.assign(HX, T(0.0)); h_xi.assign(HX, T(0.0));
        h_etap.assign(HE, T(0.0)); h_etan.assign(HE, T(0.0)); h_eta.assign(HE, T(0.0));
        theta_xip.assign((size_t)4 * (ni + 1) * nj, T(0.0)); theta_xin.assign((size_t)4 * (ni + 1) * nj, T(0.0));
        theta_etap.assign((size_t)4 * (nj + 1) * ni, T(0.0)); theta_etan.assign((size_t)4 * (nj + 1) * ni, T(0.0));
        x.assign((size_t)ni * nj, 0.0); y.assign((size_t)ni * nj, 0.0);
        bodyforce_alloc = c.if_bodyforce != 0;
    }

    // 1-based Fortran accessors
    T& C(int i, int j, int v) { return cons[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)NJp * (v - 1))]; }
    T& Pm(int i, int j, int v) { return prim[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)NJp * (v - 1))]; }
    T& CT(int i, int j, int v) { return cons_temp[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)NJp * (v - 1))]; }
    T& BF(int i, int j, int v) { return bodyforce[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)NJp * (v - 1))]; }
    T& FXP(int i, int j, int v) { return flux_xip[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)nj * (v - 1))]; }
    T& FXN(int i, int j, int v) { return flux_xin[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)nj * (v - 1))]; }
    T& FX(int i, int j, int v) { return flux_xi[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)nj * (v - 1))]; }
    T& FEP(int j, int i, int v) { return flux_etap[(size_t)(j - 1) + (size_t)NJp * ((size_t)(i - 1) + (size_t)ni * (v - 1))]; }
    T& FEN(int j, int i, int v) { return flux_etan[(size_t)(j - 1) + (size_t)NJp * ((size_t)(i - 1) + (size_t)ni * (v - 1))]; }
    T& FE(int j, int i, int v) { return flux_eta[(size_t)(j - 1) + (size_t)NJp * ((size_t)(i - 1) + (size_t)ni * (v - 1))]; }
    T& HXP(int i, int j, int v) { return h_xip[(size_t)(i - 1) + (size_t)(ni + 1) * ((size_t)(j - 1) + (size_t)nj * (v - 1))]; }
    T& HXN(int i, int j, int v) { return h_xin[(size_t)(i - 1) + (size_t)(ni + 1) * ((size_t)(j - 1) + (size_t)nj * (v - 1))]; }
    T& HX(int i, int j, int v) { return h_xi[(size_t)(i - 1) + (size_t)(ni + 1) * ((size_t)(j - 1) + (size_t)nj * (v - 1))]; }
    T& HEP(int j, int i, int v) { return h_etap[(size_t)(j - 1) + (size_t)(nj + 1) * ((size_t)(i - 1) + (size_t)ni * (v - 1))]; }
    T& HEN(int j, int i, int v) { return h_etan[(size_t)(j - 1) + (size_t)(nj + 1) * ((size_t)(i - 1) + (size_t)ni * (v - 1))]; }
    T& HE(int j, int i, int v) { return h_eta[(size_t)(j - 1) + (size_t)(nj + 1) * ((size_t)(i - 1) + (size_t)ni * (v - 1))]; }
    T& TXP(int k, int i, int j) { return theta_xip[(size_t)(k - 1) + 4 * ((size_t)(i - 1) + (size_t)(ni + 1) * (j - 1))]; }
    T& TXN(int k, int i, int j) { return theta_xin[(size_t)(k - 1) + 4 * ((size_t)(i - 1) + (size_t)(ni + 1) * (j - 1))]; }
    T& TEP(int k, int j, int i) { return theta_etap[(size_t)(k - 1) + 4 * ((size_t)(j - 1) + (size_t)(nj + 1) * (i - 1))]; }
    T& TEN(int k, int j, int i) { return theta_etan[(size_t)(k - 1) + 4 * ((size_t)(j - 1) + (size_t)(nj + 1) * (i - 1))]; }
    double& X(int i, int j) { return x[(size_t)(i - 1) + (size_t)ni * (j - 1)]; }
    double& Y(int i, int j) { return y[(size_t)(i - 1) + (size_t)ni * (j - 1)]; }

    // =========================================================================================
    // get_primary_block (source/utility/get_primary.f90:25-78)
    void get_primary() {
        double mi = 0.0, mj = 0.0;
        T tmi = 0.0, tmj = 0.0;
        if (kPar) {
#if defined(_OPENMP)
#pragma omp parallel for schedule(static) reduction(max : mi, mj)
#endif
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) {
                    T e1, e2;
                    prim_cell(i, j, e1, e2);
                    mi = std::max(mi, val(e1));
                    mj = std::max(mj, val(e2));
                }
            max_eig_i = mi; max_eig_j = mj;
        } else {
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) {
                    T e1, e2;
                    prim_cell(i, j, e1, e2);
                    if (val(e1) > val(tmi)) tmi = e1;
                    if (val(e2) > val(tmj)) tmj = e2;
                }
            max_eig_i = tmi; max_eig_j = tmj;
        }
    }
    inline void prim_cell(int i, int j, T& e1, T& e2) {
        T rho = C(i, j, 1);
        T u = C(i, j, 2) / rho;
        T v = C(i, j, 3) / rho;
        T p = T(gamma - 1.0) * (C(i, j, 4) - T(0.5) * rho * (u * u + v * v));
        if (p < T(0.0)) p = T(SP(1.0e-6f));
        T alpha = sqrt(T(gamma) * p / rho);
        Pm(i, j, 1) = rho; Pm(i, j, 2) = u; Pm(i, j, 3) = v; Pm(i, j, 4) = p; Pm(i, j, 5) = alpha;
        Pm(i, j, 6) = log(p) - log(rho);
        e1 = fabs(u) + alpha;
        e2 = fabs(v) + alpha;
    }

    // =========================================================================================
    // Boundary rules (source/boundary/*.f90)
    // Recursive 4/3,-1/3 extrapolation: g = c(i+1)*4.0/3.0 - c(i+2)/3.0
    static inline T extrap(T near, T far) { return near * T(4.0) / T(3.0) - far / T(3.0); }

    void extrap_left_all() {  // boundary_ivc_general.f90:101-119
        for (int v = 1; v <= 4; ++v)
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = b; i >= 1; --i) C(i, j, v) = extrap(C(i + 1, j, v), C(i + 2, j, v));
        for (int v = 1; v <= 6; ++v)
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = b; i >= 1; --i) Pm(i, j, v) = extrap(Pm(i + 1, j, v), Pm(i + 2, j, v));
    }
    void extrap_right_all() {  // boundary_ivc_general.f90:122-141
        for (int v = 1; v <= 4; ++v)
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = ni + b + 1; i <= ni + 2 * b; ++i) C(i, j, v) = extrap(C(i - 1, j, v), C(i - 2, j, v));
        for (int v = 1; v <= 6; ++v)
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = ni + b + 1; i <= ni + 2 * b; ++i) Pm(i, j, v) = extrap(Pm(i - 1, j, v), Pm(i - 2, j, v));
    }
    void extrap_top_all() {  // boundary_sedov_general.f90:46-65
        for (int v = 1; v <= 4; ++v)
            for (int j = nj + b + 1; j <= nj + 2 * b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) C(i, j, v) = extrap(C(i, j - 1, v), C(i, j - 2, v));
        for (int v = 1; v <= 6; ++v)
            for (int j = nj + b + 1; j <= nj + 2 * b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) Pm(i, j, v) = extrap(Pm(i, j - 1, v), Pm(i, j - 2, v));
    }
    void periodic_y_all() {  // boundary_ivc_general.f90:13-35
        for (int v = 1; v <= 4; ++v)
            for (int j = 1; j <= b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) {
                    C(i, j, v) = C(i, nj + j, v);
                    C(i, nj + b + j, v) = C(i, b + j, v);
                }
        for (int v = 1; v <= 6; ++v)
            for (int j = 1; j <= b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) {
                    Pm(i, j, v) = Pm(i, nj + j, v);
                    Pm(i, nj + b + j, v) = Pm(i, b + j, v);
                }
    }
    void periodic_x_all() {  // boundary_rt_general.f90:129-151 (and the commented IVC x-copy)
        for (int v = 1; v <= 4; ++v)
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = 1; i <= b; ++i) {
                    C(i, j, v) = C(ni + i, j, v);
                    C(ni + b + i, j, v) = C(b + i, j, v);
                }
        for (int v = 1; v <= 6; ++v)
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = 1; i <= b; ++i) {
                    Pm(i, j, v) = Pm(ni + i, j, v);
                    Pm(ni + b + i, j, v) = Pm(b + i, j, v);
                }
    }
    // Reflect across the bottom wall: v (index 3) negated; prim 1..5 only.
    void reflect_bottom_cell(int i, int j) {
        int s = 2 * b - j + 1;
        C(i, j, 1) = C(i, s, 1); C(i, j, 2) = C(i, s, 2); C(i, j, 3) = -C(i, s, 3); C(i, j, 4) = C(i, s, 4);
        Pm(i, j, 1) = Pm(i, s, 1); Pm(i, j, 2) = Pm(i, s, 2); Pm(i, j, 3) = -Pm(i, s, 3);
        Pm(i, j, 4) = Pm(i, s, 4); Pm(i, j, 5) = Pm(i, s, 5);
    }
    void reflect_bottom() {  // e.g. boundary_rm_general.f90:14-43
        for (int j = 1; j <= b; ++j)
            for (int i = b + 1; i <= ni + b; ++i) reflect_bottom_cell(i, j);
    }
    void reflect_top() {  // boundary_rm_general.f90:46-78
        for (int j = nj + b + 1; j <= nj + 2 * b; ++j)
            for (int i = b + 1; i <= ni + b; ++i) {
                int s = 2 * nj + 2 * b - j + 1;
                C(i, j, 1) = C(i, s, 1); C(i, j, 2) = C(i, s, 2); C(i, j, 3) = -C(i, s, 3); C(i, j, 4) = C(i, s, 4);
                Pm(i, j, 1) = Pm(i, s, 1); Pm(i, j, 2) = Pm(i, s, 2); Pm(i, j, 3) = -Pm(i, s, 3);
                Pm(i, j, 4) = Pm(i, s, 4); Pm(i, j, 5) = Pm(i, s, 5);
            }
    }
    void reflect_left() {  // boundary_sedov_general.f90:68-99 (u negated)
        for (int j = b + 1; j <= nj + b; ++j)
            for (int i = 1; i <= b; ++i) {
                int s = 2 * b - i + 1;
                C(i, j, 1) = C(s, j, 1); C(i, j, 2) = -C(s, j, 2); C(i, j, 3) = C(s, j, 3); C(i, j, 4) = C(s, j, 4);
                Pm(i, j, 1) = Pm(s, j, 1); Pm(i, j, 2) = -Pm(s, j, 2); Pm(i, j, 3) = Pm(s, j, 3);
                Pm(i, j, 4) = Pm(s, j, 4); Pm(i, j, 5) = Pm(s, j, 5);
            }
    }
    void reflect_right() {  // boundary_rt_general.f90:94-127 (commented in the reference), u negated
        for (int j = b + 1; j <= nj + b; ++j)
            for (int i = ni + b + 1; i <= ni + 2 * b; ++i) {
                int s = 2 * ni + 2 * b + 1 - i;
                C(i, j, 1) = C(s, j, 1); C(i, j, 2) = -C(s, j, 2); C(i, j, 3) = C(s, j, 3); C(i, j, 4) = C(s, j, 4);
                Pm(i, j, 1) = Pm(s, j, 1); Pm(i, j, 2) = -Pm(s, j, 2); Pm(i, j, 3) = Pm(s, j, 3);
                Pm(i, j, 4) = Pm(s, j, 4); Pm(i, j, 5) = Pm(s, j, 5);
            }
    }
    // A Dirichlet ghost state (cons 1..4, prim 1..5), e.g. boundary_rt_general.f90:23-32.
    void set_state(int i, int j, double rho, double u, double v, double p) {
        C(i, j, 1) = T(rho); C(i, j, 2) = T(rho) * T(u); C(i, j, 3) = T(rho) * T(v);
        // p/(gamma-1.d0)+0.5*rho*(u**2+v**2): 0.5 is exact in either precision
        C(i, j, 4) = T(p) / T(gamma - 1.0) + T(0.5) * T(rho) * (T(u) * T(u) + T(v) * T(v));
        Pm(i, j, 1) = T(rho); Pm(i, j, 2) = T(u); Pm(i, j, 3) = T(v); Pm(i, j, 4) = T(p);
        Pm(i, j, 5) = sqrt(T(gamma) * T(p) / T(rho));
    }

    void boundary_rt(bool reflective) {  // boundary_rt_general.f90:1-156
        for (int j = 1; j <= b; ++j)
            for (int i = b + 1; i <= ni + b; ++i) set_state(i, j, 2.0, 0.0, 0.0, 1.0);
        for (int j = nj + b + 1; j <= nj + 2 * b; ++j)
            for (int i = b + 1; i <= ni + b; ++i) set_state(i, j, 1.0, 0.0, 0.0, 2.5);
        if (reflective) {
            reflect_left();
            reflect_right();
        } else {
            periodic_x_all();
        }
        // bodyforce(:,:,3)=cons(:,:,1); bodyforce(:,:,4)=cons(:,:,3) (:154-155), whole padded array
        size_t P = (size_t)NIp * NJp;
        for (size_t k = 0; k < P; ++k) {
            bodyforce[2 * P + k] = cons[0 * P + k];
            bodyforce[3 * P + k] = cons[2 * P + k];
        }
    }

    void boundary_dmr() {  // boundary_doublemach_general.f90:1-142
        const double us = SP(8.25f) * std::sqrt(3.0) * 0.5, vs = -SP(8.25f) * 0.5;
        for (int j = 1; j <= b; ++j)
            for (int i = b + 1; i <= ni + b; ++i) {
                double xx = X(i - b, 1);
                if (xx >= 1.0 / 6.0) reflect_bottom_cell(i, j);
                else set_state(i, j, 8.0, us, vs, 116.5);
            }
        for (int j = nj + b + 1; j <= nj + 2 * b; ++j)
            for (int i = b + 1; i <= ni + b; ++i) {
                double xx = X(i - b, nj);
                if (xx < (1.0 / 6.0 + (1.0 + 20.0 * current_time) / std::sqrt(3.0)))
                    set_state(i, j, 8.0, us, vs, 116.5);
                else
                    set_state(i, j, 1.4, 0.0, 0.0, 1.0);
            }
        for (int j = b + 1; j <= nj + b; ++j)
            for (int i = 1; i <= b; ++i) set_state(i, j, 8.0, us, vs, 116.5);
        extrap_right_all();
    }

    void boundary_ssl() {  // boundary_ssl_general.f90:1-109
        reflect_bottom();
        // top boundary: loop body is empty (:47-52): ghosts keep their values
        for (int j = b + 1; j <= nj + b; ++j)
            for (int i = 1; i <= b; ++i) {
                double yy = Y(1, j - b);
                double rho, p;
                if (yy >= 0.0) { rho = 1.6374; p = 0.3327; } else { rho = 0.3626; p = 0.3327; }
                T u = T(2.5) + T(0.5) * tanh(T(2.0 * yy));
                T v = T(0.05) * cos(T(2.0 * pie * current_time / (30.0 / 2.68))) * exp(T(-(yy * yy) / 10.0))
                    + T(0.05) * cos(T(2.0 * pie * 2.0 * current_time / (30.0 / 2.68) + pie / 2.0)) * exp(T(-(yy * yy) / 10.0));
                C(i, j, 1) = T(rho); C(i, j, 2) = T(rho) * u; C(i, j, 3) = T(rho) * v;
                C(i, j, 4) = T(p) / T(gamma - 1.0) + T(0.5) * T(rho) * (u * u + v * v);
                Pm(i, j, 1) = T(rho); Pm(i, j, 2) = u; Pm(i, j, 3) = v; Pm(i, j, 4) = T(p);
                Pm(i, j, 5) = sqrt(T(gamma) * T(p) / T(rho));
            }
        extrap_right_all();
    }

    int boundary_general() {  // boundary_general.f90:1-33
        switch (cfg.benchmark) {
        case 1:  // boundary_ivc_general.f90
            periodic_y_all(); extrap_left_all(); extrap_right_all(); break;
        case 2:  // boundary_sedov_general.f90
            reflect_bottom(); extrap_top_all(); reflect_left(); extrap_right_all(); break;
        case 3: boundary_rt(false); break;
        case 4:  // boundary_rm_general.f90
            reflect_bottom(); reflect_top(); extrap_left_all(); extrap_right_all(); break;
        case 5: boundary_dmr(); break;
        case 6: boundary_ssl(); break;
        case 7: case 8: case 0: break;
        case 9:  // boundary_shockvortex_general.f90
            reflect_bottom(); reflect_top(); extrap_left_all(); extrap_right_all(); break;
        case 11: case 14: periodic_y_all(); periodic_x_all(); break;
        case 13: boundary_rt(true); break;
        default: return DENSE_ERR_BENCHMARK;
        }
        return DENSE_OK;
    }

    // =========================================================================================
    // Flux-vector splittings (source/flux_splitting/*.f90), cartesian parts
    // LF family: lam_mode 0 = local |u|+alpha (LLF), 1 = global max_eig (GLF, CH, SC)
    void split_lf_xi(int lam_mode, bool surrogate) {
        OMP_FOR
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= NIp; ++i) {
                T rho = Pm(i, j + b, 1);
                T u = Pm(i, j + b, 2), p = Pm(i, j + b, 4), alpha = Pm(i, j + b, 5);
                T lam = lam_mode == 0 ? fabs(u) + alpha : max_eig_i;
                T up = u + lam, un = u - lam, upp = u * p;
                FXP(i, j, 1) = T(0.5) * (up * C(i, j + b, 1));
                FXP(i, j, 2) = T(0.5) * (up * C(i, j + b, 2) + p);
                FXP(i, j, 3) = T(0.5) * (up * C(i, j + b, 3));
                FXP(i, j, 4) = T(0.5) * (up * C(i, j + b, 4) + upp);
                FXN(i, j, 1) = T(0.5) * (un * C(i, j + b, 1));
                FXN(i, j, 2) = T(0.5) * (un * C(i, j + b, 2) + p);
                FXN(i, j, 3) = T(0.5) * (un * C(i, j + b, 3));
                FXN(i, j, 4) = T(0.5) * (un * C(i, j + b, 4) + upp);
                if (surrogate) {  // flux_splitting_SC.f90:175-176
                    FX(i, j, 1) = rho + FXP(i, j, 2);
                    FX(i, j, 2) = rho + FXN(i, j, 2);
                }
            }
    }
    void split_lf_eta(int lam_mode, bool surrogate) {
        OMP_FOR
        for (int i = 1; i <= ni; ++i)
            for (int j = 1; j <= NJp; ++j) {
                T rho = Pm(i + b, j, 1);
                T v = Pm(i + b, j, 3), p = Pm(i + b, j, 4), alpha = Pm(i + b, j, 5);
                T lam = lam_mode == 0 ? fabs(v) + alpha : max_eig_j;
                T vp = v + lam, vn = v - lam, vpp = v * p;
                FEP(j, i, 1) = T(0.5) * (vp * C(i + b, j, 1));
                FEP(j, i, 2) = T(0.5) * (vp * C(i + b, j, 2));
                FEP(j, i, 3) = T(0.5) * (vp * C(i + b, j, 3) + p);
                FEP(j, i, 4) = T(0.5) * (vp * C(i + b, j, 4) + vpp);
                FEN(j, i, 1) = T(0.5) * (vn * C(i + b, j, 1));
                FEN(j, i, 2) = T(0.5) * (vn * C(i + b, j, 2));
                FEN(j, i, 3) = T(0.5) * (vn * C(i + b, j, 3) + p);
                FEN(j, i, 4) = T(0.5) * (vn * C(i + b, j, 4) + vpp);
                if (surrogate) {  // flux_splitting_SC.f90:206-207
                    FE(j, i, 1) = rho + FEP(j, i, 3);
                    FE(j, i, 2) = rho + FEN(j, i, 3);
                }
            }
    }

    // Steger-Warming (flux_splitting_SW.f90:14-168)
    void sw_cell(T rho, T u, T v, T alpha, bool xi, T* fp, T* fm) {
        const double epsl2 = 0.125 * 0.125;  // epsl**2, a compile-time constant
        const double g1 = gamma - 1.0, two_g1 = 2.0 * (gamma - 1.0), two_g = 2.0 * gamma;
        T uu2 = u * u + v * v;
        T un = xi ? u : v, ut = xi ? v : u;
        T l1 = un, l2 = un - alpha, l3 = un + alpha;
        T s1 = sqrt(l1 * l1 + T(epsl2)), s2 = sqrt(l2 * l2 + T(epsl2)), s3 = sqrt(l3 * l3 + T(epsl2));
        T a2 = alpha * alpha;
        T nm = un - alpha, np = un + alpha;
        T q2 = nm * nm + ut * ut, q3 = np * np + ut * ut;
        for (int sgn = 0; sgn < 2; ++sgn) {
            T lp1 = sgn == 0 ? (l1 + s1) / T(2.0) : (l1 - s1) / T(2.0);
            T lp2 = sgn == 0 ? (l2 + s2) / T(2.0) : (l2 - s2) / T(2.0);
            T lp3 = sgn == 0 ? (l3 + s3) / T(2.0) : (l3 - s3) / T(2.0);
            T* f = sgn == 0 ? fp : fm;
            T wii = T(3.0 - gamma) * (lp2 + lp3) * a2 / T(two_g1);
            T A = lp1 * T(2.0) * T(g1);
            f[0] = (A + lp2 + lp3) * rho / T(two_g);
            T fn = (A * un + lp2 * nm + lp3 * np) * rho / T(two_g);
            T ft = (A * ut + lp2 * ut + lp3 * ut) * rho / T(two_g);
            if (xi) { f[1] = fn; f[2] = ft; } else { f[1] = ft; f[2] = fn; }
            // (lambda_pm(2)*0.5d0)*((un-alpha)**2+ut**2), as associated in the reference
            f[3] = (lp1 * T(g1) * uu2 + lp2 * T(0.5) * q2 + lp3 * T(0.5) * q3 + wii) * rho / T(two_g);
        }
    }
    void split_sw() {
        in_dir(0, [&] { split_sw_xi(); });
        in_dir(1, [&] { split_sw_eta(); });
    }
    void split_sw_xi() {
        OMP_FOR
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= NIp; ++i) {
                T fp[4], fm[4];
                sw_cell(Pm(i, j + b, 1), Pm(i, j + b, 2), Pm(i, j + b, 3), Pm(i, j + b, 5), true, fp, fm);
                for (int v = 1; v <= 4; ++v) { FXP(i, j, v) = fp[v - 1]; FXN(i, j, v) = fm[v - 1]; }
            }
    }
    void split_sw_eta() {
        OMP_FOR
        for (int i = 1; i <= ni; ++i)
            for (int j = 1; j <= NJp; ++j) {
                T fp[4], fm[4];
                sw_cell(Pm(i + b, j, 1), Pm(i + b, j, 2), Pm(i + b, j, 3), Pm(i + b, j, 5), false, fp, fm);
                for (int v = 1; v <= 4; ++v) { FEP(j, i, v) = fp[v - 1]; FEN(j, i, v) = fm[v - 1]; }
            }
    }

    // =========================================================================================
    // Component-wise reconstruction (scheme_{upwind5,weno5js,weno5z}_general.f90)
    template <int R> static inline T recon(const T lf[5]) {
        if (R == 251) return upwind5(lf);
        if (R == 253) return weno5js(lf);
        return weno5z(lf);
    }
    long long dir_ops[2] = {0, 0};  // counted operations attributed to the xi / eta sweep
    long long n_smooth[2] = {0, 0}, n_char[2] = {0, 0};  // AdaWENO branch decisions per direction (interface x sign)
    template <class F> void in_dir(int d, F&& f) {
        long long t0 = ops_now();
        f();
        dir_ops[d] += ops_now() - t0;
    }
    template <int R> void recon_all() {
        in_dir(0, [&] { recon_xi<R>(); });
        in_dir(1, [&] { recon_eta<R>(); });
        in_dir(0, [&] { for (size_t k = 0; k < h_xi.size(); ++k) h_xi[k] = h_xip[k] + h_xin[k]; });
        in_dir(1, [&] { for (size_t k = 0; k < h_eta.size(); ++k) h_eta[k] = h_etap[k] + h_etan[k]; });
    }
    template <int R> void recon_xi() {
        // xi+: lf(m)=flux_xip(i+m+b-1,j,eq); xi-: lf(m)=flux_xin(i-m+b,j,eq)
        for (int v = 1; v <= 4; ++v) {
            OMP_FOR
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni + 1; ++i) {
                    T lf[5];
                    for (int m = -2; m <= 2; ++m) lf[m + 2] = FXP(i + m + b - 1, j, v);
                    HXP(i, j, v) = recon<R>(lf);
                }
            OMP_FOR
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni + 1; ++i) {
                    T lf[5];
                    for (int m = -2; m <= 2; ++m) lf[m + 2] = FXN(i - m + b, j, v);
                    HXN(i, j, v) = recon<R>(lf);
                }
        }
    }
    template <int R> void recon_eta() {
        for (int v = 1; v <= 4; ++v) {
            OMP_FOR
            for (int i = 1; i <= ni; ++i)
                for (int j = 1; j <= nj + 1; ++j) {
                    T lf[5];
                    for (int m = -2; m <= 2; ++m) lf[m + 2] = FEP(j + m + b - 1, i, v);
                    HEP(j, i, v) = recon<R>(lf);
                }
            OMP_FOR
            for (int i = 1; i <= ni; ++i)
                for (int j = 1; j <= nj + 1; ++j) {
                    T lf[5];
                    for (int m = -2; m <= 2; ++m) lf[m + 2] = FEN(j - m + b, i, v);
                    HEN(j, i, v) = recon<R>(lf);
                }
        }
    }
    void sum_fields() {  // sum_field (field_op.f90:1-21)
        in_dir(0, [&] { for (size_t k = 0; k < h_xi.size(); ++k) h_xi[k] = h_xip[k] + h_xin[k]; });
        in_dir(1, [&] { for (size_t k = 0; k < h_eta.size(); ++k) h_eta[k] = h_etap[k] + h_etan[k]; });
    }

    // =========================================================================================
    // Characteristic machinery (scheme_weno5th_CH.f90, scheme_weno5th_SC.f90)
    // Roe average of the two cells next to an interface (scheme_weno5th_CH.f90:44-62)
    inline void roe(T rhol, T rhor, T ul, T ur, T vl, T vr, T pl, T pr, T& u0, T& v0, T& h0, T& a0) {
        T hl = pl / T(gamma - 1.0) / rhol + T(0.5) * (ul * ul + vl * vl) + pl / rhol;
        T hr = pr / T(gamma - 1.0) / rhor + T(0.5) * (ur * ur + vr * vr) + pr / rhor;
        T sr = sqrt(rhor), sl = sqrt(rhol), den = sr + sl;
        u0 = (sr * ur + sl * ul) / den;
        v0 = (sr * vr + sl * vl) / den;
        h0 = (sr * hr + sl * hl) / den;
        a0 = sqrt(T(gamma - 1.0) * (h0 - T(0.5) * (u0 * u0 + v0 * v0)));
    }
    // get_l_r_vec_xi / _eta (scheme_weno5th_SC.f90:277-328, 607-658).
    // L[c][k] = l(c+1,k+1) (column k: k-th left eigenvector); R[k][e] = r(k+1,e+1).
    inline void lr_vec(bool xi, T u0, T v0, T h0, T a0, T L[4][4], T R[4][4]) {
        T uu0 = T(0.5) * (u0 * u0 + v0 * v0);
        T hh0 = a0 * a0 / T(gamma - 1.0);
        T un = xi ? u0 : v0;
        // right eigenvectors
        R[0][0] = 1.0; R[1][0] = 1.0; R[2][0] = 0.0; R[3][0] = 1.0;
        if (xi) {
            R[0][1] = u0 - a0; R[1][1] = u0; R[2][1] = 0.0; R[3][1] = u0 + a0;
            R[0][2] = v0; R[1][2] = v0; R[2][2] = 1.0; R[3][2] = v0;
            R[0][3] = h0 - a0 * u0; R[1][3] = uu0; R[2][3] = v0; R[3][3] = h0 + a0 * u0;
        } else {
            R[0][1] = u0; R[1][1] = u0; R[2][1] = 1.0; R[3][1] = u0;
            R[0][2] = v0 - a0; R[1][2] = v0; R[2][2] = 0.0; R[3][2] = v0 + a0;
            R[0][3] = h0 - a0 * v0; R[1][3] = uu0; R[2][3] = u0; R[3][3] = h0 + a0 * v0;
        }
        // left eigenvectors
        T hu = T(0.5) * uu0 / hh0, nu = T(0.5) * un / a0, ia = T(0.5) / a0;
        T pu = T(0.5) * u0 / hh0, pv = T(0.5) * v0 / hh0, ih = T(0.5) / hh0;
        if (xi) {
            L[0][0] = hu + nu; L[1][0] = -pu - ia; L[2][0] = -pv; L[3][0] = ih;
            L[0][3] = hu - nu; L[1][3] = -pu + ia; L[2][3] = -pv; L[3][3] = ih;
            L[0][2] = -v0; L[1][2] = 0.0; L[2][2] = 1.0; L[3][2] = 0.0;
        } else {
            L[0][0] = hu + nu; L[1][0] = -pu; L[2][0] = -pv - ia; L[3][0] = ih;
            L[0][3] = hu - nu; L[1][3] = -pu; L[2][3] = -pv + ia; L[3][3] = ih;
            L[0][2] = -u0; L[1][2] = 1.0; L[2][2] = 0.0; L[3][2] = 0.0;
        }
        L[0][1] = -uu0 / hh0 + T(1.0); L[1][1] = u0 / hh0; L[2][1] = v0 / hh0; L[3][1] = T(-1.0) / hh0;
    }
    // characteristic WENO-Z at one interface for one sign (CH.f90:66-81); F[m][c] stencil of F
    inline void char_weno(const T L[4][4], const T R[4][4], const T F[5][4], T h[4]) {
        T cv[4];
        for (int k = 0; k < 4; ++k) {
            T lf[5];
            for (int m = 0; m < 5; ++m)
                lf[m] = L[0][k] * F[m][0] + L[1][k] * F[m][1] + L[2][k] * F[m][2] + L[3][k] * F[m][3];
            cv[k] = weno5z(lf);
        }
        for (int e = 0; e < 4; ++e) h[e] = R[0][e] * cv[0] + R[1][e] * cv[1] + R[2][e] * cv[2] + R[3][e] * cv[3];
    }

    // sign: +1 for the "p" routines, -1 for the "n" routines; adaptive selects AdaWENO (105).
    void char_xi(int sign, bool adaptive) {
        std::vector<T>& TH = sign > 0 ? theta_xip : theta_xin;
        OMP_FOR
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni + 1; ++i) {
                auto F = [&](int cell, int v) -> T& { return sign > 0 ? FXP(cell, j, v) : FXN(cell, j, v); };
                auto cell_of = [&](int m) { return sign > 0 ? i + m + b - 1 : i - m + b; };
                T* hout[4];
                for (int v = 0; v < 4; ++v) hout[v] = sign > 0 ? &HXP(i, j, v + 1) : &HXN(i, j, v + 1);
                if (adaptive) {
                    T* th = &TH[(size_t)4 * ((size_t)(i - 1) + (size_t)(ni + 1) * (j - 1))];
                    if (th[0] > T(delta)) {  // scheme_weno5th_SC.f90:110-124
                        n_smooth[0]++;
                        T w0 = th[1], w1 = th[2], w2 = th[3];
                        for (int v = 1; v <= 4; ++v) {
                            T lf[5], q30, q31, q32;
                            for (int m = -2; m <= 2; ++m) lf[m + 2] = F(cell_of(m), v);
                            candidates(lf, q30, q31, q32);
                            *hout[v - 1] = w0 * q30 + w1 * q31 + w2 * q32;
                        }
                        continue;
                    }
                }
                if (adaptive) n_char[0]++;
                T u0, v0, h0, a0, L[4][4], R[4][4], Fs[5][4], h[4];
                roe(Pm(i + b - 1, j + b, 1), Pm(i + b, j + b, 1), Pm(i + b - 1, j + b, 2), Pm(i + b, j + b, 2),
                    Pm(i + b - 1, j + b, 3), Pm(i + b, j + b, 3), Pm(i + b - 1, j + b, 4), Pm(i + b, j + b, 4),
                    u0, v0, h0, a0);
                lr_vec(true, u0, v0, h0, a0, L, R);
                for (int m = -2; m <= 2; ++m)
                    for (int c = 0; c < 4; ++c) Fs[m + 2][c] = F(cell_of(m), c + 1);
                char_weno(L, R, Fs, h);
                for (int v = 0; v < 4; ++v) *hout[v] = h[v];
            }
    }
    void char_eta(int sign, bool adaptive) {
        std::vector<T>& TH = sign > 0 ? theta_etap : theta_etan;
        OMP_FOR
        for (int i = 1; i <= ni; ++i)
            for (int j = 1; j <= nj + 1; ++j) {
                auto F = [&](int cell, int v) -> T& { return sign > 0 ? FEP(cell, i, v) : FEN(cell, i, v); };
                auto cell_of = [&](int m) { return sign > 0 ? j + b - 1 + m : j + b - m; };
                T* hout[4];
                for (int v = 0; v < 4; ++v) hout[v] = sign > 0 ? &HEP(j, i, v + 1) : &HEN(j, i, v + 1);
                if (adaptive) {
                    T* th = &TH[(size_t)4 * ((size_t)(j - 1) + (size_t)(nj + 1) * (i - 1))];
                    if (th[0] > T(delta)) {  // scheme_weno5th_SC.f90:439-454
                        n_smooth[1]++;
                        T w0 = th[1], w1 = th[2], w2 = th[3];
                        for (int v = 1; v <= 4; ++v) {
                            T lf[5], q30, q31, q32;
                            for (int m = -2; m <= 2; ++m) lf[m + 2] = F(cell_of(m), v);
                            candidates(lf, q30, q31, q32);
                            *hout[v - 1] = w0 * q30 + w1 * q31 + w2 * q32;
                        }
                        continue;
                    }
                }
                if (adaptive) n_char[1]++;
                T u0, v0, h0, a0, L[4][4], R[4][4], Fs[5][4], h[4];
                roe(Pm(i + b, j + b - 1, 1), Pm(i + b, j + b, 1), Pm(i + b, j + b - 1, 2), Pm(i + b, j + b, 2),
                    Pm(i + b, j + b - 1, 3), Pm(i + b, j + b, 3), Pm(i + b, j + b - 1, 4), Pm(i + b, j + b, 4),
                    u0, v0, h0, a0);
                lr_vec(false, u0, v0, h0, a0, L, R);
                for (int m = -2; m <= 2; ++m)
                    for (int c = 0; c < 4; ++c) Fs[m + 2][c] = F(cell_of(m), c + 1);
                char_weno(L, R, Fs, h);
                for (int v = 0; v < 4; ++v) *hout[v] = h[v];
            }
    }
    // get_theta_* (scheme_weno5th_SC.f90:1-64, 330-393): (theta, w0, w1, w2) per interface
    void get_theta_xi(int sign) {
        std::vector<T>& TH = sign > 0 ? theta_xip : theta_xin;
        int comp = sign > 0 ? 1 : 2;
        OMP_FOR
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni + 1; ++i) {
                T lf[5];
                for (int m = -2; m <= 2; ++m) lf[m + 2] = FX(sign > 0 ? i + m + b - 1 : i - m + b, j, comp);
                T* th = &TH[(size_t)4 * ((size_t)(i - 1) + (size_t)(ni + 1) * (j - 1))];
                weno5z_omega_theta(lf, th[1], th[2], th[3], th[0]);
            }
    }
    void get_theta_eta(int sign) {
        std::vector<T>& TH = sign > 0 ? theta_etap : theta_etan;
        int comp = sign > 0 ? 1 : 2;
        OMP_FOR
        for (int i = 1; i <= ni; ++i)
            for (int j = 1; j <= nj + 1; ++j) {
                T lf[5];
                for (int m = -2; m <= 2; ++m) lf[m + 2] = FE(sign > 0 ? j + m + b - 1 : j - m + b, i, comp);
                T* th = &TH[(size_t)4 * ((size_t)(j - 1) + (size_t)(nj + 1) * (i - 1))];
                weno5z_omega_theta(lf, th[1], th[2], th[3], th[0]);
            }
    }

    // flux_splitting_general (flux_splitting.f90:1-34)
    int flux_splitting_general() {
        switch (cfg.splitting) {
        case 101: case 102: case 103:
            if (cfg.splitting == 103) split_sw();
            else {
                in_dir(0, [&] { split_lf_xi(cfg.splitting == 101 ? 0 : 1, false); });
                in_dir(1, [&] { split_lf_eta(cfg.splitting == 101 ? 0 : 1, false); });
            }
            // scheme_invis_general (scheme_invs_general.f90:1-28)
            if (cfg.recon == 251) recon_all<251>();
            else if (cfg.recon == 253) recon_all<253>();
            else if (cfg.recon == 255) recon_all<255>();
            else recon_noop = true;  // silent no-op: h_xi/h_eta keep their values
            return DENSE_OK;
        case 104:  // flux_splitting_CH_block (flux_splitting_CH.f90:24-110)
            in_dir(0, [&] { split_lf_xi(1, false); char_xi(+1, false); char_xi(-1, false); });
            in_dir(1, [&] { split_lf_eta(1, false); char_eta(+1, false); char_eta(-1, false); });
            sum_fields();
            return DENSE_OK;
        case 105:  // flux_splitting_SC_block (flux_splitting_SC.f90:141-237)
            in_dir(0, [&] {
                split_lf_xi(1, true);
                get_theta_xi(+1); char_xi(+1, true);
                get_theta_xi(-1); char_xi(-1, true);
            });
            in_dir(1, [&] {
                split_lf_eta(1, true);
                get_theta_eta(+1); char_eta(+1, true);
                get_theta_eta(-1); char_eta(-1, true);
            });
            sum_fields();
            return DENSE_OK;
        default:
            return DENSE_ERR_SPLITTING;
        }
    }

    // =========================================================================================
    // time_rk3_general (source/time_advance/time_advance_general.f90:1-269)
    void time_rk3(int irk) {
        const double dxi = dx, deta = dy;
        if (irk == 1) {
            if (!cfg.if_const_dt) {
                double dt_xi = dx / val(max_eig_i);
                double dt_eta = dy / val(max_eig_j);
                dt = cfl * dt_xi * dt_eta / (dt_xi + dt_eta);
            }
            cons_temp = cons;  // copy_field over the whole padded array (:26-33)
        }
        const double dtdx = dt / dxi, dtdy = dt / deta;
        for (int v = 1; v <= 4; ++v) {
            OMP_FOR
            for (int j = b + 1; j <= nj + b; ++j)
                for (int i = b + 1; i <= ni + b; ++i) {
                    T dh_dxi = HX(i - b + 1, j - b, v) - HX(i - b, j - b, v);
                    T dh_deta = HE(j - b + 1, i - b, v) - HE(j - b, i - b, v);
                    T q;
                    if (irk == 1) {
                        T q0 = C(i, j, v);
                        q = q0 - T(dtdx) * dh_dxi - T(dtdy) * dh_deta;
                    } else if (irk == 2) {
                        T q0 = CT(i, j, v), q1 = C(i, j, v);
                        q = T(3.0 / 4.0) * q0 + T(1.0 / 4.0) * q1 - T(1.0 / 4.0) * (T(dtdx) * dh_dxi + T(dtdy) * dh_deta);
                    } else {
                        T q0 = CT(i, j, v), q1 = C(i, j, v);
                        q = T(1.0 / 3.0) * q0 + T(2.0 / 3.0) * q1 - T(2.0 / 3.0) * (T(dtdx) * dh_dxi + T(dtdy) * dh_deta);
                    }
                    C(i, j, v) = q;
                }
        }
        // source and viscous terms: their arrays are never filled in the reference, so they add 0
        if (cfg.if_bodyforce && bodyforce_alloc) {  // :71-84, :152-165, :234-247
            double f = irk == 1 ? dt : (irk == 2 ? 1.0 / 4.0 * dt : SP(2.0f / 3.0f) * dt);
            for (int v = 1; v <= 4; ++v) {
                OMP_FOR
                for (int j = b + 1; j <= nj + b; ++j)
                    for (int i = b + 1; i <= ni + b; ++i) C(i, j, v) = C(i, j, v) + T(f) * BF(i, j, v);
            }
        }
    }

    // general_main.f90:26-31. phase_ops[k] receives the operation count of each phase when
    // counting (k = 0 get_primary, 1 boundary_general, 2 flux_splitting_general, 3 time_rk3).
    long long phase_ops[4] = {0, 0, 0, 0};
    int stage(int irk) {
        long long t0 = ops_now();
        get_primary();
        long long t1 = ops_now();
        int rc = boundary_general();
        if (rc) return rc;
        long long t2 = ops_now();
        rc = flux_splitting_general();
        if (rc) return rc;
        long long t3 = ops_now();
        time_rk3(irk);
        long long t4 = ops_now();
        phase_ops[0] += t1 - t0; phase_ops[1] += t2 - t1; phase_ops[2] += t3 - t2; phase_ops[3] += t4 - t3;
        return DENSE_OK;
    }
    // general_main.f90:23-38, without the save block
    int steps(int nsteps, double t_end, int total_step) {
        for (int s = 0; s < nsteps; ++s) {
            if (!(current_time < t_end && current_step < total_step)) break;
            for (int irk = 1; irk <= cfg.stages; ++irk) {
                int rc = stage(irk);
                if (rc) return rc;
            }
            current_step += 1;
            current_time = current_time + dt;
            elasp_time = elasp_time + dt;
        }
        return DENSE_OK;
    }

    // =========================================================================================
    // Initial setups (source/initial/*.f90). They fill the interior of cons and prim.
    void set_interior(int i, int j, double rho, double u, double v, double p) {
        int I = i + b, J = j + b;
        C(I, J, 1) = T(rho); C(I, J, 2) = T(rho * u); C(I, J, 3) = T(rho * v);
        C(I, J, 4) = T(p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v));
        Pm(I, J, 1) = T(rho); Pm(I, J, 2) = T(u); Pm(I, J, 3) = T(v); Pm(I, J, 4) = T(p);
        Pm(I, J, 5) = T(std::sqrt(gamma * p / rho));
    }
    void cell_centres(double xl, double yl, double yshift) {
        dx = xl / ni; dy = yl / nj;
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                X(i, j) = (i - 0.5) * dx;
                Y(i, j) = (j - 0.5) * dy - yshift;
            }
    }
    int init_general() {
        switch (cfg.benchmark) {
        case 1: {  // init_IVC_general.f90:1-58
            double bb = 0.5;
            cell_centres(10.0, 10.0, 0.0);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    double r = std::sqrt((X(i, j) - 5.0) * (X(i, j) - 5.0) + (Y(i, j) - 5.0) * (Y(i, j) - 5.0));
                    double rho = std::pow(1.0 - (gamma - 1.0) * (bb * bb) * std::exp(1.0 - r * r) / (8.0 * gamma * (pie * pie)), 2.5);
                    double u = 0.0 - bb / (2.0 * pie) * std::exp((1.0 - r * r) / 2.0) * (Y(i, j) - 5.0);
                    double v = bb / (2.0 * pie) * std::exp((1.0 - r * r) / 2.0) * (X(i, j) - 5.0);
                    double p = std::pow(rho, gamma);
                    set_interior(i, j, rho, u, v, p);
                }
            break;
        }
        case 11: {  // periodic translating vortex (the IVC test with a freestream, periodic in x and y)
            double eps = cfg.var_eps, xc = cfg.var_xc, yc = cfg.var_yc;
            cell_centres(10.0, 10.0, 0.0);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    double r = std::sqrt((X(i, j) - xc) * (X(i, j) - xc) + (Y(i, j) - yc) * (Y(i, j) - yc));
                    double rho = std::pow(1.0 - (gamma - 1.0) * (eps * eps) * std::exp(1.0 - r * r) / (8.0 * gamma * (pie * pie)), 1.0 / (gamma - 1.0));
                    double u = 1.0 - eps / (2.0 * pie) * std::exp((1.0 - r * r) / 2.0) * (Y(i, j) - yc);
                    double v = 1.0 + eps / (2.0 * pie) * std::exp((1.0 - r * r) / 2.0) * (X(i, j) - xc);
                    double p = std::pow(rho, gamma);
                    set_interior(i, j, rho, u, v, p);
                }
            break;
        }
        case 2: {  // init_sedov_general.f90:1-69
            cell_centres(1.2, 1.2, 0.0);
            double e = 0.244816 / (dx * dy);
            double p0 = e * (gamma - 1.0), p1 = SP(1.0e-6f);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) set_interior(i, j, 1.0, 0.0, 0.0, p1);
            set_interior(1, 1, 1.0, 0.0, 0.0, p0);
            break;
        }
        case 3: case 13: {  // init_RT_general.f90:1-67
            cfg.if_bodyforce = 1; bodyforce_alloc = true;
            gamma = 5.0 / 3.0; cfg.gamma = gamma;
            dx = 0.25 / (ni - 1.0); dy = 1.0 / (nj - 1.0);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) { X(i, j) = (i - 1.0) * dx; Y(i, j) = (j - 1.0) * dy; }
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    double rho, p, u = 0.0, c, v;
                    if (Y(i, j) <= 0.5) {
                        rho = 2.0; p = 2.0 * Y(i, j) + 1.0; c = std::sqrt(gamma * p / rho);
                        v = -0.025 * c * std::cos(8.0 * pie * X(i, j));
                    } else {
                        rho = 1.0; p = Y(i, j) + 1.5; c = std::sqrt(gamma * p / rho);
                        v = -SP(0.025f) * c * std::cos(8.0 * pie * X(i, j));
                    }
                    set_interior(i, j, rho, u, v, p);
                    BF(i + b, j + b, 3) = T(rho); BF(i + b, j + b, 4) = T(rho * v);
                }
            break;
        }
        case 4: {  // init_RM_general.f90:1-66
            cell_centres(4.0, 1.0, 0.0);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    double xx = X(i, j), yy = Y(i, j), rho, u, v, p;
                    if (xx < SP(0.05f)) { rho = SP(1.376364f); u = SP(0.394729f); v = 0.0; p = SP(1.569800f); }
                    else if (xx < (1.0 - SP(0.05f) * std::sin(2.0 * pie * (yy - 0.25))) && xx > SP(0.05f)) { rho = 1.0; u = 0.0; v = 0.0; p = 1.0; }
                    else { rho = SP(0.1358f); u = 0.0; v = 0.0; p = 1.0; }
                    set_interior(i, j, rho, u, v, p);
                }
            break;
        }
        case 14: {  // periodic Richtmyer-Meshkov variant on [0,1]^2
            cell_centres(1.0, 1.0, 0.0);
            const double M = 1.2, g = gamma;
            double rho2 = (g + 1.0) * M * M / ((g - 1.0) * M * M + 2.0);
            double p2 = 1.0 + 2.0 * g / (g + 1.0) * (M * M - 1.0);
            double u2 = M * std::sqrt(g) * (1.0 - 1.0 / rho2);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    double xx = X(i, j), yy = Y(i, j);
                    double xi_if = 0.5 + cfg.var_amp * std::cos(2.0 * pie * yy);
                    if (xx < 0.2) set_interior(i, j, rho2, u2, 0.0, p2);
                    else if (xx < xi_if) set_interior(i, j, 1.0, 0.0, 0.0, 1.0);
                    else set_interior(i, j, 3.0, 0.0, 0.0, 1.0);
                }
            break;
        }
        case 5: {  // init_doublemach_general.f90:1-61
            cell_centres(4.0, 1.0, 0.0);
            const double us = SP(8.25f) * std::sqrt(3.0) * 0.5, vs = -SP(8.25f) * 0.5;
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    if (X(i, j) < (1.0 / 6.0 + Y(i, j) * std::sqrt(1.0 / 3.0))) set_interior(i, j, 8.0, us, vs, 116.5);
                    else set_interior(i, j, 1.4, 0.0, 0.0, 1.0);
                }
            break;
        }
        case 6: {  // init_ssl_general.f90:1-82
            cell_centres(200.0, 40.0, 40.0 / 2.0);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    if (Y(i, j) >= 0) set_interior(i, j, 1.6374, 3.0, 0.0, 0.3327);
                    else set_interior(i, j, 0.3626, 2.0, 0.0, 0.3327);
                }
            // rows nj..nj+b (interior top row and the top ghost rows) get the post-shock state
            for (int j = nj; j <= nj + b; ++j)
                for (int i = 1; i <= ni; ++i) set_interior(i, j, 2.1101, 2.9709, -0.1367, SP(0.4754f));
            break;
        }
        case 9: {  // init_shockvortex_general.f90:1-67
            const double x_c = SP(0.25f), y_c = SP(0.5f), epsl = SP(0.3f), r_c = SP(0.05f), alpha = SP(0.204f);
            cell_centres(2.0, 1.0, 0.0);
            for (int j = 1; j <= nj; ++j)
                for (int i = 1; i <= ni; ++i) {
                    double xx = X(i, j), yy = Y(i, j);
                    double r = std::sqrt((xx - x_c) * (xx - x_c) + (yy - y_c) * (yy - y_c));
                    double tau = r / r_c;
                    double rho, u, v, p;
                    if (xx < 0.5) {
                        rho = std::pow(1.0 - (gamma - 1.0) * (epsl * epsl) * std::exp(2.0 * alpha * (1.0 - tau * tau)) / (4.0 * alpha * gamma), 1.0 / (gamma - 1.0));
                        u = SP(1.1f) * std::sqrt(gamma) + epsl * tau * std::exp(alpha * (1.0 - tau * tau)) * (yy - y_c) / r;
                        v = -(epsl * tau * std::exp(alpha * (1.0 - tau * tau)) * (xx - x_c) / r);
                        p = std::pow(rho, gamma);
                    } else { rho = 1.169082; u = 1.113299; v = 0.0; p = 1.245000; }
                    set_interior(i, j, rho, u, v, p);
                }
            break;
        }
        case 0: case 7: case 8: break;
        default: return DENSE_ERR_BENCHMARK;
        }
        cfg.dx = dx; cfg.dy = dy;
        return DENSE_OK;
    }
};

}  // namespace oracle

// =============================================================================================
// C interface for the tests (ctypes)
using oracle::Solver;
using oracle::Counted;

extern "C" {

void* oracle_create(const dense_config_t* cfg) { return new Solver<double>(*cfg); }
void oracle_destroy(void* h) { delete (Solver<double>*)h; }

// init_general; returns the config as the setup left it (dx, dy, gamma, if_bodyforce).
int oracle_init(void* h, dense_config_t* cfg_out) {
    auto* s = (Solver<double>*)h;
    int rc = s->init_general();
    if (cfg_out) *cfg_out = s->cfg;
    return rc;
}
void oracle_set_config(void* h, const dense_config_t* cfg) {
    auto* s = (Solver<double>*)h;
    s->cfg = *cfg; s->gamma = cfg->gamma; s->cfl = cfg->cfl; s->delta = cfg->delta;
    s->dx = cfg->dx; s->dy = cfg->dy;
    if (cfg->if_bodyforce) s->bodyforce_alloc = true;
}
void oracle_get_state(void* h, double* cons, double* prim) {
    auto* s = (Solver<double>*)h;
    if (cons) std::memcpy(cons, s->cons.data(), s->cons.size() * sizeof(double));
    if (prim) std::memcpy(prim, s->prim.data(), s->prim.size() * sizeof(double));
}
void oracle_set_state(void* h, const double* cons, const double* prim) {
    auto* s = (Solver<double>*)h;
    if (cons) std::memcpy(s->cons.data(), cons, s->cons.size() * sizeof(double));
    if (prim) std::memcpy(s->prim.data(), prim, s->prim.size() * sizeof(double));
}
void oracle_get_grid(void* h, double* x, double* y) {
    auto* s = (Solver<double>*)h;
    if (x) std::memcpy(x, s->x.data(), s->x.size() * sizeof(double));
    if (y) std::memcpy(y, s->y.data(), s->y.size() * sizeof(double));
}
void oracle_get_bodyforce(void* h, double* bf) {
    auto* s = (Solver<double>*)h;
    std::memcpy(bf, s->bodyforce.data(), s->bodyforce.size() * sizeof(double));
}
void oracle_set_bodyforce(void* h, const double* bf) {
    auto* s = (Solver<double>*)h;
    std::memcpy(s->bodyforce.data(), bf, s->bodyforce.size() * sizeof(double));
}
void oracle_get_fluxes(void* h, double* hxi, double* heta) {
    auto* s = (Solver<double>*)h;
    if (hxi) std::memcpy(hxi, s->h_xi.data(), s->h_xi.size() * sizeof(double));
    if (heta) std::memcpy(heta, s->h_eta.data(), s->h_eta.size() * sizeof(double));
}
void oracle_get_theta(void* h, double* txp, double* txn, double* tep, double* ten) {
    auto* s = (Solver<double>*)h;
    if (txp) std::memcpy(txp, s->theta_xip.data(), s->theta_xip.size() * sizeof(double));
    if (txn) std::memcpy(txn, s->theta_xin.data(), s->theta_xin.size() * sizeof(double));
    if (tep) std::memcpy(tep, s->theta_etap.data(), s->theta_etap.size() * sizeof(double));
    if (ten) std::memcpy(ten, s->theta_etan.data(), s->theta_etan.size() * sizeof(double));
}
// scalars: [dt, max_eig_i, max_eig_j, current_time, elasp_time, current_step, recon_noop]
void oracle_get_scalars(void* h, double* out) {
    auto* s = (Solver<double>*)h;
    out[0] = s->dt; out[1] = s->max_eig_i; out[2] = s->max_eig_j; out[3] = s->current_time;
    out[4] = s->elasp_time; out[5] = s->current_step; out[6] = s->recon_noop ? 1.0 : 0.0;
}
void oracle_set_time(void* h, double t, int step, double dt) {
    auto* s = (Solver<double>*)h;
    s->current_time = t; s->current_step = step; s->dt = dt;
}
int oracle_get_primary(void* h) { ((Solver<double>*)h)->get_primary(); return 0; }
int oracle_boundary(void* h) { return ((Solver<double>*)h)->boundary_general(); }
int oracle_flux(void* h) { return ((Solver<double>*)h)->flux_splitting_general(); }
int oracle_time_rk3(void* h, int irk) { ((Solver<double>*)h)->time_rk3(irk); return 0; }
int oracle_stage(void* h, int irk) { return ((Solver<double>*)h)->stage(irk); }
int oracle_steps(void* h, int nsteps, double t_end, int total_step) {
    return ((Solver<double>*)h)->steps(nsteps, t_end, total_step);
}
int oracle_threads(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}
// Threads of the following OpenMP regions (the CPU baseline is timed at 1 thread and at all).
void oracle_set_threads(int n) {
#if defined(_OPENMP)
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// Count the floating-point operations of one full step (all stages) on field values, starting
// from the given padded state (or the benchmark's setup when cons is NULL).
// out: [add, mul, div, sqrt, transcendental, interior cells,
//       get_primary, boundary_general, flux_splitting_general, time_rk3 (add+mul+div+sqrt each),
//       flux xi sweep, flux eta sweep]
int oracle_count_step(const dense_config_t* cfg, const double* cons, long long* out) {
    Solver<Counted> s(*cfg);
    if (cons) {
        for (size_t k = 0; k < s.cons.size(); ++k) s.cons[k] = Counted(cons[k]);
    } else {
        int rc = s.init_general();
        if (rc) return rc;
    }
    if (s.cfg.benchmark == 3 || s.cfg.benchmark == 13) s.bodyforce_alloc = true;
    oracle::g_ops = oracle::OpCount();
    for (int irk = 1; irk <= s.cfg.stages; ++irk) {
        int rc = s.stage(irk);
        if (rc) return rc;
    }
    out[0] = oracle::g_ops.add; out[1] = oracle::g_ops.mul; out[2] = oracle::g_ops.div;
    out[3] = oracle::g_ops.sqrt; out[4] = oracle::g_ops.transc; out[5] = (long long)s.ni * s.nj;
    for (int k = 0; k < 4; ++k) out[6 + k] = s.phase_ops[k];
    out[10] = s.dir_ops[0];
    out[11] = s.dir_ops[1];
    out[12] = s.n_smooth[0]; out[14] = s.n_smooth[1];
    out[13] = s.n_char[0]; out[15] = s.n_char[1];
    return 0;
}

// Operations of one AdaWENO branch at one interface and sign, the same for any data:
// out[0] = the smooth branch (component-wise with the surrogate's weights, SC.f90:110-124),
// out[1] = the characteristic branch (Roe average, eigenvectors, projection, 4 WENO-Z, back-
// projection; SC.f90:126-163, the same work as one sign of scheme 104).
int oracle_branch_costs(double gamma, long long* out) {
    dense_config_t c;
    std::memset(&c, 0, sizeof(c));
    c.ni = 3; c.nj = 3; c.gamma = gamma;
    Solver<Counted> s(c);
    Counted F[5][4], L[4][4], R[4][4], h[4], u0, v0, h0, a0;
    for (int m = 0; m < 5; ++m)
        for (int k = 0; k < 4; ++k) F[m][k] = Counted(1.0 + 0.1 * m + 0.01 * k * m * m);
    oracle::g_ops = oracle::OpCount();
    for (int v = 0; v < 4; ++v) {
        Counted lf[5], q30, q31, q32, w0 = 0.2, w1 = 0.5, w2 = 0.3;
        for (int m = 0; m < 5; ++m) lf[m] = F[m][v];
        oracle::candidates(lf, q30, q31, q32);
        h[v] = w0 * q30 + w1 * q31 + w2 * q32;
    }
    out[0] = Solver<Counted>::ops_now();
    oracle::g_ops = oracle::OpCount();
    s.roe(Counted(1.0), Counted(1.2), Counted(0.1), Counted(0.2), Counted(0.0), Counted(0.1),
          Counted(1.0), Counted(1.1), u0, v0, h0, a0);
    s.lr_vec(true, u0, v0, h0, a0, L, R);
    s.char_weno(L, R, F, h);
    out[1] = Solver<Counted>::ops_now();
    return 0;
}

// Known-answer hooks: one reconstruction of a 5-point stencil. kind 251/253/255 returns h in
// out[0]; kind 1 returns WENO-JS weights (w0,w1,w2), kind 2 WENO-Z (w0,w1,w2,theta).
int oracle_recon(int kind, const double* lf, double* out) {
    double a0, a1, a2;
    switch (kind) {
    case 251: out[0] = oracle::upwind5(lf); return 0;
    case 253: out[0] = oracle::weno5js(lf); return 0;
    case 255: out[0] = oracle::weno5z(lf); return 0;
    case 1: {
        oracle::weno5js_alpha(lf, a0, a1, a2);
        double s = a0 + a1 + a2;
        out[0] = a0 / s; out[1] = a1 / s; out[2] = a2 / s;
        return 0;
    }
    case 2: oracle::weno5z_omega_theta(lf, out[0], out[1], out[2], out[3]); return 0;
    default: return 1;
    }
}

// Roe average of two states and the left/right eigenvector matrices of get_l_r_vec_xi/_eta.
// L[c*4+k] = l(c+1,k+1), R[k*4+e] = r(k+1,e+1); roe_out = (u0, v0, h0, alpha0).
int oracle_roe_lr(int dir, double gamma, const double* left, const double* right, double* roe_out,
                  double* L, double* R) {
    dense_config_t c;
    std::memset(&c, 0, sizeof(c));
    c.ni = 3; c.nj = 3; c.gamma = gamma;
    Solver<double> s(c);
    double u0, v0, h0, a0, Lm[4][4], Rm[4][4];
    s.roe(left[0], right[0], left[1], right[1], left[2], right[2], left[3], right[3], u0, v0, h0, a0);
    s.lr_vec(dir == 0, u0, v0, h0, a0, Lm, Rm);
    roe_out[0] = u0; roe_out[1] = v0; roe_out[2] = h0; roe_out[3] = a0;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) { L[a * 4 + b] = Lm[a][b]; R[a * 4 + b] = Rm[a][b]; }
    return 0;
}

}  // extern "C"
