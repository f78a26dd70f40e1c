// host_setup.cpp — the host-side, one-time parts of the C ABI: module defaults, the input.in
// namelist reader and the benchmark initial setups.
//
// Built with -ffp-contract=off so the setups round exactly as the reference's gfortran -O2
// build does on x86-64 (no FMA); the initial state is then bit-identical to the reference's and
// the device starts from the same bits. Default-real (single precision) literals of the Fortran
// are written as (double)<float literal>.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dense2d.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

inline double SP(float f) { return (double)f; }
const double kPi = 3.141592653589793115997963468544185161590576171875;  // atan(1.d0)*4.d0

// ---------------------------------------------------------------------------------------------
// Fortran-layout views of the caller's arrays (1-based, column-major)
struct Views {
    int ni, nj, NIp, NJp;
    double *cons, *prim, *x, *y;
    double& C(int i, int j, int v) const { return cons[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)NJp * (v - 1))]; }
    double& Q(int i, int j, int v) const { return prim[(size_t)(i - 1) + (size_t)NIp * ((size_t)(j - 1) + (size_t)NJp * (v - 1))]; }
    double& X(int i, int j) const { return x[(size_t)(i - 1) + (size_t)ni * (j - 1)]; }
    double& Y(int i, int j) const { return y[(size_t)(i - 1) + (size_t)ni * (j - 1)]; }
};

// The per-cell assignment block shared by every init_*_general.f90 (e.g. init_IVC_general.f90:82-91):
// cons = (rho, rho u, rho v, p/(gamma-1)+0.5 rho (u^2+v^2)), prim = (rho, u, v, p, sqrt(gamma p/rho)).
void put(const Views& w, double gamma, int i, int j, double rho, double u, double v, double p) {
    const int I = i + 4, J = j + 4;
    w.C(I, J, 1) = rho;
    w.C(I, J, 2) = rho * u;
    w.C(I, J, 3) = rho * v;
    w.C(I, J, 4) = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
    w.Q(I, J, 1) = rho;
    w.Q(I, J, 2) = u;
    w.Q(I, J, 3) = v;
    w.Q(I, J, 4) = p;
    w.Q(I, J, 5) = std::sqrt(gamma * p / rho);
}

void centres(const Views& w, double dx, double dy, double yshift) {
    for (int j = 1; j <= w.nj; ++j)
        for (int i = 1; i <= w.ni; ++i) {
            w.X(i, j) = (i - 0.5) * dx;
            w.Y(i, j) = (j - 0.5) * dy - yshift;
        }
}

// Isentropic vortex of strength eps centred at (xc, yc) over a uniform stream (us, vs); the
// density exponent is 2.5 in the reference setup and 1/(gamma-1) in the translating variant.
void vortex(const Views& w, double gamma, double eps, double xc, double yc, double us, double vs,
            double expo) {
    for (int j = 1; j <= w.nj; ++j)
        for (int i = 1; i <= w.ni; ++i) {
            const double xx = w.X(i, j), yy = w.Y(i, j);
            const double r = std::sqrt((xx - xc) * (xx - xc) + (yy - yc) * (yy - yc));
            const double rho = std::pow(1.0 - (gamma - 1.0) * (eps * eps) * std::exp(1.0 - r * r) /
                                                  (8.0 * gamma * (kPi * kPi)), expo);
            const double u = us - eps / (2.0 * kPi) * std::exp((1.0 - r * r) / 2.0) * (yy - yc);
            const double v = vs + eps / (2.0 * kPi) * std::exp((1.0 - r * r) / 2.0) * (xx - xc);
            put(w, gamma, i, j, rho, u, v, std::pow(rho, gamma));
        }
}

int setup(dense_config_t* cfg, const Views& w) {
    double gamma = cfg->gamma;
    const int ni = w.ni, nj = w.nj;
    double dx = 0.0, dy = 0.0;
    switch (cfg->benchmark) {
    case DENSE_BENCH_USER: case 7: case 8:  // init_general.f90:26-33: nothing is initialised
        return DENSE_OK;
    case DENSE_BENCH_IVC:  // init_IVC_general.f90:1-58 (b = 0.5, no freestream)
        dx = 10.0 / ni; dy = 10.0 / nj;
        centres(w, dx, dy, 0.0);
        vortex(w, gamma, 0.5, 5.0, 5.0, 0.0, 0.0, 2.5);
        break;
    case DENSE_BENCH_IVC_PERIODIC:  // translating vortex over (1,1,1,1)
        dx = 10.0 / ni; dy = 10.0 / nj;
        centres(w, dx, dy, 0.0);
        vortex(w, gamma, cfg->var_eps, cfg->var_xc, cfg->var_yc, 1.0, 1.0, 1.0 / (gamma - 1.0));
        break;
    case DENSE_BENCH_SEDOV: {  // init_sedov_general.f90:1-69
        dx = 1.2 / ni; dy = 1.2 / nj;
        centres(w, dx, dy, 0.0);
        const double e = 0.244816 / (dx * dy);
        const double p0 = e * (gamma - 1.0), p1 = SP(1.0e-6f);
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) put(w, gamma, i, j, 1.0, 0.0, 0.0, p1);
        put(w, gamma, 1, 1, 1.0, 0.0, 0.0, p0);
        break;
    }
    case DENSE_BENCH_RT: case DENSE_BENCH_RT_REFLECT:  // init_RT_general.f90:1-67
        cfg->if_bodyforce = 1;
        gamma = 5.0 / 3.0;
        cfg->gamma = gamma;
        dx = 0.25 / (ni - 1.0); dy = 1.0 / (nj - 1.0);
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) { w.X(i, j) = (i - 1.0) * dx; w.Y(i, j) = (j - 1.0) * dy; }
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const double yy = w.Y(i, j), xx = w.X(i, j);
                double rho, p, c, v;
                if (yy <= 0.5) {
                    rho = 2.0; p = 2.0 * yy + 1.0; c = std::sqrt(gamma * p / rho);
                    v = -0.025 * c * std::cos(8.0 * kPi * xx);
                } else {  // the upper half uses a default-real 0.025 (:47)
                    rho = 1.0; p = yy + 1.5; c = std::sqrt(gamma * p / rho);
                    v = -SP(0.025f) * c * std::cos(8.0 * kPi * xx);
                }
                put(w, gamma, i, j, rho, 0.0, v, p);
            }
        break;
    case DENSE_BENCH_RM:  // init_RM_general.f90:1-66
        dx = 4.0 / ni; dy = 1.0 / nj;
        centres(w, dx, dy, 0.0);
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const double xx = w.X(i, j), yy = w.Y(i, j);
                if (xx < SP(0.05f))
                    put(w, gamma, i, j, SP(1.376364f), SP(0.394729f), 0.0, SP(1.569800f));
                else if (xx < (1.0 - SP(0.05f) * std::sin(2.0 * kPi * (yy - 0.25))) && xx > SP(0.05f))
                    put(w, gamma, i, j, 1.0, 0.0, 0.0, 1.0);
                else
                    put(w, gamma, i, j, SP(0.1358f), 0.0, 0.0, 1.0);
            }
        break;
    case DENSE_BENCH_RM_PERIODIC: {  // Mach 1.2 shock into a density-3 interface on [0,1]^2
        dx = 1.0 / ni; dy = 1.0 / nj;
        centres(w, dx, dy, 0.0);
        const double M = 1.2, g = gamma;
        const double rho2 = (g + 1.0) * M * M / ((g - 1.0) * M * M + 2.0);
        const double p2 = 1.0 + 2.0 * g / (g + 1.0) * (M * M - 1.0);
        const double u2 = M * std::sqrt(g) * (1.0 - 1.0 / rho2);
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const double xx = w.X(i, j), yy = w.Y(i, j);
                const double xi_if = 0.5 + cfg->var_amp * std::cos(2.0 * kPi * yy);
                if (xx < 0.2) put(w, gamma, i, j, rho2, u2, 0.0, p2);
                else if (xx < xi_if) put(w, gamma, i, j, 1.0, 0.0, 0.0, 1.0);
                else put(w, gamma, i, j, 3.0, 0.0, 0.0, 1.0);
            }
        break;
    }
    case DENSE_BENCH_DMR: {  // init_doublemach_general.f90:1-61
        dx = 4.0 / ni; dy = 1.0 / nj;
        centres(w, dx, dy, 0.0);
        const double us = SP(8.25f) * std::sqrt(3.0) * 0.5, vs = -SP(8.25f) * 0.5;
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                if (w.X(i, j) < (1.0 / 6.0 + w.Y(i, j) * std::sqrt(1.0 / 3.0)))
                    put(w, gamma, i, j, 8.0, us, vs, 116.5);
                else
                    put(w, gamma, i, j, 1.4, 0.0, 0.0, 1.0);
            }
        break;
    }
    case DENSE_BENCH_SSL:  // init_ssl_general.f90:1-82
        dx = 200.0 / ni; dy = 40.0 / nj;
        centres(w, dx, dy, 40.0 / 2.0);
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                if (w.Y(i, j) >= 0) put(w, gamma, i, j, 1.6374, 3.0, 0.0, 0.3327);
                else put(w, gamma, i, j, 0.3626, 2.0, 0.0, 0.3327);
            }
        // the top interior row and the four top ghost rows hold the post-shock state (:197-216)
        for (int j = nj; j <= nj + 4; ++j)
            for (int i = 1; i <= ni; ++i) put(w, gamma, i, j, 2.1101, 2.9709, -0.1367, SP(0.4754f));
        break;
    case DENSE_BENCH_SHOCKVORTEX: {  // init_shockvortex_general.f90:1-67
        const double x_c = SP(0.25f), y_c = SP(0.5f), epsl = SP(0.3f), r_c = SP(0.05f), alpha = SP(0.204f);
        dx = 2.0 / ni; dy = 1.0 / nj;
        centres(w, dx, dy, 0.0);
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i) {
                const double xx = w.X(i, j), yy = w.Y(i, j);
                const double r = std::sqrt((xx - x_c) * (xx - x_c) + (yy - y_c) * (yy - y_c));
                const double tau = r / r_c;
                if (xx < 0.5) {
                    const double rho = std::pow(1.0 - (gamma - 1.0) * (epsl * epsl) *
                                                          std::exp(2.0 * alpha * (1.0 - tau * tau)) /
                                                          (4.0 * alpha * gamma), 1.0 / (gamma - 1.0));
                    const double u = SP(1.1f) * std::sqrt(gamma) +
                                     epsl * tau * std::exp(alpha * (1.0 - tau * tau)) * (yy - y_c) / r;
                    const double v = -(epsl * tau * std::exp(alpha * (1.0 - tau * tau)) * (xx - x_c) / r);
                    put(w, gamma, i, j, rho, u, v, std::pow(rho, gamma));
                } else {
                    put(w, gamma, i, j, 1.169082, 1.113299, 0.0, 1.245000);
                }
            }
        break;
    }
    default:
        return fail(DENSE_ERR_BENCHMARK, "No such Benchmark index! (init_general.f90:34-36)");
    }
    cfg->dx = dx;
    cfg->dy = dy;
    return DENSE_OK;
}

// ---------------------------------------------------------------------------------------------
// Namelist reader
std::string lower(std::string s) {
    for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}
std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}
bool parse_logical(const std::string& v0, int* out) {
    std::string v = lower(trim(v0));
    if (!v.empty() && v[0] == '.') v = v.substr(1);
    if (v.empty()) return false;
    if (v[0] == 't') { *out = 1; return true; }
    if (v[0] == 'f') { *out = 0; return true; }
    return false;
}
bool parse_real(const std::string& v0, double* out) {
    std::string v = trim(v0);
    for (auto& ch : v) if (ch == 'd' || ch == 'D') ch = 'e';
    if (v.empty()) return false;
    char* end = nullptr;
    double d = std::strtod(v.c_str(), &end);
    if (end == v.c_str() || trim(std::string(end)).size()) return false;
    *out = d;
    return true;
}
bool parse_int(const std::string& v0, int* out) {
    std::string v = trim(v0);
    if (v.empty()) return false;
    char* end = nullptr;
    long x = std::strtol(v.c_str(), &end, 10);
    if (end == v.c_str() || trim(std::string(end)).size()) return false;
    *out = (int)x;
    return true;
}

enum Kind { kInt, kReal, kLogical };
struct Entry { Kind kind; size_t offset; };

const std::map<std::string, std::map<std::string, Entry>>& groups() {
#define E(kind, field) Entry{kind, offsetof(dense_config_t, field)}
    static const std::map<std::string, std::map<std::string, Entry>> g = {
        {"omp_pars", {{"omp_thread_num", E(kInt, omp_thread_num)}}},
        {"model_pars", {{"neq", E(kInt, neq)}, {"if_source", E(kLogical, if_source)},
                        {"if_viscous", E(kLogical, if_viscous)}, {"if_bodyforce", E(kLogical, if_bodyforce)},
                        {"mach_inf", E(kReal, mach_inf)}, {"reynolds", E(kReal, reynolds)},
                        {"benchmark_index", E(kInt, benchmark)}}},
        {"grid_pars", {{"if_curve_grid", E(kLogical, if_curve_grid)},
                       {"if_read_from_file", E(kLogical, if_read_from_file)},
                       {"single_ni", E(kInt, ni)}, {"single_nj", E(kInt, nj)}}},
        {"time_step_pars", {{"stages", E(kInt, stages)}, {"total_time", E(kReal, total_time)},
                            {"dt_save", E(kReal, dt_save)}, {"dt", E(kReal, dt)}, {"cfl", E(kReal, cfl)},
                            {"total_step", E(kInt, total_step)}, {"save_step", E(kInt, save_step)},
                            {"if_const_dt", E(kLogical, if_const_dt)},
                            {"if_save_binary", E(kLogical, if_save_binary)},
                            {"if_save_tec", E(kLogical, if_save_tec)}}},
        {"scheme_pars", {{"scheme_splitting_index", E(kInt, splitting)},
                         {"scheme_inv_index", E(kInt, recon)},
                         {"scheme_vis_index", E(kInt, scheme_vis_index)},
                         {"if_save_theta", E(kLogical, if_save_theta)}, {"delta", E(kReal, delta)}}},
        {"gas_pars", {{"gamma", E(kReal, gamma)}}},
    };
#undef E
    return g;
}

}  // namespace

extern "C" {

const char* dense_host_last_error(void) { return g_err.c_str(); }

int dense_config_size(void) { return (int)sizeof(dense_config_t); }

int dense_config_default(dense_config_t* c) {
    if (!c) return fail(DENSE_ERR_ARG, "null config");
    std::memset(c, 0, sizeof(*c));
    // flow_mod_general.f90:50-179
    c->omp_thread_num = 4;
    c->neq = 4;
    c->mach_inf = 1.0;
    c->reynolds = 500.0;
    c->benchmark = 0;
    c->ni = 64;
    c->nj = 64;
    c->bfsize = 4;
    c->stages = 3;
    c->total_time = 0.0;
    c->dt = 0.01;
    c->cfl = 0.5;
    c->total_step = 1;
    c->save_step = 100;
    c->dt_save = SP(0.01f);
    c->if_save_tec = 1;
    c->if_save_binary = 1;
    c->splitting = 101;
    c->recon = 201;
    c->scheme_vis_index = 301;
    c->delta = 0.5;
    c->gamma = 1.4;
    c->var_eps = 5.0;
    c->var_xc = 5.0;
    c->var_yc = 5.0;
    return DENSE_OK;
}

int dense_read_namelist(const char* path, dense_config_t* cfg) {
    if (!path || !cfg) return fail(DENSE_ERR_ARG, "null argument");
    std::ifstream f(path);
    if (!f) return fail(DENSE_ERR_IO, std::string("Input file ") + path + " does not exist!");
    std::stringstream ss;
    ss << f.rdbuf();
    // strip comments
    std::string text, line;
    std::istringstream lines(ss.str());
    while (std::getline(lines, line)) {
        bool q = false;
        for (size_t k = 0; k < line.size(); ++k) {
            if (line[k] == '\'' || line[k] == '"') q = !q;
            if (line[k] == '!' && !q) { line = line.substr(0, k); break; }
        }
        text += line + "\n";
    }
    const auto& G = groups();
    size_t pos = 0;
    while ((pos = text.find('&', pos)) != std::string::npos) {
        size_t nend = pos + 1;
        while (nend < text.size() && (std::isalnum((unsigned char)text[nend]) || text[nend] == '_')) ++nend;
        std::string gname = lower(text.substr(pos + 1, nend - pos - 1));
        size_t close = text.find('/', nend);
        if (close == std::string::npos) return fail(DENSE_ERR_IO, "namelist &" + gname + " is not closed by '/'");
        auto git = G.find(gname);
        if (git == G.end()) return fail(DENSE_ERR_IO, "unknown namelist group &" + gname);
        std::string body = text.substr(nend, close - nend);
        // split "name = value" items on '=' boundaries: value runs to the next "name ="
        std::vector<std::pair<std::string, std::string>> items;
        size_t k = 0;
        while (true) {
            size_t eq = body.find('=', k);
            if (eq == std::string::npos) break;
            std::string name = lower(trim(body.substr(k, eq - k)));
            // value: up to the next identifier followed by '='
            size_t nexteq = body.find('=', eq + 1);
            size_t vend = body.size();
            if (nexteq != std::string::npos) {
                size_t t = nexteq;
                while (t > eq + 1 && std::isspace((unsigned char)body[t - 1])) --t;
                while (t > eq + 1 && (std::isalnum((unsigned char)body[t - 1]) || body[t - 1] == '_')) --t;
                vend = t;
            }
            std::string value = trim(body.substr(eq + 1, vend - eq - 1));
            while (!value.empty() && (value.back() == ',' || std::isspace((unsigned char)value.back()))) value.pop_back();
            items.emplace_back(name, value);
            k = vend;
        }
        for (auto& it : items) {
            auto eit = git->second.find(it.first);
            if (eit == git->second.end())
                return fail(DENSE_ERR_IO, "Cannot match namelist object name " + it.first + " in &" + gname);
            char* base = (char*)cfg + eit->second.offset;
            bool ok = false;
            if (eit->second.kind == kInt) ok = parse_int(it.second, (int*)base);
            else if (eit->second.kind == kReal) ok = parse_real(it.second, (double*)base);
            else ok = parse_logical(it.second, (int*)base);
            if (!ok) return fail(DENSE_ERR_IO, "bad value '" + it.second + "' for " + it.first);
        }
        pos = close + 1;
    }
    return DENSE_OK;
}

int dense_setup_config(dense_config_t* cfg) {
    if (!cfg) return fail(DENSE_ERR_ARG, "null argument");
    if (cfg->ni < 3 || cfg->nj < 3) return fail(DENSE_ERR_ARG, "ni and nj must be >= 3");
    const double ni = cfg->ni, nj = cfg->nj;
    // the geometry lines of setup() above, without the arrays
    switch (cfg->benchmark) {
    case DENSE_BENCH_IVC: case DENSE_BENCH_IVC_PERIODIC: cfg->dx = 10.0 / ni; cfg->dy = 10.0 / nj; break;
    case DENSE_BENCH_SEDOV: cfg->dx = 1.2 / ni; cfg->dy = 1.2 / nj; break;
    case DENSE_BENCH_RT: case DENSE_BENCH_RT_REFLECT:
        cfg->if_bodyforce = 1;
        cfg->gamma = 5.0 / 3.0;
        cfg->dx = 0.25 / (ni - 1.0); cfg->dy = 1.0 / (nj - 1.0);
        break;
    case DENSE_BENCH_RM: case DENSE_BENCH_DMR: cfg->dx = 4.0 / ni; cfg->dy = 1.0 / nj; break;
    case DENSE_BENCH_RM_PERIODIC: cfg->dx = 1.0 / ni; cfg->dy = 1.0 / nj; break;
    case DENSE_BENCH_SSL: cfg->dx = 200.0 / ni; cfg->dy = 40.0 / nj; break;
    case DENSE_BENCH_SHOCKVORTEX: cfg->dx = 2.0 / ni; cfg->dy = 1.0 / nj; break;
    case DENSE_BENCH_USER: case 7: case 8: break;  // nothing is initialised (init_general.f90:26-33)
    default: return fail(DENSE_ERR_BENCHMARK, "No such Benchmark index! (init_general.f90:34-36)");
    }
    return DENSE_OK;
}

int dense_grid_coords(const dense_config_t* cfg, double* x, double* y, double* vx, double* vy) {
    if (!cfg || cfg->ni < 1 || cfg->nj < 1) return fail(DENSE_ERR_ARG, "bad config");
    const int ni = cfg->ni, nj = cfg->nj, b = cfg->benchmark;
    const bool vertex = b == DENSE_BENCH_RT || b == DENSE_BENCH_RT_REFLECT;  // init_RT_general.f90:16-22
    const bool none = b == DENSE_BENCH_USER || b == 7 || b == 8;
    const double ys = b == DENSE_BENCH_SSL ? 40.0 / 2.0 : 0.0;             // init_ssl_general.f90:28
    const double dx = cfg->dx, dy = cfg->dy;
    // cell coordinates x(ni,nj), y(ni,nj) as the setups write them
    for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
            const size_t o = (size_t)(i - 1) + (size_t)ni * (j - 1);
            const double cx = none ? 0.0 : vertex ? (i - 1.0) * dx : (i - 0.5) * dx;
            const double cy = none ? 0.0 : vertex ? (j - 1.0) * dy : (j - 0.5) * dy - ys;
            if (x) x[o] = cx;
            if (y) y[o] = cy;
        }
    // vertex coordinates vet_x(ni+1,nj+1), vet_y (e.g. init_IVC_general.f90:28-29; RT :29-30)
    for (int j = 1; j <= nj + 1; ++j)
        for (int i = 1; i <= ni + 1; ++i) {
            const size_t o = (size_t)(i - 1) + (size_t)(ni + 1) * (j - 1);
            const double ox = vertex ? 1.5 : 1.0;
            if (vx) vx[o] = none ? 0.0 : (i - ox) * dx;
            if (vy) vy[o] = none ? 0.0 : (j - ox) * dy - ys;
        }
    return DENSE_OK;
}

int dense_array_sizes(const dense_config_t* cfg, long long* cons_count, long long* prim_count,
                      long long* xy_count) {
    if (!cfg || cfg->ni <= 0 || cfg->nj <= 0) return fail(DENSE_ERR_ARG, "bad config");
    const long long NIp = cfg->ni + 8, NJp = cfg->nj + 8;
    if (cons_count) *cons_count = NIp * NJp * 4;
    if (prim_count) *prim_count = NIp * NJp * 6;
    if (xy_count) *xy_count = (long long)cfg->ni * cfg->nj;
    return DENSE_OK;
}

int dense_init_setup(dense_config_t* cfg, double* cons, double* prim, double* x, double* y) {
    if (!cfg || !cons || !prim || !x || !y) return fail(DENSE_ERR_ARG, "null argument");
    if (cfg->ni < 3 || cfg->nj < 3) return fail(DENSE_ERR_ARG, "ni and nj must be >= 3");
    if (cfg->bfsize != 4) return fail(DENSE_ERR_ARG, "bfsize must be 4");
    Views w{cfg->ni, cfg->nj, cfg->ni + 8, cfg->nj + 8, cons, prim, x, y};
    const size_t P = (size_t)w.NIp * w.NJp;
    std::memset(cons, 0, P * 4 * sizeof(double));
    std::memset(prim, 0, P * 6 * sizeof(double));
    std::memset(x, 0, (size_t)w.ni * w.nj * sizeof(double));
    std::memset(y, 0, (size_t)w.ni * w.nj * sizeof(double));
    return setup(cfg, w);
}

}  // extern "C"
