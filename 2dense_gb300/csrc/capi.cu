// capi.cu — the C ABI of include/dense2d.h over the sm_103a kernels: device buffers of one
// block, its stream, the CUDA graph of one time step, status and errors.
#include <cuda_runtime.h>

#include <cstdlib>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "handle.h"
#include "nvtx.h"

extern "C" const char* dense_host_last_error(void);
extern "C" const char* dense_io_last_error(void);

using dense::KernelTable;
using dense::Params;
using dense::Scalars;
using dense::kB;

namespace {

thread_local std::string g_err;

int seterr(dense_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg; else g_err = msg;
    return code;
}

#define CK(h, call)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return seterr((h), DENSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

__global__ void k_set_loop(Scalars* sc, double t, long long step, double t_end, long long total_step,
                           int active) {
    sc->t = t;
    sc->step = step;
    sc->t_end = t_end;
    sc->total_step = total_step;
    sc->active = active;
}
__global__ void k_set_dt(Scalars* sc, double dt) { sc->dt = dt; }
__global__ void k_set_bounds(Scalars* sc, double t_end, long long total_step) {
    sc->t_end = t_end;
    sc->total_step = total_step;
}
__global__ void k_set_time(Scalars* sc, double t, long long step) {
    sc->t = t;
    sc->step = step;
}
__global__ void k_set_active(Scalars* sc) { sc->active = 1; }

// A stack of rows between the padded device layout (row pitch P) and the caller's Fortran
// layout (rows of NIp doubles): one contiguous copy when the pitches agree (NIp even), a pitched
// copy otherwise.
cudaError_t copy_rows(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t rows,
                      cudaMemcpyKind kind, cudaStream_t s) {
    if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * rows, kind, s);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, s);
}

bool valid_split(int s) { return s >= DENSE_SPLIT_LLF && s <= DENSE_SPLIT_SC; }
bool valid_bench(int b) {
    return b == 0 || (b >= 1 && b <= 9) || b == DENSE_BENCH_IVC_PERIODIC || b == DENSE_BENCH_RT_REFLECT ||
           b == DENSE_BENCH_RM_PERIODIC;
}

int check_config(dense_handle* h, const dense_config_t* c) {
    if (!c) return seterr(h, DENSE_ERR_ARG, "null config");
    if (c->ni < 3 || c->nj < 3) return seterr(h, DENSE_ERR_ARG, "ni and nj must be >= 3");
    if (c->bfsize != kB) return seterr(h, DENSE_ERR_ARG, "bfsize must be 4 (allocate_block(...,4,4,neq))");
    if (c->neq != 4) return seterr(h, DENSE_ERR_ARG, "neq must be 4");
    if (c->stages != 3) return seterr(h, DENSE_ERR_ARG, "stages must be 3 (time_rk3_general)");
    if (!valid_split(c->splitting))
        return seterr(h, DENSE_ERR_SPLITTING, "No such Selection (flux_splitting.f90:30-32)");
    if (!valid_bench(c->benchmark))
        return seterr(h, DENSE_ERR_BENCHMARK, "No such Benchmark index! (boundary_general.f90:26-28)");
    if (c->dx <= 0.0 || c->dy <= 0.0) return seterr(h, DENSE_ERR_ARG, "dx and dy must be set (dense_init_setup)");
    if (c->strict < 0 || c->strict > 2) return seterr(h, DENSE_ERR_ARG, "strict must be 0 (fast), 1 (strict) or 2 (checked)");
    return DENSE_OK;
}

void fill_params(dense_handle* h) {
    Params& p = h->prm;
    const dense_config_t& c = h->cfg;
    p.cons = h->cons; p.prim = h->prim; p.cons0 = h->cons0; p.hx = h->hx; p.he = h->he;
    p.xbot = h->xbot; p.xtop = h->xtop; p.yleft = h->yleft;
    p.sc = h->sc;
    p.ni = c.ni; p.nj = c.nj; p.P = h->P;
    p.plane = (long long)h->NJp * h->P;
    p.gamma = c.gamma; p.cfl = c.cfl; p.delta = c.delta; p.dx = c.dx; p.dy = c.dy; p.dt_const = c.dt;
    p.theta_c = dense::theta_c_of(c.delta);
    p.if_const_dt = c.if_const_dt;
    // the body force is nonzero only where boundary_rt_general refreshes it (:154-155)
    p.bodyforce = c.if_bodyforce && (c.benchmark == DENSE_BENCH_RT || c.benchmark == DENSE_BENCH_RT_REFLECT);
    p.benchmark = c.benchmark; p.splitting = c.splitting; p.recon = c.recon;
    p.periodic_ghosts = dense::periodic_ghosts(c.benchmark, c.ni, c.nj);
    p.count_branches = h->count_branches;
    p.tape = nullptr;
    p.theta = c.if_save_theta && c.splitting == DENSE_SPLIT_SC ? h->theta : nullptr;
    h->kt = dense::kernels_for(c.strict);
}

// the indicator buffer, allocated while a configuration saves it
int ensure_theta(dense_handle* h) {
    if (!h->theta && h->cfg.if_save_theta && h->cfg.splitting == DENSE_SPLIT_SC) {
        const size_t n = (size_t)2 * ((size_t)h->cfg.nj * (h->cfg.ni + 1) + (size_t)(h->cfg.nj + 1) * h->cfg.ni);
        CK(h, cudaMalloc((void**)&h->theta, n * sizeof(double)));
        CK(h, cudaMemsetAsync(h->theta, 0, n * sizeof(double), h->stream));
    }
    return DENSE_OK;
}

void drop_graph(dense_handle* h) {
    if (h->step_graph) cudaGraphExecDestroy(h->step_graph);
    h->step_graph = nullptr;
    h->graph_nodes = 0;
}

int launch_check(dense_handle* h) {
    CK(h, cudaGetLastError());
    return DENSE_OK;
}

// get_primary of the current state into slot `slot`.
int ensure_prim(dense_handle* h, int slot) {
    if (h->prim_slot == slot) return DENSE_OK;
    CK(h, cudaMemsetAsync(&h->sc->maxeig[slot][0], 0, 2 * sizeof(double), h->stream));
    h->kt->prim(h->prm, slot, h->stream);
    h->launches += 1;
    h->prim_slot = slot;
    return launch_check(h);
}

// one stage: boundary_general -> flux_splitting_general -> time_rk3_general(irk)
void enqueue_stage(dense_handle* h, int irk) {
    h->kt->bc(h->prm, h->stream);
    h->kt->flux(h->prm, irk, 0, h->stream);
    h->kt->flux(h->prm, irk, 1, h->stream);
    h->kt->update(h->prm, irk, h->stream);
}
int stage_launches(dense_handle* h) {
    return 2 + h->kt->flux_launches(h->prm, 0) + h->kt->flux_launches(h->prm, 1);
}

// The stage as graph nodes: the two sweeps read the same stage input and write separate face
// fluxes, so the eta sweep is a branch beside the xi sweep; its blocks fill the SMs the xi
// sweep's last wave leaves idle. The update joins both. On grids periodic in x and y the
// previous stage's update has written the ghost layers already, so stages 2 and 3 launch no
// boundary fill (stage 1 keeps it: the step may start from an uploaded state).
cudaError_t capture_stage(dense_handle* h, int irk) {
    if (irk == 1 || !h->prm.periodic_ghosts) h->kt->bc(h->prm, h->stream);
    cudaError_t e = cudaEventRecord(h->ev_fork, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->side, h->ev_fork, 0);
    if (e != cudaSuccess) return e;
    h->kt->flux(h->prm, irk, 1, h->side);
    h->kt->flux(h->prm, irk, 0, h->stream);
    e = cudaEventRecord(h->ev_join, h->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, h->ev_join, 0);
    if (e != cudaSuccess) return e;
    h->kt->update(h->prm, irk, h->stream);
    return cudaSuccess;
}

// the side stream and the fork/join events of a stage's two sweeps
int ensure_side(dense_handle* h) {
    if (!h->side) CK(h, cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    if (!h->ev_fork) CK(h, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    if (!h->ev_join) CK(h, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    return DENSE_OK;
}

// The step graph's kernel-to-kernel edges made programmatic: a kernel's blocks may be scheduled
// as its predecessor's last blocks drain instead of after the predecessor has finished, and
// wait (griddepcontrol.wait, first thing in every step-graph kernel) for its completion and
// memory. Measured per step (CUDA events, L2 flushed): AdaWENO's double Mach reflection gains
// 0.9 % at 960 x 240, 1.6 % at 1920 x 480 and 0.5 % at 3840 x 960; the component-wise and
// characteristic schemes gain nothing on large grids (vortex 1024 x 1024, Rayleigh-Taylor
// 512 x 2048) and lose on small ones (Rayleigh-Taylor 256 x 1024 1 %, the 200 x 200 vortex 19 %:
// the early blocks wait on SMs the one-wave kernel before them still needs). So: AdaWENO grids
// of 200,000 cells or more; DENSE_PDL=0 / 1 in the environment forces it off / on.
bool use_programmatic_edges(const dense_handle* h) {
    static const int env = [] {
        const char* v = std::getenv("DENSE_PDL");
        return v && (v[0] == '0' || v[0] == '1') ? v[0] - '0' : -1;
    }();
    if (env >= 0) return env == 1;
    return h->prm.splitting == DENSE_SPLIT_SC && (long long)h->prm.ni * h->prm.nj >= 200000;
}
cudaError_t programmatic_edges(cudaGraph_t g) {
    size_t ne = 0;
    cudaError_t e = cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &ne);
    if (e != cudaSuccess || ne == 0) return e;
    std::vector<cudaGraphNode_t> from(ne), to(ne);
    std::vector<cudaGraphEdgeData> ed(ne);
    e = cudaGraphGetEdges(g, from.data(), to.data(), ed.data(), &ne);
    for (size_t k = 0; k < ne && e == cudaSuccess; ++k) {
        cudaGraphNodeType ta, tb;
        e = cudaGraphNodeGetType(from[k], &ta);
        if (e == cudaSuccess) e = cudaGraphNodeGetType(to[k], &tb);
        if (e != cudaSuccess || ta != cudaGraphNodeTypeKernel || tb != cudaGraphNodeTypeKernel) continue;
        cudaGraphEdgeData pe{};
        pe.from_port = cudaGraphKernelNodePortProgrammatic;
        pe.type = cudaGraphDependencyTypeProgrammatic;
        e = cudaGraphRemoveDependencies(g, &from[k], &to[k], &ed[k], 1);
        if (e == cudaSuccess) e = cudaGraphAddDependencies(g, &from[k], &to[k], &pe, 1);
    }
    return e;
}

int build_step_graph(dense_handle* h) {
    if (h->step_graph) return DENSE_OK;
    int rc = ensure_side(h);
    if (rc) return rc;
    cudaGraph_t g = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->kt->step_begin(h->prm, h->stream);
    cudaError_t ce = cudaSuccess;
    for (int irk = 1; irk <= 3 && ce == cudaSuccess; ++irk) ce = capture_stage(h, irk);
    h->kt->step_end(h->prm, h->stream);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e == cudaSuccess && ce != cudaSuccess) {
        cudaGraphDestroy(g);
        e = ce;
    }
    if (e != cudaSuccess) return seterr(h, DENSE_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
    if (use_programmatic_edges(h)) e = programmatic_edges(g);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return seterr(h, DENSE_ERR_CUDA, std::string("step graph edges: ") + cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&h->step_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return seterr(h, DENSE_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    h->graph_nodes = 2 + 3 * stage_launches(h) - (h->prm.periodic_ghosts ? 2 : 0);
    return DENSE_OK;
}

// rhs[v][j][i] = -(hx[v][j][i+1] - hx[v][j][i])/dx - (he[v][j+1][i] - he[v][j][i])/dy
__global__ void k_rhs(const double* __restrict__ hx, const double* __restrict__ he, int ni, int nj, double dx,
                      double dy, double* __restrict__ rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= ni || j >= nj) return;
    const long long xs = (long long)nj * (ni + 1), ys = (long long)(nj + 1) * ni;
    for (int v = 0; v < 4; ++v) {
        const double* X = hx + v * xs + (long long)j * (ni + 1) + i;
        const double* Y = he + v * ys + (long long)j * ni + i;
        rhs[(long long)v * ni * nj + (long long)j * ni + i] = -(X[1] - X[0]) / dx - (Y[ni] - Y[0]) / dy;
    }
}

// order the handle's stream after the caller's, and the caller's after the handle's
int wait_for(dense_handle* h, void* caller) {
    cudaEvent_t e;
    CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaError_t r = cudaEventRecord(e, (cudaStream_t)caller);
    if (r == cudaSuccess) r = cudaStreamWaitEvent(h->stream, e, 0);
    cudaEventDestroy(e);
    if (r != cudaSuccess) return seterr(h, DENSE_ERR_CUDA, std::string("stream order: ") + cudaGetErrorString(r));
    return DENSE_OK;
}
int signal_to(dense_handle* h, void* caller) {
    cudaEvent_t e;
    CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaError_t r = cudaEventRecord(e, h->stream);
    if (r == cudaSuccess) r = cudaStreamWaitEvent((cudaStream_t)caller, e, 0);
    cudaEventDestroy(e);
    if (r != cudaSuccess) return seterr(h, DENSE_ERR_CUDA, std::string("stream order: ") + cudaGetErrorString(r));
    return DENSE_OK;
}

}  // namespace

int dense::handle_ensure_prim(dense_handle* h, int slot) { return ensure_prim(h, slot); }
void dense::set_last_error(const char* msg) { g_err = msg ? msg : ""; }
int dense::handle_step_graph(dense_handle* h) { return build_step_graph(h); }
int dense::handle_stage_launches(dense_handle* h) { return stage_launches(h); }
int dense::handle_ensure_side(dense_handle* h) { return ensure_side(h); }

extern "C" {

const char* dense_last_error(dense_handle_t* h) {
    if (h) return h->err.c_str();
    if (!g_err.empty()) return g_err.c_str();
    const char* io = dense_io_last_error();
    if (io && *io) return io;
    return dense_host_last_error();
}

int dense_create(const dense_config_t* cfg, dense_handle_t** out) {
    if (!out) return seterr(nullptr, DENSE_ERR_ARG, "null out");
    *out = nullptr;
    int rc = check_config(nullptr, cfg);
    if (rc) return rc;
    auto* h = new dense_handle();
    h->cfg = *cfg;
    h->NIp = cfg->ni + 2 * kB;
    h->NJp = cfg->nj + 2 * kB;
    h->P = (h->NIp + 1) & ~1;  // even pitch: rows start on 16-byte boundaries
    auto cleanup = [&](int code) { dense_destroy(h); return code; };
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { g_err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); delete h; return DENSE_ERR_CUDA; }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); delete h; return DENSE_ERR_CUDA; }
    const size_t plane = (size_t)h->NJp * h->P;
    struct A { double** p; size_t n; } allocs[] = {
        {&h->cons, plane * 4}, {&h->prim, plane * 5}, {&h->cons0, plane * 4},
        {&h->hx, (size_t)4 * cfg->nj * (cfg->ni + 1)}, {&h->he, (size_t)4 * (cfg->nj + 1) * cfg->ni},
        {&h->xbot, (size_t)cfg->ni}, {&h->xtop, (size_t)cfg->ni}, {&h->yleft, (size_t)cfg->nj},
    };
    for (auto& a : allocs) {
        e = cudaMalloc((void**)a.p, a.n * sizeof(double));
        if (e != cudaSuccess) { g_err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return cleanup(DENSE_ERR_NOMEM); }
        e = cudaMemsetAsync(*a.p, 0, a.n * sizeof(double), h->stream);
        if (e != cudaSuccess) { g_err = std::string("cudaMemset: ") + cudaGetErrorString(e); return cleanup(DENSE_ERR_CUDA); }
    }
    if (ensure_theta(h) != DENSE_OK) { g_err = h->err; return cleanup(DENSE_ERR_NOMEM); }
    e = cudaMalloc((void**)&h->sc, sizeof(Scalars));
    if (e != cudaSuccess) { g_err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return cleanup(DENSE_ERR_NOMEM); }
    Scalars s0{};
    s0.dt = cfg->dt;
    s0.t_end = 0.0;
    e = cudaMemcpyAsync(h->sc, &s0, sizeof(Scalars), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { g_err = std::string("scalars: ") + cudaGetErrorString(e); return cleanup(DENSE_ERR_CUDA); }
    fill_params(h);
    *out = h;
    return DENSE_OK;
}

void dense_destroy(dense_handle_t* h) {
    if (!h) return;
    drop_graph(h);
    double* bufs[] = {h->cons, h->prim, h->cons0, h->hx, h->he, h->xbot, h->xtop, h->yleft, h->theta};
    for (double* b : bufs) if (b) cudaFree(b);
    if (h->sc) cudaFree(h->sc);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int dense_upload(dense_handle_t* h, const double* cons, const double* prim, const double* x, const double* y) {
    dense::NvtxRange nvtx_("dense_upload");
    if (!h || !cons) return seterr(h, DENSE_ERR_ARG, "null handle or cons");
    const dense_config_t& c = h->cfg;
    const size_t row = (size_t)h->NIp * sizeof(double), pitch = (size_t)h->P * sizeof(double);
    // Fortran cons(NIp,NJp,4) is a stack of 4*NJp rows of NIp doubles: one pitched copy
    CK(h, copy_rows(h->cons, pitch, cons, row, row, (size_t)h->NJp * 4, cudaMemcpyHostToDevice, h->stream));
    if (prim) {
        CK(h, copy_rows(h->prim, pitch, prim, row, row, (size_t)h->NJp * 5, cudaMemcpyHostToDevice, h->stream));
    } else {
        CK(h, cudaMemsetAsync(h->prim, 0, (size_t)h->NJp * h->P * 5 * sizeof(double), h->stream));
    }
    std::vector<double> xb(c.ni, 0.0), xt(c.ni, 0.0), yl(c.nj, 0.0);
    if (x) for (int i = 0; i < c.ni; ++i) { xb[i] = x[i]; xt[i] = x[(size_t)c.ni * (c.nj - 1) + i]; }
    if (y) for (int j = 0; j < c.nj; ++j) yl[j] = y[(size_t)c.ni * j];
    CK(h, cudaMemcpyAsync(h->xbot, xb.data(), c.ni * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->xtop, xt.data(), c.ni * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->yleft, yl.data(), c.nj * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->uploaded = true;
    h->prim_slot = -1;
    int rc = ensure_prim(h, 0);
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->stream));  // the caller's buffers may be reused on return
    return DENSE_OK;
}

int dense_stage(dense_handle_t* h, int irk, double current_time, double* dt_inout) {
    dense::NvtxRange nvtx_("dense_stage");
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    if (irk < 1 || irk > 3) return seterr(h, DENSE_ERR_ARG, "irk must be 1, 2 or 3");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_stage before dense_upload");
    int rc = ensure_prim(h, irk - 1);
    if (rc) return rc;
    k_set_loop<<<1, 1, 0, h->stream>>>(h->sc, current_time, 0, 0.0, 0, 1);
    h->launches += 1;
    enqueue_stage(h, irk);
    h->launches += stage_launches(h);
    rc = launch_check(h);
    if (rc) return rc;
    h->prim_slot = irk % 3;
    double dt = 0.0;
    CK(h, cudaMemcpyAsync(&dt, &h->sc->dt, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (dt_inout) *dt_inout = dt;
    return DENSE_OK;
}

int dense_steps(dense_handle_t* h, int nsteps, double t_end, int total_step, double* t_inout,
                int* step_inout, double* dt_out) {
    dense::NvtxRange nvtx_("dense_steps");
    if (!h || !t_inout || !step_inout) return seterr(h, DENSE_ERR_ARG, "null argument");
    if (nsteps < 0) return seterr(h, DENSE_ERR_ARG, "nsteps < 0");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_steps before dense_upload");
    int rc = ensure_prim(h, 0);
    if (rc) return rc;
    rc = build_step_graph(h);
    if (rc) return rc;
    k_set_loop<<<1, 1, 0, h->stream>>>(h->sc, *t_inout, *step_inout, t_end, total_step, 0);
    h->launches += 1;
    for (int s = 0; s < nsteps; ++s) {
        CK(h, cudaGraphLaunch(h->step_graph, h->stream));
        h->launches += h->graph_nodes;
    }
    Scalars s{};
    CK(h, cudaMemcpyAsync(&s, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *t_inout = s.t;
    *step_inout = (int)s.step;
    if (dt_out) *dt_out = s.dt;
    return DENSE_OK;
}

int dense_download(dense_handle_t* h, double* cons, double* prim) {
    dense::NvtxRange nvtx_("dense_download");
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_download before dense_upload");
    const size_t row = (size_t)h->NIp * sizeof(double), pitch = (size_t)h->P * sizeof(double);
    if (cons)
        CK(h, copy_rows(cons, row, h->cons, pitch, row, (size_t)h->NJp * 4, cudaMemcpyDeviceToHost, h->stream));
    if (prim)
        CK(h, copy_rows(prim, row, h->prim, pitch, row, (size_t)h->NJp * 5, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (prim) {
        // entropy log(p)-log(rho) of the interior (get_primary.f90:67); ghosts hold 0
        const size_t P = (size_t)h->NIp * h->NJp;
        double* s6 = prim + 5 * P;
        std::memset(s6, 0, P * sizeof(double));
        for (int J = kB; J < h->NJp - kB; ++J)
            for (int I = kB; I < h->NIp - kB; ++I) {
                const size_t o = (size_t)J * h->NIp + I;
                s6[o] = std::log(prim[3 * P + o]) - std::log(prim[o]);
            }
    }
    return DENSE_OK;
}

int dense_get_max_eig(dense_handle_t* h, double* mi, double* mj) {
    if (!h || !mi || !mj) return seterr(h, DENSE_ERR_ARG, "null argument");
    if (h->prim_slot < 0) return seterr(h, DENSE_ERR_STATE, "no get_primary yet");
    double m[2];
    CK(h, cudaMemcpyAsync(m, &h->sc->maxeig[h->prim_slot][0], sizeof(m), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *mi = m[0];
    *mj = m[1];
    return DENSE_OK;
}

int dense_reconfigure(dense_handle_t* h, const dense_config_t* cfg) {
    if (!h || !cfg) return seterr(h, DENSE_ERR_ARG, "null argument");
    if (cfg->ni != h->cfg.ni || cfg->nj != h->cfg.nj || cfg->benchmark != h->cfg.benchmark)
        return seterr(h, DENSE_ERR_ARG, "grid size and benchmark cannot change on a live handle");
    int rc = check_config(h, cfg);
    if (rc) return rc;
    h->cfg = *cfg;
    rc = ensure_theta(h);
    if (rc) return rc;
    fill_params(h);
    drop_graph(h);
    h->prim_slot = -1;  // gamma may have changed: recompute primitives before the next stage
    k_set_dt<<<1, 1, 0, h->stream>>>(h->sc, cfg->dt);
    h->launches += 1;
    return launch_check(h);
}

int dense_status(dense_handle_t* h, unsigned* flags) {
    if (!h || !flags) return seterr(h, DENSE_ERR_ARG, "null argument");
    unsigned f = 0;
    CK(h, cudaMemcpyAsync(&f, &h->sc->status, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemsetAsync(&h->sc->status, 0, sizeof(unsigned), h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *flags = f;
    return DENSE_OK;
}

int dense_get_fluxes(dense_handle_t* h, double* h_xi, double* h_eta) {
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    const int ni = h->cfg.ni, nj = h->cfg.nj;
    if (h_xi)  // device hx[v][j][f] == Fortran h_xi(f,j,v)
        CK(h, cudaMemcpyAsync(h_xi, h->hx, (size_t)4 * nj * (ni + 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    std::vector<double> tmp;
    if (h_eta) {
        tmp.resize((size_t)4 * (nj + 1) * ni);
        CK(h, cudaMemcpyAsync(tmp.data(), h->he, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    if (h_eta)  // device he[v][g][i] -> Fortran h_eta(g,i,v)
        for (int v = 0; v < 4; ++v)
            for (int g = 0; g <= nj; ++g)
                for (int i = 0; i < ni; ++i)
                    h_eta[(size_t)g + (size_t)(nj + 1) * ((size_t)i + (size_t)ni * v)] =
                        tmp[(size_t)v * (nj + 1) * ni + (size_t)g * ni + i];
    return DENSE_OK;
}

long long dense_launch_count(dense_handle_t* h) { return h ? h->launches : -1; }

int dense_get_stream(dense_handle_t* h, void** stream) {
    if (!h || !stream) return seterr(h, DENSE_ERR_ARG, "null argument");
    *stream = (void*)h->stream;
    return DENSE_OK;
}

int dense_steps_async(dense_handle_t* h, int nsteps, double t_end, int total_step) {
    dense::NvtxRange nvtx_("dense_steps_async");
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    if (nsteps < 0) return seterr(h, DENSE_ERR_ARG, "nsteps < 0");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_steps_async before dense_upload");
    int rc = ensure_prim(h, 0);
    if (rc) return rc;
    rc = build_step_graph(h);
    if (rc) return rc;
    k_set_bounds<<<1, 1, 0, h->stream>>>(h->sc, t_end, total_step);
    h->launches += 1;
    for (int s = 0; s < nsteps; ++s) {
        CK(h, cudaGraphLaunch(h->step_graph, h->stream));
        h->launches += h->graph_nodes;
    }
    return DENSE_OK;
}

int dense_get_time(dense_handle_t* h, double* t, int* step, double* dt) {
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    Scalars s{};
    CK(h, cudaMemcpyAsync(&s, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (t) *t = s.t;
    if (step) *step = (int)s.step;
    if (dt) *dt = s.dt;
    return DENSE_OK;
}

int dense_set_time(dense_handle_t* h, double t, int step) {
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    k_set_time<<<1, 1, 0, h->stream>>>(h->sc, t, step);
    h->launches += 1;
    return launch_check(h);
}

int dense_sync(dense_handle_t* h) {
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    CK(h, cudaStreamSynchronize(h->stream));
    return DENSE_OK;
}

int dense_count_branches(dense_handle_t* h, int enable) {
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    h->count_branches = enable ? 1 : 0;
    fill_params(h);
    drop_graph(h);
    CK(h, cudaMemsetAsync(h->sc->branch_count, 0, sizeof(h->sc->branch_count), h->stream));
    return DENSE_OK;
}

int dense_get_branch_counts(dense_handle_t* h, unsigned long long* counts) {
    if (!h || !counts) return seterr(h, DENSE_ERR_ARG, "null argument");
    CK(h, cudaMemcpyAsync(counts, h->sc->branch_count, sizeof(h->sc->branch_count),
                          cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return DENSE_OK;
}

int dense_profile_stage(dense_handle_t* h, int irk, float* ms) {
    if (!h || !ms) return seterr(h, DENSE_ERR_ARG, "null argument");
    if (irk < 1 || irk > 3) return seterr(h, DENSE_ERR_ARG, "irk must be 1, 2 or 3");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_profile_stage before dense_upload");
    int rc = ensure_prim(h, irk - 1);
    if (rc) return rc;
    k_set_active<<<1, 1, 0, h->stream>>>(h->sc);
    cudaEvent_t ev[5];
    for (auto& e : ev) CK(h, cudaEventCreate(&e));
    CK(h, cudaEventRecord(ev[0], h->stream));
    h->kt->bc(h->prm, h->stream);
    CK(h, cudaEventRecord(ev[1], h->stream));
    h->kt->flux(h->prm, irk, 0, h->stream);
    CK(h, cudaEventRecord(ev[2], h->stream));
    h->kt->flux(h->prm, irk, 1, h->stream);
    CK(h, cudaEventRecord(ev[3], h->stream));
    h->kt->update(h->prm, irk, h->stream);
    CK(h, cudaEventRecord(ev[4], h->stream));
    h->launches += 1 + stage_launches(h);
    CK(h, cudaEventSynchronize(ev[4]));
    for (int k = 0; k < 4; ++k) CK(h, cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]));
    for (auto& e : ev) cudaEventDestroy(e);
    h->prim_slot = irk % 3;
    return launch_check(h);
}


int dense_upload_device(dense_handle_t* h, const double* cons, const double* prim, void* stream) {
    dense::NvtxRange nvtx_("dense_upload_device");
    if (!h || !cons) return seterr(h, DENSE_ERR_ARG, "null handle or cons");
    int rc = wait_for(h, stream);
    if (rc) return rc;
    const size_t row = (size_t)h->NIp * sizeof(double), pitch = (size_t)h->P * sizeof(double);
    CK(h, copy_rows(h->cons, pitch, cons, row, row, (size_t)h->NJp * 4, cudaMemcpyDeviceToDevice, h->stream));
    if (prim)
        CK(h, copy_rows(h->prim, pitch, prim, row, row, (size_t)h->NJp * 5, cudaMemcpyDeviceToDevice, h->stream));
    h->uploaded = true;
    h->prim_slot = -1;
    rc = ensure_prim(h, 0);
    if (rc) return rc;
    return signal_to(h, stream);
}

int dense_download_device(dense_handle_t* h, double* cons, double* prim, void* stream) {
    dense::NvtxRange nvtx_("dense_download_device");
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_download_device before an upload");
    int rc = wait_for(h, stream);
    if (rc) return rc;
    const size_t row = (size_t)h->NIp * sizeof(double), pitch = (size_t)h->P * sizeof(double);
    if (cons)
        CK(h, copy_rows(cons, row, h->cons, pitch, row, (size_t)h->NJp * 4, cudaMemcpyDeviceToDevice, h->stream));
    if (prim)
        CK(h, copy_rows(prim, row, h->prim, pitch, row, (size_t)h->NJp * 5, cudaMemcpyDeviceToDevice, h->stream));
    return signal_to(h, stream);
}

int dense_rhs_device(dense_handle_t* h, int irk, double* rhs, void* stream) {
    dense::NvtxRange nvtx_("dense_rhs_device");
    if (!h || !rhs) return seterr(h, DENSE_ERR_ARG, "null argument");
    if (irk < 1 || irk > 3) return seterr(h, DENSE_ERR_ARG, "irk must be 1, 2 or 3");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_rhs_device before an upload");
    int rc = wait_for(h, stream);
    if (!rc) rc = ensure_prim(h, irk - 1);
    if (rc) return rc;
    k_set_active<<<1, 1, 0, h->stream>>>(h->sc);
    h->kt->bc(h->prm, h->stream);
    h->kt->flux(h->prm, irk, 0, h->stream);
    h->kt->flux(h->prm, irk, 1, h->stream);
    const dim3 b(32, 8), g((h->cfg.ni + 31) / 32, (h->cfg.nj + 7) / 8);
    k_rhs<<<g, b, 0, h->stream>>>(h->hx, h->he, h->cfg.ni, h->cfg.nj, h->cfg.dx, h->cfg.dy, rhs);
    h->launches += 2 + h->kt->flux_launches(h->prm, 0) + h->kt->flux_launches(h->prm, 1) + 1;
    rc = launch_check(h);
    if (rc) return rc;
    return signal_to(h, stream);
}

// dt_dev: for irk 1 without constant dt receives the CFL time step; otherwise gives it
__global__ void k_dt_in(Scalars* sc, const double* dt, int irk, int const_dt) {
    if (irk > 1 || const_dt) sc->dt = *dt;
}
__global__ void k_dt_out(const Scalars* sc, double* dt) { *dt = sc->dt; }

int dense_stage_device(dense_handle_t* h, int irk, const double* cons0, double* dt, double current_time,
                       void* stream) {
    dense::NvtxRange nvtx_("dense_stage_device");
    if (!h || !dt) return seterr(h, DENSE_ERR_ARG, "null argument");
    if (irk < 1 || irk > 3) return seterr(h, DENSE_ERR_ARG, "irk must be 1, 2 or 3");
    if (irk > 1 && !cons0) return seterr(h, DENSE_ERR_ARG, "stages 2 and 3 need the step's initial state");
    if (!h->uploaded) return seterr(h, DENSE_ERR_STATE, "dense_stage_device before an upload");
    int rc = wait_for(h, stream);
    if (rc) return rc;
    if (irk > 1) {
        const size_t row = (size_t)h->NIp * sizeof(double), pitch = (size_t)h->P * sizeof(double);
        CK(h, copy_rows(h->cons0, pitch, cons0, row, row, (size_t)h->NJp * 4, cudaMemcpyDeviceToDevice,
                                h->stream));
    }
    rc = ensure_prim(h, irk - 1);
    if (rc) return rc;
    k_set_loop<<<1, 1, 0, h->stream>>>(h->sc, current_time, 0, 0.0, 0, 1);
    k_dt_in<<<1, 1, 0, h->stream>>>(h->sc, dt, irk, h->cfg.if_const_dt);
    enqueue_stage(h, irk);
    k_dt_out<<<1, 1, 0, h->stream>>>(h->sc, dt);
    h->launches += 3 + stage_launches(h);
    rc = launch_check(h);
    if (rc) return rc;
    h->prim_slot = irk % 3;
    return signal_to(h, stream);
}

int dense_steps_device(dense_handle_t* h, int nsteps, double t_end, int total_step, void* stream) {
    dense::NvtxRange nvtx_("dense_steps_device");
    if (!h) return seterr(h, DENSE_ERR_ARG, "null handle");
    int rc = wait_for(h, stream);
    if (!rc) rc = dense_steps_async(h, nsteps, t_end, total_step);
    if (rc) return rc;
    return signal_to(h, stream);
}

}  // extern "C"
