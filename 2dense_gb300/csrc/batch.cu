// batch.cu — the batched form: many independent solver blocks of uneven size, each with its own
// configuration, CFL time step, time and step count, advanced together. One launch per phase
// covers every instance (a block table maps each CUDA block to an instance and a tile of it), and
// one time step of the whole batch is one CUDA graph. Each instance's arithmetic is the plain
// single-instance code, so results are identical to solving the instances one by one.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "internal.h"
#include "setups.cuh"
#include "nvtx.h"

using dense::BatchLaunch;
using dense::Params;
using dense::Scalars;
using dense::kB;

struct dense_batch {
    int n = 0;
    std::vector<dense_config_t> cfg;
    std::vector<Params> prm;      // host copy of the instance table
    Params* tab = nullptr;        // device instance table
    char* pool = nullptr;         // one allocation for every instance's buffers
    size_t pool_bytes = 0;
    int* maps = nullptr;          // device block maps (int3 entries)
    size_t maps_cap = 0;
    BatchLaunch bl{};
    const dense::BatchKernelTable* kt = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // the eta sweeps' branch of the step graph
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_nodes = 0;
    int order = 0;                // block order: 0 instance-major, 1 largest first, 2 interleaved
    bool prim_valid = false;
    long long launches = 0;
    std::string err;
    // the persistent step (mode 1): its item list, the per-instance phase counts, the sync words
    // (ticket, abort, items done per instance and phase; then the error word, kept across steps)
    int mode = 0;                 // 0 one launch per phase, 1 one persistent launch per step
    int* items = nullptr;         // int4 entries
    size_t items_cap = 0;
    unsigned* need = nullptr;
    unsigned* sync = nullptr;
    dense::PersistLaunch pl{};
    int hold_instance = -1;       // failure injection: this instance's boundary phase never completes
};

namespace {

thread_local std::string g_err;

int bset(dense_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg; else g_err = msg;
    return code;
}
#define BCK(b, call)                                                                             \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return bset((b), DENSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

__global__ void kb_zero_slot(Params* tab, int n, int slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { tab[i].sc->maxeig[slot][0] = 0.0; tab[i].sc->maxeig[slot][1] = 0.0; }
}
__global__ void kb_set_bounds(Params* tab, int n, double t_end, long long total_step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { tab[i].sc->t_end = t_end; tab[i].sc->total_step = total_step; }
}
__global__ void kb_set_time(Scalars* sc, double t, long long step, double dt) {
    sc->t = t; sc->step = step; sc->dt = dt;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Block list of one phase: for every instance, its grid of gx x gy blocks.
void append_blocks(std::vector<int>& out, const std::vector<std::pair<int, int>>& grid, int order) {
    const int n = (int)grid.size();
    std::vector<int> inst(n);
    std::iota(inst.begin(), inst.end(), 0);
    if (order == 1)  // largest instance first: the long tails start early
        std::stable_sort(inst.begin(), inst.end(), [&](int a, int c) {
            return (long long)grid[a].first * grid[a].second > (long long)grid[c].first * grid[c].second;
        });
    if (order == 2) {  // round-robin over instances, one block of each in turn
        std::vector<long long> next(n, 0);
        bool more = true;
        while (more) {
            more = false;
            for (int i = 0; i < n; ++i) {
                const long long tot = (long long)grid[i].first * grid[i].second;
                if (next[i] < tot) {
                    const int k = (int)next[i]++;
                    out.push_back(i); out.push_back(k % grid[i].first); out.push_back(k / grid[i].first);
                    more = true;
                }
            }
        }
        return;
    }
    for (int i : inst)
        for (int by = 0; by < grid[i].second; ++by)
            for (int bx = 0; bx < grid[i].first; ++bx) { out.push_back(i); out.push_back(bx); out.push_back(by); }
}

int build_maps(dense_batch* b, int xi_variant, int eta_variant) {
    const int n = b->n;
    const int split = b->cfg[0].splitting;
    int xtx, xty, etx, ety;
    dense::batch_tile_shape(split, 0, xi_variant, &xtx, &xty);
    dense::batch_tile_shape(split, 1, eta_variant, &etx, &ety);
    std::vector<std::pair<int, int>> g_cells(n), g_bc(n), g_xi(n), g_eta(n);
    for (int i = 0; i < n; ++i) {
        const int ni = b->cfg[i].ni, nj = b->cfg[i].nj;
        g_cells[i] = {(ni + 31) / 32, (nj + 7) / 8};
        g_bc[i] = {(2 * ni + 2 * nj + 127) / 128, 1};
        g_xi[i] = {(ni + 1 + xtx - 1) / xtx, (nj + xty - 1) / xty};
        g_eta[i] = {(ni + etx - 1) / etx, (nj + 1 + ety - 1) / ety};
    }
    std::vector<int> all;
    size_t off[4];
    off[0] = 0; append_blocks(all, g_cells, b->order);
    off[1] = all.size(); append_blocks(all, g_bc, b->order);
    off[2] = all.size(); append_blocks(all, g_xi, b->order);
    off[3] = all.size(); append_blocks(all, g_eta, b->order);
    const size_t total = all.size();
    if (total > b->maps_cap) {
        if (b->maps) cudaFree(b->maps);
        b->maps = nullptr;
        BCK(b, cudaMalloc((void**)&b->maps, total * sizeof(int)));
        b->maps_cap = total;
    }
    BCK(b, cudaMemcpy(b->maps, all.data(), total * sizeof(int), cudaMemcpyHostToDevice));
    BatchLaunch& L = b->bl;
    L.tab = b->tab; L.n = n;
    L.map_cells = b->maps + off[0]; L.nb_cells = (int)((off[1] - off[0]) / 3);
    L.map_bc = b->maps + off[1];    L.nb_bc = (int)((off[2] - off[1]) / 3);
    L.map_xi = b->maps + off[2];    L.nb_xi = (int)((off[3] - off[2]) / 3);
    L.map_eta = b->maps + off[3];   L.nb_eta = (int)((total - off[3]) / 3);
    L.xi_variant = xi_variant; L.eta_variant = eta_variant;
    L.splitting = split; L.recon = b->cfg[0].recon;
    return DENSE_OK;
}

// The persistent step's item list in phase order (dense::PersistLaunch): per phase, the
// instances in the schedule's block order, each instance's items of that phase together (an
// instance's items of one phase finish close together, so its next phase can start early).
int build_items(dense_batch* b) {
    using namespace dense;
    const int n = b->n;
    int xtx, xty, etx, ety;
    batch_tile_shape(b->cfg[0].splitting, 0, b->bl.xi_variant, &xtx, &xty);
    batch_tile_shape(b->cfg[0].splitting, 1, b->bl.eta_variant, &etx, &ety);
    std::vector<int> inst(n);
    std::iota(inst.begin(), inst.end(), 0);
    if (b->order == 1)
        std::stable_sort(inst.begin(), inst.end(), [&](int a, int c) {
            return (long long)b->cfg[a].ni * b->cfg[a].nj > (long long)b->cfg[c].ni * b->cfg[c].nj;
        });
    std::vector<int> it;
    std::vector<unsigned> need((size_t)n * kPhases, 0u);
    auto push = [&](int kind, int stage, int phase, int dep, int i, int x, int y) {
        it.push_back(persist_code(kind, stage, phase, dep)); it.push_back(i); it.push_back(x); it.push_back(y);
        need[(size_t)i * kPhases + phase] += 1;
    };
    // one phase of every instance; blocks(i, emit) emits instance i's items of the phase
    auto phase_items = [&](auto&& blocks) {
        if (b->order != 2) {
            for (int i : inst) blocks(i, -1);
            return;
        }
        // round-robin: one item of each instance in turn
        std::vector<int> k(n, 0);
        for (bool more = true; more;) {
            more = false;
            for (int i = 0; i < n; ++i)
                if (blocks(i, k[i])) { ++k[i]; more = true; }
        }
    };
    // instance i's items of a phase as a list of (kind, x, y); with sel >= 0 only item sel
    // (returns whether it exists)
    auto emit = [&](int i, int sel, int kind, int stage, int phase, int dep,
                    const std::vector<std::array<int, 3>>& list) {
        if (sel < 0) {
            for (const auto& e : list) push(e[0], stage, phase, dep, i, e[1], e[2]);
            return true;
        }
        if (sel >= (int)list.size()) return false;
        push(list[sel][0], stage, phase, dep, i, list[sel][1], list[sel][2]);
        (void)kind;
        return true;
    };
    std::vector<std::vector<std::array<int, 3>>> bc(n), sw(n), up(n);
    for (int i = 0; i < n; ++i) {
        const int ni = b->cfg[i].ni, nj = b->cfg[i].nj;
        for (int x = 0; x < (2 * ni + 2 * nj + kPersistThreads - 1) / kPersistThreads; ++x) bc[i].push_back({kItemBc, x, 0});
        for (int y = 0; y < (nj + xty - 1) / xty; ++y)
            for (int x = 0; x < (ni + 1 + xtx - 1) / xtx; ++x) sw[i].push_back({kItemXi, x, y});
        for (int y = 0; y < (nj + 1 + ety - 1) / ety; ++y)
            for (int x = 0; x < (ni + etx - 1) / etx; ++x) sw[i].push_back({kItemEta, x, y});
        for (int y = 0; y < (nj + 7) / 8; ++y)
            for (int x = 0; x < (ni + 31) / 32; ++x) up[i].push_back({kItemUpdate, x, y});
    }
    const std::vector<std::array<int, 3>> one = {{0, 0, 0}};
    phase_items([&](int i, int sel) {
        return emit(i, sel, kItemBegin, 0, 0, -1, {{kItemBegin, 0, 0}});
    });
    for (int st = 1; st <= 3; ++st) {
        const int pb = 3 * st - 2, ps = 3 * st - 1, pu = 3 * st, prev = st == 1 ? 0 : 3 * st - 3;
        phase_items([&](int i, int sel) {
            if (st > 1 && b->prm[i].periodic_ghosts) return false;  // the previous update wrote the ghosts
            return emit(i, sel, kItemBc, st, pb, prev, bc[i]);
        });
        phase_items([&](int i, int sel) {
            const bool has_bc = st == 1 || !b->prm[i].periodic_ghosts;
            return emit(i, sel, kItemXi, st, ps, has_bc ? pb : prev, sw[i]);
        });
        phase_items([&](int i, int sel) { return emit(i, sel, kItemUpdate, st, pu, ps, up[i]); });
    }
    phase_items([&](int i, int sel) { return emit(i, sel, kItemEnd, 0, kPhases - 1, 9, {{kItemEnd, 0, 0}}); });
    (void)one;
    if (b->hold_instance >= 0 && b->hold_instance < n) need[(size_t)b->hold_instance * kPhases + 1] += 1;
    const size_t total = it.size();
    if (total > b->items_cap) {
        if (b->items) cudaFree(b->items);
        b->items = nullptr;
        BCK(b, cudaMalloc((void**)&b->items, total * sizeof(int)));
        b->items_cap = total;
    }
    BCK(b, cudaMemcpy(b->items, it.data(), total * sizeof(int), cudaMemcpyHostToDevice));
    if (!b->need) BCK(b, cudaMalloc((void**)&b->need, need.size() * sizeof(unsigned)));
    BCK(b, cudaMemcpy(b->need, need.data(), need.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
    if (!b->sync) {
        BCK(b, cudaMalloc((void**)&b->sync, (2 + need.size() + 1) * sizeof(unsigned)));
        BCK(b, cudaMemset(b->sync, 0, (2 + need.size() + 1) * sizeof(unsigned)));
    }
    PersistLaunch& L = b->pl;
    L.items = b->items;
    L.nitems = (int)(total / 4);
    L.sync = b->sync;
    L.need = b->need;
    L.err = b->sync + 2 + need.size();
    if (!L.spin_limit) L.spin_limit = 1ll << 22;
    if (!b->kt->persist_shape || !b->kt->persist_shape(b->bl, &L))
        return bset(b, DENSE_ERR_ARG, "no persistent launch for this scheme and variant");
    return DENSE_OK;
}

void drop_graph(dense_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

int ensure_prim(dense_batch* b) {
    if (b->prim_valid) return DENSE_OK;
    kb_zero_slot<<<(b->n + 127) / 128, 128, 0, b->stream>>>(b->tab, b->n, 0);
    b->kt->prim(b->bl, 0, b->stream);
    b->launches += 2;
    b->prim_valid = true;
    BCK(b, cudaGetLastError());
    return DENSE_OK;
}

int build_graph(dense_batch* b) {
    if (b->graph) return DENSE_OK;
    if (!b->side) {
        BCK(b, cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
        BCK(b, cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
        BCK(b, cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
    }
    cudaGraph_t g = nullptr;
    if (b->mode == 1) {
        // the persistent step: its sync words cleared, then the one launch
        BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaMemsetAsync(b->sync, 0, (2 + (size_t)b->n * dense::kPhases) * sizeof(unsigned), b->stream);
        if (ce == cudaSuccess) b->kt->persist(b->bl, b->pl, b->stream);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e == cudaSuccess && ce != cudaSuccess) {
            cudaGraphDestroy(g);
            e = ce;
        }
        if (e != cudaSuccess) return bset(b, DENSE_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bset(b, DENSE_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        b->graph_nodes = 1;
        return DENSE_OK;
    }
    BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    b->kt->step_begin(b->bl, b->stream);
    // per stage: boundary; the eta sweep as a branch beside the xi sweep (both read the stage
    // input, each writes its own face fluxes); the update after both
    // stages 2 and 3 need no boundary launch when every instance is periodic in x and y: the
    // previous stage's update wrote their ghost layers
    bool all_periodic = true;
    for (const Params& p : b->prm) all_periodic = all_periodic && p.periodic_ghosts;
    cudaError_t ce = cudaSuccess;
    for (int irk = 1; irk <= 3 && ce == cudaSuccess; ++irk) {
        if (irk == 1 || !all_periodic) b->kt->bc(b->bl, b->stream);
        ce = cudaEventRecord(b->ev_fork, b->stream);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->side, b->ev_fork, 0);
        if (ce != cudaSuccess) break;
        b->kt->flux(b->bl, irk, 1, b->side);
        b->kt->flux(b->bl, irk, 0, b->stream);
        ce = cudaEventRecord(b->ev_join, b->side);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->stream, b->ev_join, 0);
        if (ce != cudaSuccess) break;
        b->kt->update(b->bl, irk, b->stream);
    }
    b->kt->step_end(b->bl, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e == cudaSuccess && ce != cudaSuccess) {
        cudaGraphDestroy(g);
        e = ce;
    }
    if (e != cudaSuccess) return bset(b, DENSE_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bset(b, DENSE_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    b->graph_nodes = all_periodic ? 12 : 14;
    return DENSE_OK;
}

}  // namespace

extern "C" {

const char* dense_batch_last_error(dense_batch_t* b) { return b ? b->err.c_str() : g_err.c_str(); }

int dense_batch_create(int n, const dense_config_t* cfgs, dense_batch_t** out) {
    if (!out || !cfgs || n <= 0) return bset(nullptr, DENSE_ERR_ARG, "null argument or n <= 0");
    *out = nullptr;
    const dense_config_t& c0 = cfgs[0];
    for (int i = 0; i < n; ++i) {
        const dense_config_t& c = cfgs[i];
        if (c.ni < 3 || c.nj < 3 || c.bfsize != kB || c.neq != 4 || c.stages != 3 || c.dx <= 0.0 || c.dy <= 0.0)
            return bset(nullptr, DENSE_ERR_ARG, "instance " + std::to_string(i) + ": bad size, bfsize, neq, stages or dx/dy");
        if (c.splitting < DENSE_SPLIT_LLF || c.splitting > DENSE_SPLIT_SC)
            return bset(nullptr, DENSE_ERR_SPLITTING, "No such Selection (flux_splitting.f90:30-32)");
        if (c.strict < 0 || c.strict > 2)
            return bset(nullptr, DENSE_ERR_ARG, "instance " + std::to_string(i) + ": strict must be 0, 1 or 2");
        if (c.splitting != c0.splitting || c.recon != c0.recon || c.strict != c0.strict)
            return bset(nullptr, DENSE_ERR_ARG, "all instances of a batch share splitting, recon and strict");
        const int bm = c.benchmark;
        if (!(bm == 0 || (bm >= 1 && bm <= 9) || bm == DENSE_BENCH_IVC_PERIODIC || bm == DENSE_BENCH_RT_REFLECT ||
              bm == DENSE_BENCH_RM_PERIODIC))
            return bset(nullptr, DENSE_ERR_BENCHMARK, "No such Benchmark index! (boundary_general.f90:26-28)");
    }
    if (c0.splitting <= DENSE_SPLIT_SW && c0.recon != DENSE_RECON_UPWIND5 && c0.recon != DENSE_RECON_WENOJS5 &&
        c0.recon != DENSE_RECON_WENOZ5)
        return bset(nullptr, DENSE_ERR_ARG, "the batched form needs reconstruction 251, 253 or 255");
    auto* b = new dense_batch();
    b->n = n;
    b->cfg.assign(cfgs, cfgs + n);
    b->prm.resize(n);
    b->kt = dense::batch_kernels_for(c0.strict);
    auto fail = [&](int code, const std::string& m) { g_err = m; dense_batch_destroy(b); return code; };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(DENSE_ERR_CUDA, "cudaStreamCreate failed");
    // one pool: per instance cons(4) prim(5) cons0(4) planes, hx, he, xbot, xtop, yleft, Scalars
    std::vector<size_t> base(n);
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        const dense_config_t& c = cfgs[i];
        const size_t NIp = c.ni + 2 * kB, NJp = c.nj + 2 * kB, P = (NIp + 1) & ~(size_t)1;
        const size_t plane = NJp * P;
        base[i] = total;
        total += align256(plane * 13 * sizeof(double));
        total += align256((size_t)4 * c.nj * (c.ni + 1) * sizeof(double));
        total += align256((size_t)4 * (c.nj + 1) * c.ni * sizeof(double));
        total += align256((size_t)(2 * c.ni + c.nj) * sizeof(double));
        total += align256(sizeof(Scalars));
    }
    if (cudaMalloc((void**)&b->pool, total) != cudaSuccess) return fail(DENSE_ERR_NOMEM, "cudaMalloc of the batch pool failed");
    b->pool_bytes = total;
    if (cudaMemsetAsync(b->pool, 0, total, b->stream) != cudaSuccess) return fail(DENSE_ERR_CUDA, "cudaMemset failed");
    for (int i = 0; i < n; ++i) {
        const dense_config_t& c = cfgs[i];
        const int NIp = c.ni + 2 * kB, NJp = c.nj + 2 * kB, P = (NIp + 1) & ~1;
        const size_t plane = (size_t)NJp * P;
        char* q = b->pool + base[i];
        Params& p = b->prm[i];
        std::memset(&p, 0, sizeof(p));
        p.cons = (double*)q; p.prim = p.cons + 4 * plane; p.cons0 = p.prim + 5 * plane;
        q += align256(plane * 13 * sizeof(double));
        p.hx = (double*)q; q += align256((size_t)4 * c.nj * (c.ni + 1) * sizeof(double));
        p.he = (double*)q; q += align256((size_t)4 * (c.nj + 1) * c.ni * sizeof(double));
        p.xbot = (const double*)q; p.xtop = p.xbot + c.ni; p.yleft = p.xtop + c.ni;
        q += align256((size_t)(2 * c.ni + c.nj) * sizeof(double));
        p.sc = (Scalars*)q;
        p.ni = c.ni; p.nj = c.nj; p.P = P; p.plane = (long long)plane;
        p.gamma = c.gamma; p.cfl = c.cfl; p.delta = c.delta; p.dx = c.dx; p.dy = c.dy; p.dt_const = c.dt;
        p.theta_c = dense::theta_c_of(c.delta);
        p.if_const_dt = c.if_const_dt;
        p.bodyforce = c.if_bodyforce && (c.benchmark == DENSE_BENCH_RT || c.benchmark == DENSE_BENCH_RT_REFLECT);
        p.benchmark = c.benchmark; p.splitting = c.splitting; p.recon = c.recon;
        p.periodic_ghosts = dense::periodic_ghosts(c.benchmark, c.ni, c.nj);
    }
    if (cudaMalloc((void**)&b->tab, n * sizeof(Params)) != cudaSuccess) return fail(DENSE_ERR_NOMEM, "cudaMalloc failed");
    if (cudaMemcpy(b->tab, b->prm.data(), n * sizeof(Params), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(DENSE_ERR_CUDA, "cudaMemcpy failed");
    for (int i = 0; i < n; ++i) kb_set_time<<<1, 1, 0, b->stream>>>(b->prm[i].sc, 0.0, 0, cfgs[i].dt);
    int rc = build_maps(b, 0, 0);
    if (rc) { std::string m = b->err; return fail(rc, m); }
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(DENSE_ERR_CUDA, "initialisation failed");
    *out = b;
    return DENSE_OK;
}

void dense_batch_destroy(dense_batch_t* b) {
    if (!b) return;
    drop_graph(b);
    if (b->items) cudaFree(b->items);
    if (b->need) cudaFree(b->need);
    if (b->sync) cudaFree(b->sync);
    if (b->maps) cudaFree(b->maps);
    if (b->tab) cudaFree(b->tab);
    if (b->pool) cudaFree(b->pool);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int dense_batch_upload(dense_batch_t* b, int i, const double* cons, const double* prim, const double* x,
                       const double* y) {
    dense::NvtxRange nvtx_("dense_batch_upload");
    if (!b || !cons || i < 0 || i >= b->n) return bset(b, DENSE_ERR_ARG, "bad instance or null cons");
    const dense_config_t& c = b->cfg[i];
    const Params& p = b->prm[i];
    const int NIp = c.ni + 2 * kB, NJp = c.nj + 2 * kB;
    const size_t row = (size_t)NIp * sizeof(double), pitch = (size_t)p.P * sizeof(double);
    BCK(b, cudaMemcpy2DAsync(p.cons, pitch, cons, row, row, (size_t)NJp * 4, cudaMemcpyHostToDevice, b->stream));
    if (prim) BCK(b, cudaMemcpy2DAsync(p.prim, pitch, prim, row, row, (size_t)NJp * 5, cudaMemcpyHostToDevice, b->stream));
    else BCK(b, cudaMemsetAsync(p.prim, 0, (size_t)NJp * p.P * 5 * sizeof(double), b->stream));
    std::vector<double> rows(2 * c.ni + c.nj, 0.0);
    if (x) for (int k = 0; k < c.ni; ++k) { rows[k] = x[k]; rows[c.ni + k] = x[(size_t)c.ni * (c.nj - 1) + k]; }
    if (y) for (int k = 0; k < c.nj; ++k) rows[2 * c.ni + k] = y[(size_t)c.ni * k];
    BCK(b, cudaMemcpyAsync((void*)p.xbot, rows.data(), rows.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    b->prim_valid = false;
    return DENSE_OK;
}

int dense_batch_set_time(dense_batch_t* b, int i, double t, int step) {
    if (!b || i < 0 || i >= b->n) return bset(b, DENSE_ERR_ARG, "bad instance");
    kb_set_time<<<1, 1, 0, b->stream>>>(b->prm[i].sc, t, step, b->cfg[i].dt);
    BCK(b, cudaGetLastError());
    return DENSE_OK;
}

int dense_batch_steps_async(dense_batch_t* b, int nsteps, double t_end, int total_step) {
    dense::NvtxRange nvtx_("dense_batch_steps");
    if (!b || nsteps < 0) return bset(b, DENSE_ERR_ARG, "bad argument");
    int rc = ensure_prim(b);
    if (rc) return rc;
    rc = build_graph(b);
    if (rc) return rc;
    kb_set_bounds<<<(b->n + 127) / 128, 128, 0, b->stream>>>(b->tab, b->n, t_end, total_step);
    b->launches += 1;
    for (int s = 0; s < nsteps; ++s) {
        BCK(b, cudaGraphLaunch(b->graph, b->stream));
        b->launches += b->graph_nodes;
    }
    return DENSE_OK;
}

int dense_batch_steps(dense_batch_t* b, int nsteps, double t_end, int total_step) {
    int rc = dense_batch_steps_async(b, nsteps, t_end, total_step);
    if (rc) return rc;
    BCK(b, cudaStreamSynchronize(b->stream));
    if (b->mode == 1) {
        unsigned e = 0;
        BCK(b, cudaMemcpy(&e, b->pl.err, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (e) {
            BCK(b, cudaMemset(b->pl.err, 0, sizeof(unsigned)));
            return bset(b, DENSE_ERR_TIMEOUT,
                        "a wait of the persistent step gave up (DENSE_FLAG_TIMEOUT in the instances' status); the "
                        "step's results are not valid");
        }
    }
    return DENSE_OK;
}

int dense_batch_get_time(dense_batch_t* b, int i, double* t, int* step, double* dt) {
    if (!b || i < 0 || i >= b->n) return bset(b, DENSE_ERR_ARG, "bad instance");
    Scalars s{};
    BCK(b, cudaMemcpyAsync(&s, b->prm[i].sc, sizeof(Scalars), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    if (t) *t = s.t;
    if (step) *step = (int)s.step;
    if (dt) *dt = s.dt;
    return DENSE_OK;
}

int dense_batch_download(dense_batch_t* b, int i, double* cons, double* prim) {
    dense::NvtxRange nvtx_("dense_batch_download");
    if (!b || i < 0 || i >= b->n) return bset(b, DENSE_ERR_ARG, "bad instance");
    const dense_config_t& c = b->cfg[i];
    const Params& p = b->prm[i];
    const int NIp = c.ni + 2 * kB, NJp = c.nj + 2 * kB;
    const size_t row = (size_t)NIp * sizeof(double), pitch = (size_t)p.P * sizeof(double);
    if (cons) BCK(b, cudaMemcpy2DAsync(cons, row, p.cons, pitch, row, (size_t)NJp * 4, cudaMemcpyDeviceToHost, b->stream));
    if (prim) BCK(b, cudaMemcpy2DAsync(prim, row, p.prim, pitch, row, (size_t)NJp * 5, cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    if (prim) std::memset(prim + (size_t)5 * NIp * NJp, 0, (size_t)NIp * NJp * sizeof(double));
    return DENSE_OK;
}

int dense_batch_schedule_space(int* n_xi, int* n_eta, int* n_order) {
    if (n_xi) *n_xi = dense::kXiVariants;
    if (n_eta) *n_eta = dense::kEtaVariants;
    if (n_order) *n_order = dense::kOrders;
    return DENSE_OK;
}

int dense_batch_set_schedule(dense_batch_t* b, int xi_variant, int eta_variant, int order) {
    if (!b || xi_variant < 0 || xi_variant >= dense::kXiVariants || eta_variant < 0 ||
        eta_variant >= dense::kEtaVariants || order < 0 || order >= dense::kOrders)
        return bset(b, DENSE_ERR_ARG, "bad schedule");
    BCK(b, cudaStreamSynchronize(b->stream));
    b->order = order;
    int rc = build_maps(b, xi_variant, eta_variant);
    if (!rc && b->mode == 1) rc = build_items(b);
    if (rc) return rc;
    drop_graph(b);
    return DENSE_OK;
}

int dense_batch_set_launch_mode(dense_batch_t* b, int mode) {
    if (!b || (mode != 0 && mode != 1)) return bset(b, DENSE_ERR_ARG, "launch mode must be 0 or 1");
    if (mode == 1 && (!b->kt->persist || b->cfg[0].splitting > DENSE_SPLIT_SW))
        return bset(b, DENSE_ERR_ARG,
                    "the persistent step covers the component-wise schemes (101-103 with 251/253/255) of the "
                    "fast variant");
    BCK(b, cudaStreamSynchronize(b->stream));
    const int old = b->mode;
    b->mode = mode;
    if (mode == 1) {
        const int rc = build_items(b);
        if (rc) {
            b->mode = old;
            return rc;
        }
    }
    drop_graph(b);
    return DENSE_OK;
}

int dense_batch_get_launch_mode(dense_batch_t* b, int* mode) {
    if (!b || !mode) return bset(b, DENSE_ERR_ARG, "null argument");
    *mode = b->mode;
    return DENSE_OK;
}

int dense_batch_hold_instance(dense_batch_t* b, int instance, long long spin_limit) {
    if (!b || instance < -1 || instance >= b->n || spin_limit < 0)
        return bset(b, DENSE_ERR_ARG, "bad instance or spin limit");
    BCK(b, cudaStreamSynchronize(b->stream));
    b->hold_instance = instance;
    b->pl.spin_limit = spin_limit ? spin_limit : (1ll << 22);
    if (b->mode == 1) {
        const int rc = build_items(b);
        if (rc) return rc;
    }
    drop_graph(b);
    return DENSE_OK;
}

int dense_batch_get_stream(dense_batch_t* b, void** stream) {
    if (!b || !stream) return bset(b, DENSE_ERR_ARG, "null argument");
    *stream = (void*)b->stream;
    return DENSE_OK;
}

int dense_batch_status(dense_batch_t* b, unsigned* flags) {
    if (!b || !flags) return bset(b, DENSE_ERR_ARG, "null argument");
    unsigned f = 0;
    std::vector<unsigned> fl(b->n, 0u);
    for (int i = 0; i < b->n; ++i) {
        BCK(b, cudaMemcpyAsync(&fl[i], &b->prm[i].sc->status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
        BCK(b, cudaMemsetAsync(&b->prm[i].sc->status, 0, sizeof(unsigned), b->stream));
    }
    BCK(b, cudaStreamSynchronize(b->stream));
    for (unsigned fi : fl) f |= fi;
    *flags = f;
    return DENSE_OK;
}

long long dense_batch_launch_count(dense_batch_t* b) { return b ? b->launches : -1; }

long long dense_batch_cells(dense_batch_t* b) {
    if (!b) return -1;
    long long s = 0;
    for (const auto& c : b->cfg) s += (long long)c.ni * c.nj;
    return s;
}


// ---- device-side setups ---------------------------------------------------------------------
// One thread per interior cell of every instance (the 32 x 8 cell map), each instance's setup
// parameters (eps, xc, yc, amp) from `vars`.
__global__ void kb_init(const Params* tab, const int3* map, const double* vars) {
    __shared__ Params sp;
    const int3 m = map[blockIdx.x];
    if (threadIdx.x == 0 && threadIdx.y == 0) sp = tab[m.x];
    __syncthreads();
    const int i = m.y * blockDim.x + threadIdx.x, j = m.z * blockDim.y + threadIdx.y;
    const double* v = vars + 4 * m.x;
    if (i < sp.ni && j < sp.nj) dense::setups::init_cell(sp, v[0], v[1], v[2], v[3], i, j);
}

int dense_batch_init_device(dense_batch_t* b) {
    if (!b) return bset(b, DENSE_ERR_ARG, "null batch");
    std::vector<double> vars((size_t)4 * b->n);
    for (int i = 0; i < b->n; ++i) {
        const dense_config_t& c = b->cfg[i];
        if (c.benchmark != DENSE_BENCH_IVC_PERIODIC && c.benchmark != DENSE_BENCH_RT_REFLECT &&
            c.benchmark != DENSE_BENCH_RM_PERIODIC)
            return bset(b, DENSE_ERR_BENCHMARK, "device setups exist for benchmarks 11, 13 and 14");
        vars[4 * i] = c.var_eps; vars[4 * i + 1] = c.var_xc; vars[4 * i + 2] = c.var_yc; vars[4 * i + 3] = c.var_amp;
    }
    BCK(b, cudaMemsetAsync(b->pool, 0, b->pool_bytes, b->stream));
    double* dv = nullptr;
    BCK(b, cudaMallocAsync((void**)&dv, vars.size() * sizeof(double), b->stream));
    BCK(b, cudaMemcpyAsync(dv, vars.data(), vars.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    kb_init<<<b->bl.nb_cells, dim3(32, 8), 0, b->stream>>>(b->tab, (const int3*)b->bl.map_cells, dv);
    b->launches += 1;
    BCK(b, cudaGetLastError());
    BCK(b, cudaFreeAsync(dv, b->stream));
    for (int i = 0; i < b->n; ++i) {
        int rc = dense_batch_set_time(b, i, 0.0, 0);
        if (rc) return rc;
    }
    BCK(b, cudaStreamSynchronize(b->stream));  // vars is a host buffer
    b->prim_valid = false;
    return DENSE_OK;
}

// ---- device-resident states (the PyTorch form) ----------------------------------------------
static int batch_wait(dense_batch* b, void* caller, bool caller_waits) {
    cudaEvent_t e;
    BCK(b, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaStream_t from = caller_waits ? b->stream : (cudaStream_t)caller;
    cudaStream_t to = caller_waits ? (cudaStream_t)caller : b->stream;
    cudaError_t r = cudaEventRecord(e, from);
    if (r == cudaSuccess) r = cudaStreamWaitEvent(to, e, 0);
    cudaEventDestroy(e);
    if (r != cudaSuccess) return bset(b, DENSE_ERR_CUDA, std::string("stream order: ") + cudaGetErrorString(r));
    return DENSE_OK;
}

int dense_batch_upload_device(dense_batch_t* b, int i, const double* cons, const double* prim, void* stream) {
    if (!b || !cons || i < 0 || i >= b->n) return bset(b, DENSE_ERR_ARG, "bad instance or null cons");
    int rc = batch_wait(b, stream, false);
    if (rc) return rc;
    const dense_config_t& c = b->cfg[i];
    const Params& p = b->prm[i];
    const int NIp = c.ni + 2 * kB, NJp = c.nj + 2 * kB;
    const size_t row = (size_t)NIp * sizeof(double), pitch = (size_t)p.P * sizeof(double);
    BCK(b, cudaMemcpy2DAsync(p.cons, pitch, cons, row, row, (size_t)NJp * 4, cudaMemcpyDeviceToDevice, b->stream));
    if (prim) BCK(b, cudaMemcpy2DAsync(p.prim, pitch, prim, row, row, (size_t)NJp * 5, cudaMemcpyDeviceToDevice, b->stream));
    b->prim_valid = false;
    return batch_wait(b, stream, true);
}

int dense_batch_download_device(dense_batch_t* b, int i, double* cons, double* prim, void* stream) {
    if (!b || i < 0 || i >= b->n) return bset(b, DENSE_ERR_ARG, "bad instance");
    int rc = batch_wait(b, stream, false);
    if (rc) return rc;
    const dense_config_t& c = b->cfg[i];
    const Params& p = b->prm[i];
    const int NIp = c.ni + 2 * kB, NJp = c.nj + 2 * kB;
    const size_t row = (size_t)NIp * sizeof(double), pitch = (size_t)p.P * sizeof(double);
    if (cons) BCK(b, cudaMemcpy2DAsync(cons, row, p.cons, pitch, row, (size_t)NJp * 4, cudaMemcpyDeviceToDevice, b->stream));
    if (prim) BCK(b, cudaMemcpy2DAsync(prim, row, p.prim, pitch, row, (size_t)NJp * 5, cudaMemcpyDeviceToDevice, b->stream));
    return batch_wait(b, stream, true);
}

int dense_batch_steps_device(dense_batch_t* b, int nsteps, double t_end, int total_step, void* stream) {
    if (!b) return bset(b, DENSE_ERR_ARG, "null batch");
    int rc = batch_wait(b, stream, false);
    if (!rc) rc = dense_batch_steps_async(b, nsteps, t_end, total_step);
    if (rc) return rc;
    return batch_wait(b, stream, true);
}

}  // extern "C"
