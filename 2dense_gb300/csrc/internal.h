// internal.h — types shared by the kernels (kernels.cu, compiled once per arithmetic variant)
// and the C ABI layer (capi.cu). Not part of the public interface.
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/dense2d.h"

namespace dense {

constexpr int kB = 4;  // ghost layers per side: allocate_block(...,4,4,neq)

// Planes per direction of the adjoint tape (Params::tape): 40 stencil gradients (none for
// upwind5) and 4 fluxes.
constexpr int tape_planes(int recon) { return recon == DENSE_RECON_UPWIND5 ? 4 : 44; }

// Device-resident scalars of one block: the module globals of flow_general that the hot path
// reads and writes (max_eig_i/j, dt, current_time, current_step), plus the loop predicate.
struct Scalars {
    double maxeig[3][2];  // slot s = stage (0..2) that reads it: (max_eig_i, max_eig_j)
    double dt;            // flow_general::dt
    double dtdx, dtdy;    // dt/dx, dt/dy (time_advance_general.f90:49)
    double t;             // current_time
    double elasp;         // elasp_time
    double t_end;         // loop bound on time (general_main.f90:23)
    long long step;       // current_step
    long long total_step; // loop bound on steps
    int active;           // this step is taken (the while-condition held at its start)
    unsigned status;      // DENSE_FLAG_* bits
    int pad[2];
    // AdaWENO branch counts over (interface, sign) pairs while Params::count_branches is set,
    // per sweep direction d (xi 0, eta 1) at [4d + k]: k = 0 smooth branch, 1 characteristic
    // branch, 2 warps, 3 warps with a characteristic lane
    unsigned long long branch_count[8];
    // save predicate of the driver loop (dense_run, general_main.f90:40-41): with save_mode set,
    // a step after which step % save_step == 0 or elasp >= dt_save holds the following steps
    // (their while-condition fails) until the host has taken the save and clears `hold`
    int save_mode, hold;
    long long save_step;
    double dt_save;
};

// Everything a kernel needs, passed by value.
struct Params {
    double* cons;    // [4][NJp][P] padded conserved variables
    double* prim;    // [5][NJp][P] padded rho,u,v,p,alpha
    double* cons0;   // [4][NJp][P] stage-1 copy (cons_temp); interior is read
    double* hx;      // [4][nj][ni+1] interface fluxes h_xi
    double* he;      // [4][nj+1][ni] interface fluxes h_eta
    const double* xbot;   // x(i,1),  i=1..ni  (DMR bottom rule)
    const double* xtop;   // x(i,nj), i=1..ni  (DMR top rule)
    const double* yleft;  // y(1,j),  j=1..nj  (SSL inflow rule)
    Scalars* sc;
    int ni, nj;
    int P;           // row pitch of the padded arrays, in doubles
    long long plane; // doubles per variable plane = NJp * P
    double gamma, cfl, delta, dx, dy, dt_const;
    // AdaWENO switch theta > delta written without a divide (fast kernels): with
    // theta = 1/(1 + (sum alpha - 1)^2), N = (sum alpha) D and N - D = tau^2 Q >= 0 (common
    // denominator D), theta > delta <=> D > k (N - D) with k = sqrt(delta/(1-delta))
    // <=> D > theta_c N with theta_c = k/(1+k), for 0 <= delta < 1; theta_c = 0 for delta < 0
    // (always smooth), 1 for delta >= 1 (never smooth: N >= D)
    double theta_c;
    int if_const_dt, bodyforce, benchmark, splitting, recon;
    // periodic in x and y with at least 2 kB cells each way (benchmarks 11 and 14): the update
    // also writes each boundary cell's periodic images into the ghost layers, which is the whole
    // of the next stage's boundary fill (set by periodic_ghosts() below)
    int periodic_ghosts;
    int count_branches;  // accumulate Scalars::branch_count in the AdaWENO sweeps
    // Tape of the sweeps for the discrete adjoint (flux_tape launches only; for the characteristic
    // sweeps (104) only the fluxes, 4 planes a direction; for AdaWENO (105) the branches taken,
    // bit 0 "+" smooth and bit 1 "-" smooth, then the fluxes, 5 planes a direction). The
    // component-wise LLF/GLF/SW sweeps':
    // per direction tape_planes(recon) planes of the direction's face array (xi [nj][ni+1], eta
    // [nj+1][ni], eta after xi): the reconstructions' stencil gradients g[(s*5 + m)*4 + v] (s = 0
    // for F+, 1 for F-; none for upwind5, whose gradient is constant), then the fluxes h[v].
    double* tape;
    // AdaWENO indicator theta of every (interface, sign) of the last stage, when it is saved
    // (if_save_theta): xi [2][nj][ni+1], then eta [2][nj+1][ni] (sign 0 = "+"); else null
    double* theta;
};

// Params::theta_c of an AdaWENO threshold delta.
inline double theta_c_of(double delta) {
    if (delta < 0.0) return 0.0;
    if (delta >= 1.0) return 1.0;
    const double k = __builtin_sqrt(delta / (1.0 - delta));
    return k / (1.0 + k);
}

// Whether the update of a configuration writes the periodic ghost images (Params::periodic_ghosts).
inline int periodic_ghosts(int benchmark, int ni, int nj) {
    return (benchmark == DENSE_BENCH_IVC_PERIODIC || benchmark == DENSE_BENCH_RM_PERIODIC) &&
           ni >= 2 * kB && nj >= 2 * kB;
}

// One arithmetic variant of the kernels (fast or strict), as a table of launchers.
struct KernelTable {
    const char* name;
    // get_primary over the interior; max wave speeds into slot `slot`
    void (*prim)(const Params&, int slot, void* stream);
    // boundary_general
    void (*bc)(const Params&, void* stream);
    // flux_splitting_general (+ scheme_invis_general) in one direction: dir 0 writes hx (and
    // computes dt on stage 1, dt/dx, dt/dy, and zeroes the next max slot), dir 1 writes he.
    void (*flux)(const Params&, int irk, int dir, void* stream);
    // time_rk3_general(irk) fused with get_primary of the new state
    void (*update)(const Params&, int irk, void* stream);
    // loop bookkeeping: step_begin evaluates the while-condition, step_end advances time
    void (*step_begin)(const Params&, void* stream);
    void (*step_end)(const Params&, void* stream);
    // kernel launches issued by flux(dir) for this configuration
    int (*flux_launches)(const Params&, int dir);
    // flux(dir) of the component-wise LLF/GLF/Steger-Warming sweeps with reconstruction
    // 251/253/255 that also writes Params::tape; identical fluxes and state updates
    void (*flux_tape)(const Params&, int irk, int dir, void* stream);
};

const KernelTable* kernels_fast();
const KernelTable* kernels_strict();
const KernelTable* kernels_checked();
// the kernel table of a configuration's variant (dense_config_t::strict: 0 fast, 1 strict,
// 2 checked)
inline const KernelTable* kernels_for(int strict) {
    return strict == 1 ? kernels_strict() : strict == 2 ? kernels_checked() : kernels_fast();
}

// The error text that dense_last_error(NULL) returns, for entry points without a handle that
// live outside capi.cu (the allocation-free stage); the calling thread's own copy.
void set_last_error(const char* msg);

// ---- batched form: many independent blocks of uneven size advanced by one launch per phase
struct int3_ { int x, y, z; };  // host mirror of CUDA's int3 (instance, block x, block y)

// Tile shapes (threads x, threads y) the batched flux sweeps can run with; an autotuner picks
// one per direction. Variant 0 is the single-instance shape.
constexpr int kXiVariants = 4, kEtaVariants = 5, kOrders = 3;
void batch_tile_shape(int splitting, int dir, int variant, int* tx, int* ty);

struct BatchLaunch {
    const Params* tab;  // device array: one Params per instance
    int n;              // instances
    const void* map_cells; int nb_cells;  // 32 x 8 blocks over each instance's interior cells
    const void* map_bc;    int nb_bc;     // 128-thread blocks over each instance's ghost lines
    const void* map_xi;    int nb_xi;     // xi-sweep tiles
    const void* map_eta;   int nb_eta;    // eta-sweep tiles
    int xi_variant, eta_variant;
    int splitting, recon;  // common to the batch
};

// The persistent step of a batch (component-wise schemes, fast variant): one launch of resident
// blocks of kPersistThreads threads works through a list of items, each a piece of one phase of
// one instance. Phases of an instance, in order: 0 the loop predicate; per stage s = 1..3 the
// boundary lines (3s - 2), the xi and eta tiles (3s - 1) and the update's cell blocks (3s); 10
// the time advance. An item waits until every item of one earlier phase of its own instance
// (its dependency) has finished.
constexpr int kPersistThreads = 256;
constexpr int kPhases = 11;
enum PersistKind { kItemBegin = 0, kItemBc = 1, kItemXi = 2, kItemEta = 3, kItemUpdate = 4, kItemEnd = 5 };
// item (x, y, z, w): x = kind | stage << 4 | phase << 8 | (dependency phase + 1) << 16, y the
// instance, (z, w) the block coordinates within the instance (tile, boundary-line block of
// kPersistThreads lines, or cell block of 32 x 8)
inline int persist_code(int kind, int stage, int phase, int dep) {
    return kind | stage << 4 | phase << 8 | (dep + 1) << 16;
}
struct PersistLaunch {
    const void* items; int nitems;   // int4 items in list order
    unsigned* sync;                  // [0] ticket, [1] abort word, [2 + kPhases i + ph] items done
    const unsigned* need;            // [kPhases i + ph]: items of phase ph of instance i
    unsigned* err;                   // set by a wait that gave up; kept across steps
    long long spin_limit;            // polls before a wait gives up (DENSE_FLAG_TIMEOUT)
    int grid;                        // resident blocks
    size_t smem;                     // dynamic shared memory per block
};

struct BatchKernelTable {
    void (*prim)(const BatchLaunch&, int slot, void* stream);
    void (*bc)(const BatchLaunch&, void* stream);
    void (*flux)(const BatchLaunch&, int irk, int dir, void* stream);
    void (*update)(const BatchLaunch&, int irk, void* stream);
    void (*step_begin)(const BatchLaunch&, void* stream);
    void (*step_end)(const BatchLaunch&, void* stream);
    // the persistent step (null where the variant has none); persist_shape fills the launch's
    // grid and shared memory for the batch's scheme and tiles, false if it has none
    void (*persist)(const BatchLaunch&, const PersistLaunch&, void* stream);
    bool (*persist_shape)(const BatchLaunch&, PersistLaunch*);
};
const BatchKernelTable* batch_kernels_fast();
const BatchKernelTable* batch_kernels_strict();
const BatchKernelTable* batch_kernels_checked();
inline const BatchKernelTable* batch_kernels_for(int strict) {
    return strict == 1 ? batch_kernels_strict() : strict == 2 ? batch_kernels_checked() : batch_kernels_fast();
}

}  // namespace dense
