/*
 * dense2d.h — C ABI of the GB300 (sm_103a) implementation of 2DENSE's per-stage hot path:
 * primitive recovery, boundary (ghost) fill, flux-vector splitting, WENO reconstruction and
 * the TVD-RK3 stage update.
 *
 * The reference has no FFI. Its seam is the four argument-less subroutines that the Fortran
 * driver calls once per Runge-Kutta stage (source/utility/general_main.f90:27-30):
 *     call get_primary; call boundary_general; call flux_splitting_general; call time_rk3_general(irk)
 * and the module globals they share (source/utility/flow_mod_general.f90:47-183).
 * dense_stage() replaces those four calls; dense_steps() replaces the whole stage loop of
 * general_main.f90:23-38. Each declaration below names the reference code it stands in for.
 *
 * Conventions
 *  - Every entry point returns an int status (DENSE_OK == 0) and never exits the process;
 *    the reference instead prints and stops (flux_splitting.f90:30-32, boundary_general.f90:26-28).
 *  - Host arrays use the reference's Fortran layout: column-major, i fastest, padded with
 *    `bfsize` ghost layers on every side: cons(ni+2b, nj+2b, 4), prim(ni+2b, nj+2b, 6),
 *    x(ni, nj), y(ni, nj) (source/utility/flow_mod_general.f90:205-206,251-252).
 *  - Host arrays stay owned by the caller; the handle owns its device buffers and stream.
 *    One handle per host thread; calls are ordered on the handle's stream.
 *  - All arithmetic is IEEE binary64.
 */
#ifndef DENSE2D_H
#define DENSE2D_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define DENSE_OK              0
#define DENSE_ERR_ARG         1  /* null pointer, bad size or bad index argument              */
#define DENSE_ERR_SPLITTING   2  /* unknown scheme_splitting_index (flux_splitting.f90:30-32) */
#define DENSE_ERR_BENCHMARK   3  /* unknown benchmark_index (boundary_general.f90:26-28,
                                    init_general.f90:34-36)                                  */
#define DENSE_ERR_CUDA        4  /* a CUDA runtime call failed; see dense_last_error()        */
#define DENSE_ERR_NUMERIC     5  /* the device status word holds a numeric fault flag         */
#define DENSE_ERR_TIMEOUT     6  /* a bounded device-side wait gave up                        */
#define DENSE_ERR_IO          7  /* file could not be opened, read or written                 */
#define DENSE_ERR_STATE       8  /* call out of order, e.g. dense_stage() before dense_upload() */
#define DENSE_ERR_NOMEM       9  /* device allocation failed                                  */
#define DENSE_ERR_LIMIT      10  /* a size exceeds a documented maximum                       */

/* ---- device status-word bits (dense_status) -------------------------------------------- */
#define DENSE_FLAG_NAN          0x01u /* a NaN appeared in the updated state                 */
#define DENSE_FLAG_NEG_RHO      0x02u /* density <= 0 in an updated cell                      */
#define DENSE_FLAG_P_FLOOR      0x04u /* the p<0 -> 1.0e-6 floor fired (get_primary.f90:57-59) */
#define DENSE_FLAG_ROE_IMAG     0x08u /* Roe sound speed squared < 0 (sqrt of a negative)    */
#define DENSE_FLAG_RECON_NOOP   0x10u /* unknown scheme_inv_index: h stays zero, as in the
                                         reference's silent no-op (scheme_invs_general.f90:4-27) */
#define DENSE_FLAG_TIMEOUT      0x20u /* a bounded device wait gave up                        */
#define DENSE_FLAG_BOUNDS       0x40u /* checked variant (strict = 2): an array index fell outside
                                         its array; it was clamped, not dereferenced            */

/* ---- scheme and benchmark indices (the reference's namelist values) --------------------- */
#define DENSE_SPLIT_LLF   101  /* local Lax-Friedrichs       flux_splitting_LLF.f90:13-77    */
#define DENSE_SPLIT_GLF   102  /* global Lax-Friedrichs      flux_splitting_GLF.f90:13-70    */
#define DENSE_SPLIT_SW    103  /* Steger-Warming             flux_splitting_SW.f90:14-168    */
#define DENSE_SPLIT_CH    104  /* characteristic WENO-Z, Roe + GLF  flux_splitting_CH.f90   */
#define DENSE_SPLIT_SC    105  /* AdaWENO (adaptive characteristic) flux_splitting_SC.f90   */
#define DENSE_RECON_UPWIND5  251 /* scheme_upwind5_general.f90 */
#define DENSE_RECON_WENOJS5  253 /* scheme_weno5js_general.f90 */
#define DENSE_RECON_WENOZ5   255 /* scheme_weno5z_general.f90  */

#define DENSE_BENCH_USER          0  /* nothing initialised, no ghost fill (init_general.f90:32-33) */
#define DENSE_BENCH_IVC           1  /* isentropic vortex, reference setup                        */
#define DENSE_BENCH_SEDOV         2
#define DENSE_BENCH_RT            3  /* Rayleigh-Taylor, periodic sides, body force               */
#define DENSE_BENCH_RM            4  /* Richtmyer-Meshkov                                         */
#define DENSE_BENCH_DMR           5  /* double Mach reflection                                    */
#define DENSE_BENCH_SSL           6  /* shock / shear layer                                       */
#define DENSE_BENCH_SHOCKVORTEX   9
/* Variants that the reference does not ship (its commented-out code paths and the published
 * test problems' standard forms). They keep the reference's formulas where it has them. */
#define DENSE_BENCH_IVC_PERIODIC 11  /* translating vortex: freestream (1,1,1,1), strength var_eps,
                                        centre (var_xc,var_yc), periodic in x and y             */
#define DENSE_BENCH_RT_REFLECT   13  /* RT with reflective side walls (boundary_rt_general.f90:59-127,
                                        commented out in the reference)                         */
#define DENSE_BENCH_RM_PERIODIC  14  /* Mach 1.2 shock into a density-3 sinusoidal interface of
                                        amplitude var_amp, periodic in x and y                   */

/* ---- configuration: the six namelists of input.in (flow_mod_general.f90:50-179) ---------- */
typedef struct dense_config_t {
    /* grid_pars */
    int ni, nj;               /* single_ni, single_nj                                       */
    int bfsize;               /* ghost layers per side; the reference always uses 4          */
    int neq;                  /* number of equations, 4                                      */
    /* model_pars */
    int benchmark;            /* benchmark_index                                             */
    int if_bodyforce, if_source, if_viscous;
    /* scheme_pars */
    int splitting;            /* scheme_splitting_index                                      */
    int recon;                /* scheme_inv_index                                            */
    double delta;             /* AdaWENO switch threshold on theta                           */
    /* time_step_pars */
    int stages;               /* 3                                                           */
    int if_const_dt;
    double cfl, dt;
    double total_time, dt_save;
    int total_step, save_step;
    int if_save_binary, if_save_tec, if_save_theta;
    /* gas_pars */
    double gamma;
    /* block geometry, written by dense_init_setup() (init_*_general.f90) */
    double dx, dy;
    /* parameters of the variant benchmarks 11, 13, 14 */
    double var_eps, var_xc, var_yc, var_amp;
    /* remaining namelist entries, carried so an input.in round-trips */
    int omp_thread_num, if_curve_grid, if_read_from_file, scheme_vis_index;
    double mach_inf, reynolds;
    /* kernel variant: 0 = fast (FMA contraction and algebraic rewrites, agrees with the
       reference to <= 1e-12 relative after one step); 1 = strict (the reference's evaluation
       order, no FMA contraction, IEEE divide and sqrt: bit-identical on the reference's
       x86-64 arithmetic except where a boundary rule calls a transcendental function);
       2 = checked (debug build of the fast variant: the same results, with every array index
       checked against its array; a bad one sets DENSE_FLAG_BOUNDS) */
    int strict;
    int reserved[7];
} dense_config_t;

typedef struct dense_handle dense_handle_t;

/* ---- configuration and initial setup (host side, one-time) ----------------------------- */

/* Module defaults of flow_mod_general.f90:50-179 (e.g. splitting 101, recon 201, cfl 0.5). */
int dense_config_default(dense_config_t* cfg);

/* read_par_namelist (flow_mod_general.f90:297-334): parse the six namelists of an input.in.
   Entries absent from the file keep the values already in *cfg. */
int dense_read_namelist(const char* path, dense_config_t* cfg);

/* init_general (init_general.f90:13-37): fill the interior of cons and prim and the cell
   centres x, y for cfg->benchmark; set cfg->dx, cfg->dy (and, for Rayleigh-Taylor, gamma=5/3
   and if_bodyforce=1 as init_RT_general.f90:9-10 does). Ghost cells are zeroed, like
   allocate_block (flow_mod_general.f90:207-208), except where the setup writes them. */
int dense_init_setup(dense_config_t* cfg, double* cons, double* prim, double* x, double* y);
/* the configuration part of dense_init_setup alone: cfg->dx, cfg->dy (and gamma, if_bodyforce
   for Rayleigh-Taylor), without building any array */
int dense_setup_config(dense_config_t* cfg);

/* Bytes of the host arrays for cfg: cons, prim, x (== y). */
int dense_array_sizes(const dense_config_t* cfg, long long* cons_count, long long* prim_count,
                      long long* xy_count);

/* ---- solver handle --------------------------------------------------------------------- */

/* allocate_block (flow_mod_general.f90:190-295) on the device: state, stage copy, interface
   fluxes, scratch. Picks device 0 unless CUDA_VISIBLE_DEVICES says otherwise. */
int dense_create(const dense_config_t* cfg, dense_handle_t** out);

/* Copy the caller's state to the device (block_grid(1)%cons / %prim / %x / %y). prim may be
   NULL: interior primitives are then recomputed on the device (get_primary) and ghost
   primitives are zero. x and y are needed only by boundary rules that read them
   (DMR, SSL); they may be NULL otherwise. */
int dense_upload(dense_handle_t* h, const double* cons, const double* prim,
                 const double* x, const double* y);

/* One Runge-Kutta stage: get_primary -> boundary_general -> flux_splitting_general ->
   time_rk3_general(irk) (general_main.f90:27-30). current_time is the driver's time at the
   start of the step (boundary rules read it). On irk == 1 without if_const_dt the CFL time
   step is computed on the device (time_advance_general.f90:20-24) and returned in *dt_inout;
   otherwise *dt_inout is the dt used. Synchronises the stream to return dt. */
int dense_stage(dense_handle_t* h, int irk, double current_time, double* dt_inout);

/* The device-resident step loop of general_main.f90:23-38: up to nsteps steps of `stages`
   stages, each taken only while (*t_inout < t_end && *step_inout < total_step), advancing
   time and step on the device; no host synchronisation between steps. On return *t_inout,
   *step_inout and *dt_out hold the driver's current_time, current_step and dt. One CUDA graph
   runs a step; for AdaWENO (105) grids of 200,000 cells or more its kernel-to-kernel edges are
   programmatic (each kernel scheduled as the one before it drains), which the environment
   variable DENSE_PDL=0 or 1 turns off or on for every grid. Results are the same either way. */
int dense_steps(dense_handle_t* h, int nsteps, double t_end, int total_step,
                double* t_inout, int* step_inout, double* dt_out);

/* Copy the state back (Fortran layout). prim may be NULL; when given, the interior is
   recomputed exactly as get_primary does (rho,u,v,p,alpha and entropy log(p)-log(rho)) and
   the ghosts hold what the last boundary fill wrote. */
int dense_download(dense_handle_t* h, double* cons, double* prim);

/* max_eig_i / max_eig_j of the most recent get_primary (get_primary.f90:69-73). */
int dense_get_max_eig(dense_handle_t* h, double* max_eig_i, double* max_eig_j);

/* The namelist re-read at every save (general_main.f90:53) changes gamma, cfl, dt, flags
   and scheme indices mid-run; apply such a change to a live handle. Grid sizes and the
   benchmark must not change (DENSE_ERR_ARG). */
int dense_reconfigure(dense_handle_t* h, const dense_config_t* cfg);

/* Read (and clear) the device status word: DENSE_FLAG_* bits. Synchronises. */
int dense_status(dense_handle_t* h, unsigned* flags);

/* Text of the last error on this handle (or of the last handle-less call when h is NULL). */
const char* dense_last_error(dense_handle_t* h);

void dense_destroy(dense_handle_t* h);

/* ---- inspection (tests and tooling) ---------------------------------------------------- */

/* Interface fluxes of the last stage, in the reference's layout:
   h_xi(ni+1, nj, 4) and h_eta(nj+1, ni, 4) (flow_mod_general.f90:236-237). */
int dense_get_fluxes(dense_handle_t* h, double* h_xi, double* h_eta);

/* Number of kernel launches this handle has issued (including those inside CUDA graphs,
   counted once per graph launch per node). */
long long dense_launch_count(dense_handle_t* h);

/* ---- asynchronous loop and timing (callers that own the clock: benchmarks, PyTorch) ---- */

/* The handle's CUDA stream (cudaStream_t), so a caller can order its own work and events. */
int dense_get_stream(dense_handle_t* h, void** stream);

/* dense_steps without host synchronisation: continue from the device-resident time and step
   (set by dense_set_time or a previous dense_steps) and enqueue nsteps step graphs. */
int dense_steps_async(dense_handle_t* h, int nsteps, double t_end, int total_step);

/* Set / read the device-resident current_time and current_step (dense_get_time syncs). */
int dense_set_time(dense_handle_t* h, double t, int step);
int dense_get_time(dense_handle_t* h, double* t, int* step, double* dt);

/* Wait for all work on the handle's stream. */
int dense_sync(dense_handle_t* h);

/* ---- save path: the driver loop's files (general_main.f90:40-60) ------------------------- */

/* write_tec_at_time_cartisian (output_test_general.f90:18-59): Tecplot ASCII of the current
   state at `path` -- title and variables lines, one zone of (ni+1) x (nj+1) vertices
   (vet_x, vet_y as the setups define them), then prim(:,:,1..6) of the interior, cell-centred,
   one value per line with 17 significant digits. Like the reference, the header names seven
   variables and six primitive blocks follow (prim_lastvar_index = 6, var_index.f90:11). */
int dense_write_tecplot(dense_handle_t* h, const char* path);
/* write_theta_at_time_cartisian (output_test_general.f90:61-119): the AdaWENO indicators of
   the last stage per cell (the larger of its two faces' theta) for xi +/- and eta +/-, as
   Tecplot ASCII; zeros unless the splitting is 105 and cfg.if_save_theta is set (the sweeps
   record theta only then). */
int dense_write_theta(dense_handle_t* h, const char* path);
/* theta of every (interface, sign) of the last stage: xi [2][nj][ni+1] then eta [2][nj+1][ni]
   (sign 0 = "+"); DENSE_ERR_STATE unless the splitting is 105 and cfg.if_save_theta is set */
int dense_get_theta(dense_handle_t* h, double* theta);
/* write_date_binary (read_WriteAndLoad.f90:1-26): the unformatted checkpoint, gfortran
   sequential records (4-byte lengths around each): (step int32, time), num_block = 1,
   index = 1, (ni, nj), (bfsize_i, bfsize_j), cons(NIp,NJp,4), x(ni,nj), y(ni,nj), (dx, dy). */
int dense_write_binary(dense_handle_t* h, const char* path);
/* load_date_binary (read_WriteAndLoad.f90:28-70): read such a checkpoint; sets cfg->ni, nj,
   bfsize, dx, dy and fills cons(NIp,NJp,4), x, y (each may be NULL; size them after a first
   call with NULL arrays), *step and *time. */
int dense_read_binary(const char* path, dense_config_t* cfg, double* cons, double* x, double* y,
                      int* step, double* time);
/* The loop of general_main.f90:23-60 on the device: steps while current_time < total_time and
   current_step < total_step; after every step with MOD(current_step, save_step) == 0 or
   elasp_time >= dt_save it writes 2d_<step>.dat2d (if_save_binary) and 2d_<step>.dat
   (if_save_tec, which also resets elasp_time; and 2d_theta_<step>.dat if if_save_theta) into
   `dir`, then reads `namelist_path` again (if not NULL) and applies it (dense_reconfigure); at
   the end it writes the final 2d_<step>.dat (and 2d_theta_<step>.dat). The saves are formatted and written by a host thread from a device snapshot
   while the device runs on. *saves counts them (may be NULL). At the end it appends the
   reference's timing log to `dir`/CpuTime.dat (general_main.f90:20,56-58): the wall time of the
   step loop without the saves, the step count, and their ratio. */
int dense_run(dense_handle_t* h, const char* dir, const char* namelist_path, int* saves);

/* Cell x(ni,nj), y(ni,nj) and vertex vet_x(ni+1,nj+1), vet_y coordinates of cfg's benchmark as
   the setups define them (any pointer may be NULL). */
int dense_grid_coords(const dense_config_t* cfg, double* x, double* y, double* vx, double* vy);

/* ---- device-side setups and error norms: no counterpart in the reference ------------------ */

/* The initial state of the handle's benchmark computed on the device (benchmarks 11, 13 and 14,
   the variants that workloads generate in bulk; cfg as dense_setup_config leaves it), time and
   step set to 0. Same formulas as dense_init_setup with CUDA's pow/exp/cos/sqrt: within a few
   ulp of the host setup, not bit-identical to it. */
int dense_init_device(dense_handle_t* h);
/* Translating vortex (11): mean and max over the interior of |rho - rho_exact| at the handle's
   current time, rho_exact the initial vortex moved by (t, t) on the periodic square (syncs). */
int dense_vortex_error(dense_handle_t* h, double* l1, double* linf);

/* ---- device-resident state (the PyTorch form): no counterpart in the reference ---------- */

/* Device arrays in the layout of dense_upload's host arrays: cons[4][NJp][NIp] (Fortran
   cons(NIp,NJp,4)), prim[5][NJp][NIp] (rho, u, v, p, alpha; may be NULL: get_primary of cons).
   `stream` is the caller's cudaStream_t (0 for the default stream): each call starts after the
   work already queued there and makes it wait for the call's own work; none blocks the host. */
int dense_upload_device(dense_handle_t* h, const double* cons, const double* prim, void* stream);
int dense_download_device(dense_handle_t* h, double* cons, double* prim, void* stream);
/* rhs[4][nj][ni] = L(u) of the current state, -(h_xi(i+1)-h_xi(i))/dx - (h_eta(j+1)-h_eta(j))/dy,
   the operator one stage applies (boundary fill and both sweeps of stage `irk`; the state is
   left unchanged) */
int dense_rhs_device(dense_handle_t* h, int irk, double* rhs, void* stream);
/* one stage (dense_stage) on the uploaded state; cons0[4][NJp][NIp] is the step's initial state
   (needed by stages 2 and 3, NULL for stage 1); *dt (a device double) receives the CFL time step
   of stage 1 and gives dt to stages 2 and 3 and to constant-dt runs */
int dense_stage_device(dense_handle_t* h, int irk, const double* cons0, double* dt, double current_time,
                       void* stream);
/* nsteps step graphs as dense_steps_async, ordered on the caller's stream */
int dense_steps_device(dense_handle_t* h, int nsteps, double t_end, int total_step, void* stream);

/* Run one stage with CUDA events between its kernels; ms[0..3] = boundary fill, xi flux,
   eta flux, update (+ get_primary). Advances the state like dense_stage. */
int dense_profile_stage(dense_handle_t* h, int irk, float* ms);

/* Branch mix of the AdaWENO sweeps (scheme 105), for counting the algorithmic work of the
   steps actually run: while enabled, the sweeps of direction d (xi 0, eta 1) add to counts8[4d+k]:
   k = 0 (interface, sign) pairs that took the smooth branch, 1 pairs that took the characteristic
   branch, 2 warps, 3 warps with at least one characteristic lane. Enabling or disabling zeroes
   the counters. */
int dense_count_branches(dense_handle_t* h, int enable);
int dense_get_branch_counts(dense_handle_t* h, unsigned long long* counts8);

/* Throughput probe of the FP64 pipe on the current device: kind 0 = FMA (FLOP/s, one FMA
   counted as two), kind 1 = IEEE double divides per second. */
int dense_measure_fp64(int kind, double* result);

/* Accuracy check of the fast kernels' Newton-refined reciprocal and inverse square root:
   out[4k..4k+3] = (fast 1/x[k], IEEE 1/x[k], fast 1/sqrt(x[k]), IEEE 1/sqrt(x[k])). */
int dense_fastmath_check(const double* x, double* out, int n);

/* ---- batched form: many independent blocks of uneven size in one launch per phase ------- */

/* The reference advances one block per process (num_block = 1, init_*_general.f90); the batched
   form runs n independent blocks -- each its own dense_config_t (grid size, benchmark, gamma,
   cfl) with its own CFL time step, time and step count -- through one launch per phase and one
   CUDA graph per step. All instances share splitting, recon and strict. Each instance's results
   are bit-identical to a plain dense_create/dense_steps solve of the same configuration. */
typedef struct dense_batch dense_batch_t;
int dense_batch_create(int n, const dense_config_t* cfgs, dense_batch_t** out);
void dense_batch_destroy(dense_batch_t* b);
/* instance i's state in the layout of dense_upload / dense_download */
int dense_batch_upload(dense_batch_t* b, int i, const double* cons, const double* prim,
                       const double* x, const double* y);
int dense_batch_download(dense_batch_t* b, int i, double* cons, double* prim);
int dense_batch_set_time(dense_batch_t* b, int i, double t, int step);
int dense_batch_get_time(dense_batch_t* b, int i, double* t, int* step, double* dt);
/* up to nsteps steps of every instance, each while its t < t_end and step < total_step;
   the _async form does not wait */
int dense_batch_steps(dense_batch_t* b, int nsteps, double t_end, int total_step);
int dense_batch_steps_async(dense_batch_t* b, int nsteps, double t_end, int total_step);
/* launch schedule (picked by the autotuner): tile shape variants of the component-wise xi and
   eta sweeps and the block order (0 instance-major, 1 largest instance first, 2 round-robin);
   the characteristic sweeps (104, 105) keep their one shape. Variant 0 is the single-instance
   tile: xi (32,4) (64,2) (32,8) (32,2); eta (8,32) (8,16) (32,8) (16,16) (4,64) threads. */
int dense_batch_set_schedule(dense_batch_t* b, int xi_variant, int eta_variant, int order);
/* the number of xi variants, eta variants and block orders dense_batch_set_schedule accepts */
int dense_batch_schedule_space(int* n_xi, int* n_eta, int* n_order);
/* How a step is launched. Mode 0 (the default): one launch per phase (boundary, xi sweep, eta
   sweep, update per stage) over every instance, a CUDA graph per step. Mode 1: one persistent
   launch per step (captured in the step's CUDA graph) of resident 256-thread blocks that take the
   step's pieces -- per instance its loop predicate, boundary lines, sweep tiles (the schedule's
   tiles with threads per interface added to make 256) and update blocks per stage, and its time
   advance -- in list order, each piece waiting only for the phase before it of its own instance,
   so an instance's next stage overlaps other instances' sweeps. Results are bit-identical to
   mode 0. Every wait is bounded; one that gives up sets DENSE_FLAG_TIMEOUT, the step's results
   are not valid and dense_batch_steps returns DENSE_ERR_TIMEOUT. Mode 1 covers the
   component-wise schemes (101-103 with 251/253/255) of the fast variant (strict = 0); anything
   else returns DENSE_ERR_ARG. */
int dense_batch_set_launch_mode(dense_batch_t* b, int mode);
int dense_batch_get_launch_mode(dense_batch_t* b, int* mode);
/* Failure injection for tests of the persistent step's bounded waits: the boundary phase of
   stage 1 of `instance` is given one piece more than it has, so the pieces that wait for it give
   up after spin_limit polls (0: the default limit of 2^22). instance = -1 removes the hold. */
int dense_batch_hold_instance(dense_batch_t* b, int instance, long long spin_limit);
int dense_batch_get_stream(dense_batch_t* b, void** stream);
/* Read (and clear) every instance's device status word: DENSE_FLAG_* bits, OR-ed. Synchronises. */
int dense_batch_status(dense_batch_t* b, unsigned* flags);
long long dense_batch_launch_count(dense_batch_t* b);
long long dense_batch_cells(dense_batch_t* b);
const char* dense_batch_last_error(dense_batch_t* b);
/* every instance's initial state computed on the device (dense_init_device; benchmarks 11, 13,
   14), times and steps set to 0 */
int dense_batch_init_device(dense_batch_t* b);
/* device-array forms for the PyTorch form (layouts and stream ordering as dense_upload_device;
   the double Mach reflection and shock / shear layer rules' x, y rows come only from
   dense_batch_upload) */
int dense_batch_upload_device(dense_batch_t* b, int i, const double* cons, const double* prim, void* stream);
int dense_batch_download_device(dense_batch_t* b, int i, double* cons, double* prim, void* stream);
int dense_batch_steps_device(dense_batch_t* b, int nsteps, double t_end, int total_step, void* stream);

/* ---- discrete adjoint of the time step -------------------------------------------------- */

/* No counterpart in the reference (it has no derivatives): the reverse mode of n steps of the
   plain solver, for the LLF, GLF or Steger-Warming splitting (101-103) with upwind5, WENO-JS5
   or WENO-Z5 (251/253/255), or the characteristic schemes (104, AdaWENO 105; recon not read),
   on grids periodic in x and y (benchmarks 11 and 14) or with extrapolated, mirror and
   fixed-state sides (benchmarks 1, 2, 4, 9, Rayleigh-Taylor's 3 and 13 with its body force,
   the double Mach reflection 5, and the shear layer 6, whose inflow moves with the start time
   that the time steps make a function of the state), CFL or constant dt. GLF's global wave speed of each stage
   (104 and 105 split by GLF) is differentiated like the time step: its gradient goes to the cell
   where the maximum is attained; AdaWENO's branch at each face and sign is the one the forward
   took (a switch, held fixed like the maxima's cells). States and gradients
   are device arrays of the interior, u[4][nj][ni] (conserved variables, i fastest). The
   forward runs the plain solver's kernels and keeps the state every `checkpoint_every` steps;
   the reverse recomputes each segment from its checkpoint, storing the three stage states of
   each step, and runs the adjoint kernels back through it. The time step's dependence on the
   state (dt from the max wave speeds) is differentiated: its gradient goes to the cells where
   the maxima are attained. `stream` is the caller's cudaStream_t (0 for the default stream):
   each call starts after the work queued there and makes it wait for the call's work; the
   call itself does not block the host. */
typedef struct dense_adjoint dense_adjoint_t;
int dense_adjoint_create(const dense_config_t* cfg, int checkpoint_every, dense_adjoint_t** out);
void dense_adjoint_destroy(dense_adjoint_t* a);
/* uT = the state after nsteps steps from u0; keeps the checkpoints for dense_adjoint_backward */
int dense_adjoint_forward(dense_adjoint_t* a, const double* u0, int nsteps, double* uT, void* stream);
/* g0 = (d uT / d u0)^T gT for the last forward */
int dense_adjoint_backward(dense_adjoint_t* a, const double* gT, double* g0, void* stream);
/* one right-hand side L(u) = -(dh_xi/dx + dh_eta/dy) (the operator each stage applies):
   out = (dL/du)^T v at the state u; *vdotl = v . L(u) (host, the call waits) */
int dense_adjoint_rhs_vjp(dense_adjoint_t* a, const double* u, const double* v, double* out,
                          double* vdotl, void* stream);
/* the time steps of the last forward, on the host (the call waits) */
int dense_adjoint_get_dts(dense_adjoint_t* a, double* dts, int n);
/* after dense_adjoint_backward: per step k, the interior cells j*ni+i where max(|u|+alpha) and
   max(|v|+alpha) were attained (idx[2k], idx[2k+1]); -1 for constant dt (the call waits) */
int dense_adjoint_get_argmax(dense_adjoint_t* a, int* idx, int n);
/* the forward solver the adjoint drives (its state after the last call; owned by a) */
int dense_adjoint_get_solver(dense_adjoint_t* a, dense_handle_t** h);
long long dense_adjoint_launch_count(dense_adjoint_t* a);
const char* dense_adjoint_last_error(dense_adjoint_t* a);

/* ---- one stage without any device allocation ------------------------------------------- */

/* No counterpart in the reference: an addition for callers that cannot let the library
   allocate device memory -- host codes that manage every device byte through their own pool or
   a fixed budget (for example a Fortran driver that allocates all block arrays itself), for
   which dense_create's cudaMalloc calls are not allowed.
   One stage (get_primary, boundary_general, flux_splitting_general, time_rk3_general(irk)) on
   the caller's device arrays cons[4][NJp][P], prim[5][NJp][P], cons0[4][NJp][P] (P = ni+8
   rounded up to even; all in/out), with xbot = x(:,1), xtop = x(:,nj), yleft = y(1,:) on the
   device (needed by the double Mach reflection and shock / shear layer rules, else NULL).
   *dt_inout gives dt for irk 2 and 3 and constant-dt runs and returns the dt used. Work is
   queued on `stream` (a cudaStream_t, 0 for the default stream) and the call waits for it.
   The scratch (interface fluxes, per-stage scalars) is a fixed 8 MiB device array inside the
   library, held by every GPU that loads it until exit: grids needing more than 2^20 doubles of
   fluxes (4 nj (ni+1) + 4 (nj+1) ni, about 360 x 360 cells) fail with DENSE_ERR_LIMIT. All calls
   share that array, so calls whose GPU work overlaps race and must be serialised. The first
   call on a device (and the first in a new context of it, after cudaDeviceReset) resolves the
   array's device address; make it before any stream capture. The call allocates nothing and
   calls no allocating routine. After the stage it reads the device status word: a NaN, a
   density <= 0 or a Roe sound speed squared < 0 returns DENSE_ERR_NUMERIC, an index outside its
   array in the checked variant (strict = 2) DENSE_ERR_ARG, with the flags in
   dense_last_error(NULL); the pressure floor and an unknown reconstruction index are not
   failures. */
int dense_stage_noalloc(const dense_config_t* cfg, int irk, double current_time, double* cons,
                        double* prim, double* cons0, const double* xbot, const double* xtop,
                        const double* yleft, double* dt_inout, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DENSE2D_H */
