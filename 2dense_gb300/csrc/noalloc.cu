// noalloc.cu — one Runge-Kutta stage with no device allocation: dense_stage_noalloc().
//
// Who needs it: callers that must not have the library call cudaMalloc. A host code that
// manages all device memory through its own pool or a fixed budget (a Fortran driver that
// allocates every block array itself, or a framework whose allocator must see every byte)
// cannot let a library allocate behind its back, and dense_create allocates the handle's
// buffers. Such a caller keeps the state in its own device arrays and calls this entry point;
// the stage's scratch -- the interface fluxes h_xi/h_eta that the flux sweeps write and the
// update reads, and the per-stage scalars (max wave speeds, dt) -- lives in file-scope device
// arrays of fixed size instead of buffers owned by a handle.
//
// Limits and sharing:
//  * the flux scratch holds kScratchDoubles doubles (8 MiB); a grid needs
//    4*nj*(ni+1) + 4*(nj+1)*ni of them, e.g. up to 360 x 360 cells. Larger grids are rejected
//    with DENSE_ERR_LIMIT. Every GPU that loads the library holds these 8 MiB until exit;
//  * all calls share the arrays, which keep the last call's contents. The stage clears what
//    must start at zero (the wave-speed slots, the status word, the fluxes when the
//    reconstruction index is unknown). Calls whose GPU work overlaps -- on two streams, or
//    from two host threads -- race on the arrays and must be serialised by the caller;
//  * the first call on a device resolves the device addresses of the arrays
//    (cudaGetSymbolAddress) with that device current; make that first call before any stream
//    capture begins. Later calls allocate nothing and call no allocating routine. A call made
//    in a new context of the device (after cudaDeviceReset, say) resolves them again;
//  * after the stage the call reads the device status word back: a NaN, a non-positive density
//    or a negative Roe sound speed squared returns DENSE_ERR_NUMERIC, an index outside its array
//    in the checked variant (strict = 2) DENSE_ERR_ARG, each with the flags in the error text
//    (dense_last_error(NULL)). The pressure floor and an unknown reconstruction index are not
//    failures, as in the reference, which goes on after both.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "internal.h"

namespace {

constexpr long long kScratchDoubles = 1LL << 20;  // 8 MiB of interface fluxes
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_flux_scratch[kScratchDoubles];
__device__ __align__(256) dense::Scalars g_scalars_scratch;

struct DevicePtrs {
    double* flux = nullptr;
    dense::Scalars* sc = nullptr;
    CUcontext ctx = nullptr;  // the context the addresses belong to
};
DevicePtrs g_ptrs[kMaxDevices];
std::mutex g_mu;

// the message goes where dense_last_error(NULL) reads it
int fail(int code, const std::string& msg) {
    dense::set_last_error(msg.c_str());
    return code;
}

// The current context, through the runtime's driver entry point (the library does not link the
// driver library itself, so it still loads on machines without one).
CUcontext current_context() {
    using Fn = CUresult (*)(CUcontext*);
    static const Fn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess)
            return (Fn) nullptr;
        return (Fn)f;
    }();
    CUcontext ctx = nullptr;
    if (!fn || fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    return ctx;
}

// Device addresses of the scratch arrays on the current device, resolved once per device and
// context (the module, and with it the arrays, is loaded again in a new context).
int resolve(int dev, DevicePtrs& out) {
    std::lock_guard<std::mutex> lock(g_mu);
    DevicePtrs& p = g_ptrs[dev];
    const CUcontext ctx = current_context();
    if (!p.flux || p.ctx != ctx) {
        void* f = nullptr;
        void* s = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&f, g_flux_scratch);
        if (e != cudaSuccess) return fail(DENSE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        e = cudaGetSymbolAddress(&s, g_scalars_scratch);
        if (e != cudaSuccess) return fail(DENSE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        p.flux = (double*)f;
        p.sc = (dense::Scalars*)s;
        p.ctx = ctx;
    }
    out = p;
    return DENSE_OK;
}

__global__ void k_noalloc_scalars(dense::Scalars* sc, int slot, double t, double dt) {
    sc->maxeig[slot][0] = 0.0;
    sc->maxeig[slot][1] = 0.0;
    sc->t = t;
    sc->dt = dt;
    sc->active = 1;
    sc->status = 0;
}

}  // namespace

// One stage on caller-owned device arrays (layout of the handle's buffers: variable planes of
// NJp rows with a row pitch P = (ni+8) rounded up to an even number of doubles):
//   cons [4][NJp][P]  in/out   conserved variables, ghosts included
//   prim [5][NJp][P]  in/out   rho,u,v,p,alpha; the interior is recomputed, ghosts filled
//   cons0[4][NJp][P]  in/out   the stage-1 copy (written at irk 1, read at irk 2 and 3)
//   xbot, xtop [ni], yleft [nj]  x(i,1), x(i,nj), y(1,j); needed by the double Mach reflection
//                                and shock / shear layer boundary rules, else may be NULL
// *dt_inout: in, the step's dt for irk 2 and 3 and for if_const_dt; out, the dt used (computed
// from the CFL condition at irk 1). The call waits for its work on `stream` to finish.
extern "C" int dense_stage_noalloc(const dense_config_t* cfg, int irk, double current_time,
                                   double* cons, double* prim, double* cons0, const double* xbot,
                                   const double* xtop, const double* yleft, double* dt_inout,
                                   void* stream) {
    using dense::kB;
    if (!cfg || !cons || !prim || !cons0 || !dt_inout) return fail(DENSE_ERR_ARG, "null argument");
    if (irk < 1 || irk > 3) return fail(DENSE_ERR_ARG, "irk must be 1, 2 or 3");
    if (cfg->ni < 3 || cfg->nj < 3 || cfg->bfsize != kB || cfg->neq != 4 || cfg->stages != 3)
        return fail(DENSE_ERR_ARG, "ni, nj >= 3, bfsize 4, neq 4 and stages 3 are required");
    if (cfg->splitting < DENSE_SPLIT_LLF || cfg->splitting > DENSE_SPLIT_SC)
        return fail(DENSE_ERR_SPLITTING, "No such Selection (flux_splitting.f90:30-32)");
    if (cfg->dx <= 0.0 || cfg->dy <= 0.0) return fail(DENSE_ERR_ARG, "dx and dy must be set");
    if (cfg->strict < 0 || cfg->strict > 2)
        return fail(DENSE_ERR_ARG, "strict must be 0 (fast), 1 (strict) or 2 (checked)");
    const int b = cfg->benchmark;
    const bool bench_ok = b == 0 || (b >= 1 && b <= 9) || b == DENSE_BENCH_IVC_PERIODIC ||
                          b == DENSE_BENCH_RT_REFLECT || b == DENSE_BENCH_RM_PERIODIC;
    if (!bench_ok) return fail(DENSE_ERR_BENCHMARK, "No such Benchmark index! (boundary_general.f90:26-28)");
    if ((b == DENSE_BENCH_DMR && (!xbot || !xtop)) || (b == DENSE_BENCH_SSL && !yleft))
        return fail(DENSE_ERR_ARG, "this benchmark's boundary rule needs the cell-centre rows");
    const long long ni = cfg->ni, nj = cfg->nj;
    const long long hx_n = 4 * nj * (ni + 1), he_n = 4 * (nj + 1) * ni;
    if (hx_n + he_n > kScratchDoubles)
        return fail(DENSE_ERR_LIMIT, "grid too large for the fixed scratch: needs " +
                                         std::to_string(hx_n + he_n) + " doubles, the maximum is " +
                                         std::to_string(kScratchDoubles));
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(DENSE_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(DENSE_ERR_LIMIT, "device ordinal out of range");
    DevicePtrs ptr;
    int rc = resolve(dev, ptr);
    if (rc) return rc;

    dense::Params p{};
    const int NIp = cfg->ni + 2 * kB, NJp = cfg->nj + 2 * kB;
    p.cons = cons; p.prim = prim; p.cons0 = cons0;
    p.hx = ptr.flux; p.he = ptr.flux + hx_n;
    p.xbot = xbot; p.xtop = xtop; p.yleft = yleft;
    p.sc = ptr.sc;
    p.ni = cfg->ni; p.nj = cfg->nj; p.P = (NIp + 1) & ~1;
    p.plane = (long long)NJp * p.P;
    p.gamma = cfg->gamma; p.cfl = cfg->cfl; p.delta = cfg->delta; p.dx = cfg->dx; p.dy = cfg->dy;
    p.dt_const = cfg->dt;
    p.theta_c = dense::theta_c_of(cfg->delta);
    p.if_const_dt = cfg->if_const_dt;
    p.bodyforce = cfg->if_bodyforce && (b == DENSE_BENCH_RT || b == DENSE_BENCH_RT_REFLECT);
    p.benchmark = b; p.splitting = cfg->splitting; p.recon = cfg->recon;
    const dense::KernelTable* kt = dense::kernels_for(cfg->strict);

    cudaStream_t s = (cudaStream_t)stream;
    k_noalloc_scalars<<<1, 1, 0, s>>>(ptr.sc, irk - 1, current_time, *dt_inout);
    const bool recon_known = cfg->recon == DENSE_RECON_UPWIND5 || cfg->recon == DENSE_RECON_WENOJS5 ||
                             cfg->recon == DENSE_RECON_WENOZ5;
    if (cfg->splitting <= DENSE_SPLIT_SW && !recon_known) {
        // the reference leaves h_xi/h_eta at their zero start when the index is unknown
        e = cudaMemsetAsync(ptr.flux, 0, (size_t)(hx_n + he_n) * sizeof(double), s);
        if (e != cudaSuccess) return fail(DENSE_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    }
    kt->prim(p, irk - 1, s);                // get_primary
    kt->bc(p, s);                           // boundary_general
    kt->flux(p, irk, 0, s);                 // flux_splitting_general, xi
    kt->flux(p, irk, 1, s);                 // flux_splitting_general, eta
    kt->update(p, irk, s);                  // time_rk3_general(irk)
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(DENSE_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    double dt = 0.0;
    unsigned flags = 0;
    e = cudaMemcpyAsync(&dt, &ptr.sc->dt, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&flags, &ptr.sc->status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(DENSE_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(e));
    *dt_inout = dt;
    char hex[16];
    snprintf(hex, sizeof hex, "0x%02x", flags);
    if (flags & DENSE_FLAG_BOUNDS)
        return fail(DENSE_ERR_ARG, std::string("device status flags ") + hex +
                                       ": an array index fell outside its array (checked variant)");
    if (flags & (DENSE_FLAG_NAN | DENSE_FLAG_NEG_RHO | DENSE_FLAG_ROE_IMAG))
        return fail(DENSE_ERR_NUMERIC, std::string("device status flags ") + hex +
                                           ": NaN (0x01), density <= 0 (0x02) or Roe sound speed "
                                           "squared < 0 (0x08) in the stage");
    return DENSE_OK;
}
