// io.cu — the save path of the reference's driver loop: the Tecplot ASCII file of
// write_tec_at_time_cartisian (output_test_general.f90:18-59), the unformatted checkpoint of
// write_date_binary / load_date_binary (read_WriteAndLoad.f90:1-70), and the loop of
// general_main.f90:23-55 with its saves, run on the device.
//
// In the driver loop the device does not wait for the files: the step after which a save is due
// holds the following steps (Scalars::hold, set in step_end); the host copies the state into a
// device snapshot, lets the device run on, and a writer thread copies the snapshot to host memory
// on its own stream and formats the files. The device waits only if the next save comes before the previous
// one is written.
#include <cuda_runtime.h>

#include <chrono>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "handle.h"
#include "nvtx.h"

extern "C" int dense_grid_coords(const dense_config_t* cfg, double* x, double* y, double* vx, double* vy);

using dense::Scalars;
using dense::kB;

namespace {

thread_local std::string g_err;

int ioerr(dense_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg; else g_err = msg;
    return code;
}

#define ICK(h, call)                                                                             \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return ioerr((h), DENSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// A state on the host, in the reference's array order: cons(NIp,NJp,4), prim(NIp,NJp,5).
struct HostState {
    dense_config_t cfg{};
    long long step = 0;
    double t = 0.0;
    std::vector<double> cons, prim;
    std::vector<double> theta;  // AdaWENO indicators, xi [2][nj][ni+1] then eta [2][nj+1][ni]; empty: none
};

size_t theta_size(const dense_config_t& c) {
    return (size_t)2 * ((size_t)c.nj * (c.ni + 1) + (size_t)(c.nj + 1) * c.ni);
}

// One value per line, as list-directed output writes them (17 significant digits: the file
// reads back to the same doubles).
void put_value(FILE* f, double v) { std::fprintf(f, " %#.17G\n", v); }

// write_tec_at_time_cartisian: vertex coordinates (ni+1)x(nj+1), then every primitive
// variable of the interior, cell-centred, i fastest. The variables are prim(:,:,1..6) -- rho,
// u, v, p, alpha and the entropy log(p) - log(rho) -- as the reference writes them
// (prim_lastvar_index = 6, var_index.f90:5-11), under its header naming seven variables.
int write_tec(dense_handle* h, const HostState& s, const std::string& path) {
    const dense_config_t& c = s.cfg;
    const int ni = c.ni, nj = c.nj, NIp = ni + 2 * kB, NJp = nj + 2 * kB;
    std::vector<double> vx((size_t)(ni + 1) * (nj + 1)), vy(vx.size());
    int rc = dense_grid_coords(&c, nullptr, nullptr, vx.data(), vy.data());
    if (rc) return ioerr(h, rc, "grid coordinates");
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return ioerr(h, DENSE_ERR_IO, "cannot open " + path);
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    std::fprintf(f, " title=\"flow time %#.17G\"\n", s.t);
    std::fprintf(f, " variables=\"x\",\"y\",\"rho\",\"u\",\"v\",\"p\",\"alpha\"\n");
    std::fprintf(f, " ZONE I=%12d  J=%12d DATAPACKING=BLOCK, VARLOCATION=([3-7]=CELLCENTERED)\n", ni + 1, nj + 1);
    for (double v : vx) put_value(f, v);
    for (double v : vy) put_value(f, v);
    const size_t P = (size_t)NIp * NJp;
    for (int var = 0; var < 6; ++var)
        for (int j = kB; j < nj + kB; ++j)
            for (int i = kB; i < ni + kB; ++i) {
                const size_t o = (size_t)j * NIp + i;
                const double v = var < 5 ? s.prim[var * P + o] : std::log(s.prim[3 * P + o]) - std::log(s.prim[o]);
                put_value(f, v);
            }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    if (!ok) return ioerr(h, DENSE_ERR_IO, "write failed: " + path);
    return DENSE_OK;
}

// write_theta_at_time_cartisian (output_test_general.f90:61-119): the AdaWENO indicator per
// cell, the larger of its two faces' values, for xi "+" / "-" and eta "+" / "-"; zeros when the
// sweeps have none (the reference's theta arrays start at zero, flow_mod_general.f90:241-250).
int write_theta(dense_handle* h, const HostState& s, const std::string& path) {
    const dense_config_t& c = s.cfg;
    const int ni = c.ni, nj = c.nj;
    std::vector<double> vx((size_t)(ni + 1) * (nj + 1)), vy(vx.size());
    int rc = dense_grid_coords(&c, nullptr, nullptr, vx.data(), vy.data());
    if (rc) return ioerr(h, rc, "grid coordinates");
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return ioerr(h, DENSE_ERR_IO, "cannot open " + path);
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    std::fprintf(f, " title=\"flow time %#.17G\"\n", s.t);
    std::fprintf(f, " variables=\"x\",\"y\",\"xp\",\"xn\",\"ep\",\"en\"\n");
    std::fprintf(f, " ZONE I=%12d  J=%12d DATAPACKING=BLOCK, VARLOCATION=([3-6]=CELLCENTERED)\n", ni + 1, nj + 1);
    for (double v : vx) put_value(f, v);
    for (double v : vy) put_value(f, v);
    const size_t xs = (size_t)nj * (ni + 1), es = (size_t)(nj + 1) * ni;
    const bool have = !s.theta.empty();
    for (int sg = 0; sg < 2; ++sg)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                const double* T = have ? s.theta.data() + sg * xs + (size_t)j * (ni + 1) : nullptr;
                put_value(f, have ? std::fmax(T[i], T[i + 1]) : 0.0);
            }
    for (int sg = 0; sg < 2; ++sg)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                const double* T = have ? s.theta.data() + 2 * xs + sg * es : nullptr;
                put_value(f, have ? std::fmax(T[(size_t)j * ni + i], T[(size_t)(j + 1) * ni + i]) : 0.0);
            }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    if (!ok) return ioerr(h, DENSE_ERR_IO, "write failed: " + path);
    return DENSE_OK;
}

// gfortran unformatted sequential records: a 4-byte length before and after each record.
struct Rec {
    std::vector<char> b;
    template <class T> Rec& operator<<(const T& v) {
        const char* p = (const char*)&v;
        b.insert(b.end(), p, p + sizeof(T));
        return *this;
    }
    Rec& raw(const void* p, size_t n) {
        b.insert(b.end(), (const char*)p, (const char*)p + n);
        return *this;
    }
};
bool put_rec(FILE* f, const Rec& r) {
    const int32_t n = (int32_t)r.b.size();
    return std::fwrite(&n, 4, 1, f) == 1 && (r.b.empty() || std::fwrite(r.b.data(), 1, r.b.size(), f) == r.b.size()) &&
           std::fwrite(&n, 4, 1, f) == 1;
}

// write_date_binary (read_WriteAndLoad.f90:1-26) for the one Cartesian block: (step, time),
// num_block, index, (ni, nj), (bfsize_i, bfsize_j), cons, x, y, (dx, dy).
int write_bin(dense_handle* h, const HostState& s, const std::string& path) {
    const dense_config_t& c = s.cfg;
    std::vector<double> x((size_t)c.ni * c.nj), y(x.size());
    int rc = dense_grid_coords(&c, x.data(), y.data(), nullptr, nullptr);
    if (rc) return ioerr(h, rc, "grid coordinates");
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return ioerr(h, DENSE_ERR_IO, "cannot open " + path);
    bool ok = put_rec(f, Rec() << (int32_t)s.step << s.t) && put_rec(f, Rec() << (int32_t)1) &&
              put_rec(f, Rec() << (int32_t)1) && put_rec(f, Rec() << (int32_t)c.ni << (int32_t)c.nj) &&
              put_rec(f, Rec() << (int32_t)kB << (int32_t)kB) &&
              put_rec(f, Rec().raw(s.cons.data(), s.cons.size() * sizeof(double))) &&
              put_rec(f, Rec().raw(x.data(), x.size() * sizeof(double))) &&
              put_rec(f, Rec().raw(y.data(), y.size() * sizeof(double))) && put_rec(f, Rec() << c.dx << c.dy);
    ok = ok && std::fflush(f) == 0;
    std::fclose(f);
    if (!ok) return ioerr(h, DENSE_ERR_IO, "write failed: " + path);
    return DENSE_OK;
}

int get_rec(FILE* f, std::vector<char>& out) {
    int32_t n = 0, m = 0;
    if (std::fread(&n, 4, 1, f) != 1 || n < 0) return DENSE_ERR_IO;
    out.resize((size_t)n);
    if (n && std::fread(out.data(), 1, (size_t)n, f) != (size_t)n) return DENSE_ERR_IO;
    if (std::fread(&m, 4, 1, f) != 1 || m != n) return DENSE_ERR_IO;
    return DENSE_OK;
}

std::string save_name(const std::string& dir, long long step, const char* ext) {
    // "2d_"//trim(adjustl(temp))//ext with temp = step in i8 (output_test_general.f90:26-27)
    char b[64];
    std::snprintf(b, sizeof b, "2d_%lld%s", step, ext);
    return dir.empty() ? std::string(b) : dir + "/" + b;
}

std::string theta_name(const std::string& dir, long long step) {
    char b[64];
    std::snprintf(b, sizeof b, "2d_theta_%lld.dat", step);  // output_test_general.f90:72
    return dir.empty() ? std::string(b) : dir + "/" + b;
}

// the handle's state (cons, prim interior as the last get_primary left them) on the host
int snapshot_now(dense_handle* h, HostState& s) {
    s.cfg = h->cfg;
    const int NIp = h->NIp, NJp = h->NJp;
    s.cons.assign((size_t)NIp * NJp * 4, 0.0);
    s.prim.assign((size_t)NIp * NJp * 5, 0.0);
    const size_t row = (size_t)NIp * sizeof(double), pitch = (size_t)h->P * sizeof(double);
    ICK(h, cudaMemcpy2DAsync(s.cons.data(), row, h->cons, pitch, row, (size_t)NJp * 4, cudaMemcpyDeviceToHost, h->stream));
    ICK(h, cudaMemcpy2DAsync(s.prim.data(), row, h->prim, pitch, row, (size_t)NJp * 5, cudaMemcpyDeviceToHost, h->stream));
    s.theta.clear();
    if (h->prm.theta) {
        s.theta.resize(theta_size(h->cfg));
        ICK(h, cudaMemcpyAsync(s.theta.data(), h->prm.theta, s.theta.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
    }
    Scalars sc{};
    ICK(h, cudaMemcpyAsync(&sc, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream));
    ICK(h, cudaStreamSynchronize(h->stream));
    s.step = sc.step;
    s.t = sc.t;
    return DENSE_OK;
}

__global__ void k_save_mode(Scalars* sc, int mode, long long save_step, double dt_save, double t_end,
                            long long total_step) {
    sc->save_mode = mode;
    sc->save_step = save_step;
    sc->dt_save = dt_save;
    sc->t_end = t_end;
    sc->total_step = total_step;
    sc->hold = 0;
}
__global__ void k_release(Scalars* sc, int reset_elasp) {
    if (reset_elasp) sc->elasp = 0.0;
    sc->hold = 0;
}

}  // namespace

extern "C" {

int dense_write_tecplot(dense_handle_t* h, const char* path) {
    dense::NvtxRange nvtx_("dense_write_tecplot");
    if (!h || !path) return ioerr(h, DENSE_ERR_ARG, "null argument");
    if (!h->uploaded) return ioerr(h, DENSE_ERR_STATE, "dense_write_tecplot before an upload");
    HostState s;
    int rc = dense::handle_ensure_prim(h, h->prim_slot < 0 ? 0 : h->prim_slot);
    if (!rc) rc = snapshot_now(h, s);
    if (rc) return rc;
    return write_tec(h, s, path);
}

int dense_write_theta(dense_handle_t* h, const char* path) {
    dense::NvtxRange nvtx_("dense_write_theta");
    if (!h || !path) return ioerr(h, DENSE_ERR_ARG, "null argument");
    if (!h->uploaded) return ioerr(h, DENSE_ERR_STATE, "dense_write_theta before an upload");
    HostState s;
    int rc = snapshot_now(h, s);
    if (rc) return rc;
    return write_theta(h, s, path);
}

int dense_get_theta(dense_handle_t* h, double* theta) {
    if (!h || !theta) return ioerr(h, DENSE_ERR_ARG, "null argument");
    if (!h->prm.theta) return ioerr(h, DENSE_ERR_STATE, "no indicators: if_save_theta is off or the splitting is not 105");
    ICK(h, cudaMemcpyAsync(theta, h->prm.theta, theta_size(h->cfg) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ICK(h, cudaStreamSynchronize(h->stream));
    return DENSE_OK;
}

int dense_write_binary(dense_handle_t* h, const char* path) {
    dense::NvtxRange nvtx_("dense_write_binary");
    if (!h || !path) return ioerr(h, DENSE_ERR_ARG, "null argument");
    if (!h->uploaded) return ioerr(h, DENSE_ERR_STATE, "dense_write_binary before an upload");
    HostState s;
    int rc = snapshot_now(h, s);
    if (rc) return rc;
    return write_bin(h, s, path);
}

int dense_read_binary(const char* path, dense_config_t* cfg, double* cons, double* x, double* y, int* step,
                      double* time) {
    if (!path || !cfg) return ioerr(nullptr, DENSE_ERR_ARG, "null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return ioerr(nullptr, DENSE_ERR_IO, std::string("cannot open ") + path);
    std::vector<char> r[9];
    int rc = DENSE_OK;
    for (int k = 0; k < 9 && !rc; ++k) rc = get_rec(f, r[k]);
    std::fclose(f);
    if (rc) return ioerr(nullptr, DENSE_ERR_IO, std::string("not a checkpoint of one block: ") + path);
    int32_t st, nb, ni, nj, bi, bj;
    double t;
    if (r[0].size() != 12 || r[1].size() != 4 || r[3].size() != 8 || r[4].size() != 8 || r[8].size() != 16)
        return ioerr(nullptr, DENSE_ERR_IO, std::string("unexpected record sizes in ") + path);
    std::memcpy(&st, r[0].data(), 4); std::memcpy(&t, r[0].data() + 4, 8);
    std::memcpy(&nb, r[1].data(), 4);
    std::memcpy(&ni, r[3].data(), 4); std::memcpy(&nj, r[3].data() + 4, 4);
    std::memcpy(&bi, r[4].data(), 4); std::memcpy(&bj, r[4].data() + 4, 4);
    if (nb != 1 || bi != kB || bj != kB || ni < 1 || nj < 1)
        return ioerr(nullptr, DENSE_ERR_IO, "only one Cartesian block with 4 ghost layers is supported");
    const size_t nc = (size_t)(ni + 2 * kB) * (nj + 2 * kB) * 4, nx = (size_t)ni * nj;
    if (r[5].size() != nc * 8 || r[6].size() != nx * 8 || r[7].size() != nx * 8)
        return ioerr(nullptr, DENSE_ERR_IO, std::string("array records do not match ni, nj in ") + path);
    cfg->ni = ni; cfg->nj = nj; cfg->bfsize = kB;
    std::memcpy(&cfg->dx, r[8].data(), 8);
    std::memcpy(&cfg->dy, r[8].data() + 8, 8);
    if (cons) std::memcpy(cons, r[5].data(), nc * 8);
    if (x) std::memcpy(x, r[6].data(), nx * 8);
    if (y) std::memcpy(y, r[7].data(), nx * 8);
    if (step) *step = st;
    if (time) *time = t;
    return DENSE_OK;
}

int dense_run(dense_handle_t* h, const char* dir, const char* namelist_path, int* saves_out) {
    dense::NvtxRange nvtx_("dense_run");
    if (!h) return ioerr(h, DENSE_ERR_ARG, "null handle");
    if (!h->uploaded) return ioerr(h, DENSE_ERR_STATE, "dense_run before an upload");
    const std::string d = dir ? dir : "";
    const int kChunk = 32;  // step graphs between looks at the device's loop state
    double* snap = nullptr;
    const size_t plane = (size_t)h->NJp * h->P, nth = theta_size(h->cfg);
    ICK(h, cudaMalloc((void**)&snap, (plane * 9 + nth) * sizeof(double)));
    cudaEvent_t ev = nullptr;
    cudaStream_t io = nullptr;
    cudaError_t ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&io, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        cudaFree(snap);
        if (ev) cudaEventDestroy(ev);
        return ioerr(h, DENSE_ERR_CUDA, std::string("dense_run setup: ") + cudaGetErrorString(ce));
    }
    std::thread writer;
    int writer_rc = DENSE_OK, saves = 0, rc = DENSE_OK;
    auto join = [&]() {
        if (writer.joinable()) writer.join();
    };
    auto bounds = [&]() {
        const dense_config_t& c = h->cfg;
        k_save_mode<<<1, 1, 0, h->stream>>>(h->sc, 1, c.save_step, c.dt_save, c.total_time, c.total_step);
        h->launches += 1;
    };
    bounds();
    // cpu_t of general_main.f90:22-31: wall time of the step loop, saves excluded
    double cpu_t = 0.0;
    long long last_step = 0;
    for (;;) {
        const auto t0 = std::chrono::steady_clock::now();
        rc = dense_steps_async(h, kChunk, h->cfg.total_time, h->cfg.total_step);
        if (rc) break;
        Scalars sc{};
        ce = cudaMemcpyAsync(&sc, h->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, h->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
        cpu_t += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        last_step = sc.step;
        if (ce != cudaSuccess) { rc = ioerr(h, DENSE_ERR_CUDA, std::string("dense_run: ") + cudaGetErrorString(ce)); break; }
        if (sc.hold) {
            // general_main.f90:40-54: the binary checkpoint, then get_primary and the Tecplot
            // file (which resets elasp_time), then the namelists are read again
            join();
            if (writer_rc) { rc = writer_rc; break; }
            ce = cudaMemcpyAsync(snap, h->cons, plane * 4 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream);
            if (ce == cudaSuccess) ce = cudaMemcpyAsync(snap + plane * 4, h->prim, plane * 5 * sizeof(double),
                                                        cudaMemcpyDeviceToDevice, h->stream);
            const bool with_theta = h->prm.theta != nullptr;
            if (ce == cudaSuccess && with_theta)
                ce = cudaMemcpyAsync(snap + plane * 9, h->prm.theta, nth * sizeof(double), cudaMemcpyDeviceToDevice,
                                     h->stream);
            if (ce == cudaSuccess) ce = cudaEventRecord(ev, h->stream);
            if (ce != cudaSuccess) { rc = ioerr(h, DENSE_ERR_CUDA, std::string("snapshot: ") + cudaGetErrorString(ce)); break; }
            const dense_config_t cfg = h->cfg;
            const long long step = sc.step;
            const double t = sc.t;
            const int NIp = h->NIp, NJp = h->NJp, P = h->P;
            writer = std::thread([&writer_rc, h, snap, ev, io, cfg, step, t, NIp, NJp, P, plane, nth, with_theta, d]() {
                HostState s;
                s.cfg = cfg; s.step = step; s.t = t;
                s.cons.assign((size_t)NIp * NJp * 4, 0.0);
                s.prim.assign((size_t)NIp * NJp * 5, 0.0);
                const size_t rowb = (size_t)NIp * sizeof(double), pitch = (size_t)P * sizeof(double);
                cudaError_t e = cudaStreamWaitEvent(io, ev, 0);
                if (e == cudaSuccess)
                    e = cudaMemcpy2DAsync(s.cons.data(), rowb, snap, pitch, rowb, (size_t)NJp * 4, cudaMemcpyDeviceToHost, io);
                if (e == cudaSuccess)
                    e = cudaMemcpy2DAsync(s.prim.data(), rowb, snap + plane * 4, pitch, rowb, (size_t)NJp * 5,
                                          cudaMemcpyDeviceToHost, io);
                if (e == cudaSuccess && with_theta) {
                    s.theta.resize(nth);
                    e = cudaMemcpyAsync(s.theta.data(), snap + plane * 9, nth * sizeof(double), cudaMemcpyDeviceToHost, io);
                }
                if (e == cudaSuccess) e = cudaStreamSynchronize(io);
                if (e != cudaSuccess) { writer_rc = DENSE_ERR_CUDA; return; }
                int r = DENSE_OK;
                if (cfg.if_save_binary) r = write_bin(nullptr, s, save_name(d, step, ".dat2d"));
                if (!r && cfg.if_save_tec) r = write_tec(nullptr, s, save_name(d, step, ".dat"));
                // write_tec_at_time writes the indicators too (output_test_general.f90:10-12)
                if (!r && cfg.if_save_tec && cfg.if_save_theta) r = write_theta(nullptr, s, theta_name(d, step));
                writer_rc = r;
            });
            ++saves;
            k_release<<<1, 1, 0, h->stream>>>(h->sc, cfg.if_save_tec ? 1 : 0);
            h->launches += 1;
            if (namelist_path) {
                dense_config_t nc = h->cfg;
                rc = dense_read_namelist(namelist_path, &nc);
                if (!rc) {
                    nc.ni = h->cfg.ni; nc.nj = h->cfg.nj; nc.benchmark = h->cfg.benchmark;
                    nc.dx = h->cfg.dx; nc.dy = h->cfg.dy;
                    rc = dense_reconfigure(h, &nc);
                }
                if (rc) break;
                bounds();
            }
            continue;
        }
        if (!sc.active) break;  // the while-condition of general_main.f90:23 failed
    }
    join();
    if (!rc && writer_rc) rc = writer_rc;
    k_save_mode<<<1, 1, 0, h->stream>>>(h->sc, 0, 0, 0.0, h->cfg.total_time, h->cfg.total_step);
    h->launches += 1;
    cudaStreamSynchronize(h->stream);
    cudaEventDestroy(ev);
    cudaStreamDestroy(io);
    cudaFree(snap);
    if (rc) return rc;
    if (saves_out) *saves_out = saves;
    // general_main.f90:20,56-58: the timing log, appended
    if (FILE* f = fopen((d.empty() ? std::string("CpuTime.dat") : d + "/CpuTime.dat").c_str(), "a")) {
        fprintf(f, " Total time and steps:%25.17g%12lld\n", cpu_t, last_step);
        fprintf(f, " averaged time:%25.17g\n", cpu_t / (double)last_step);
        fclose(f);
    } else {
        return ioerr(h, DENSE_ERR_IO, "cannot open CpuTime.dat in " + d);
    }
    // general_main.f90:59-60: get_primary and the final Tecplot file
    HostState s;
    rc = snapshot_now(h, s);
    if (!rc) rc = write_tec(h, s, save_name(d, s.step, ".dat"));
    if (!rc && h->cfg.if_save_theta) rc = write_theta(h, s, theta_name(d, s.step));
    return rc;
}

// errors of calls without a handle (dense_read_binary), read by dense_last_error(NULL)
const char* dense_io_last_error(void) { return g_err.c_str(); }

}  // extern "C"
