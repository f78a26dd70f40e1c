// setup_device.cu — device-side initial states of the variant benchmarks 11, 13, 14 and the
// error of the translating vortex against its exact solution (csrc/setups.cuh).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "handle.h"
#include "setups.cuh"

namespace {

using dense::Params;
using dense::kB;

__global__ void k_init(Params p, double eps, double xc, double yc, double amp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < p.ni && j < p.nj) dense::setups::init_cell(p, eps, xc, yc, amp, i, j);
}

// Per block: sum and max of |rho - rho_exact| over its cells. The exact solution of the
// translating vortex at time t is the initial vortex moved by (t, t) on the periodic square
// [0,10]^2 (nearest periodic image of the centre).
__global__ void k_vortex_error(Params p, double eps, double xc, double yc, double t, double* part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    double e = 0.0;
    if (i < p.ni && j < p.nj) {
        const double x = (i + 0.5) * p.dx, y = (j + 0.5) * p.dy;
        double rx = x - (xc + t), ry = y - (yc + t);
        rx -= 10.0 * rint(rx / 10.0);
        ry -= 10.0 * rint(ry / 10.0);
        const double g = p.gamma, pi = dense::setups::kPi;
        const double rho = pow(1.0 - (g - 1.0) * (eps * eps) * exp(1.0 - (rx * rx + ry * ry)) / (8.0 * g * (pi * pi)),
                               1.0 / (g - 1.0));
        e = fabs(p.cons[(long long)(j + kB) * p.P + (i + kB)] - rho);
    }
    double s = e, m = e;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    __shared__ double rs[8], rm[8];
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if ((tid & 31) == 0) { rs[tid >> 5] = s; rm[tid >> 5] = m; }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < (int)(blockDim.x * blockDim.y + 31) / 32; ++w) { s += rs[w]; m = fmax(m, rm[w]); }
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
        part[2 * b] = s;
        part[2 * b + 1] = m;
    }
}

thread_local std::string g_err;

int err(dense_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg; else g_err = msg;
    return code;
}

bool has_device_setup(int b) {
    return b == DENSE_BENCH_IVC_PERIODIC || b == DENSE_BENCH_RT_REFLECT || b == DENSE_BENCH_RM_PERIODIC;
}

}  // namespace

extern "C" {

int dense_init_device(dense_handle_t* h) {
    if (!h) return err(h, DENSE_ERR_ARG, "null handle");
    const dense_config_t& c = h->cfg;
    if (!has_device_setup(c.benchmark))
        return err(h, DENSE_ERR_BENCHMARK, "device setups exist for benchmarks 11, 13 and 14");
    const size_t plane = (size_t)h->NJp * h->P;
    cudaError_t e = cudaMemsetAsync(h->cons, 0, plane * 4 * sizeof(double), h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->prim, 0, plane * 5 * sizeof(double), h->stream);
    if (e != cudaSuccess) return err(h, DENSE_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const dim3 b(32, 8), g((c.ni + 31) / 32, (c.nj + 7) / 8);
    k_init<<<g, b, 0, h->stream>>>(h->prm, c.var_eps, c.var_xc, c.var_yc, c.var_amp);
    h->launches += 1;
    e = cudaGetLastError();
    if (e != cudaSuccess) return err(h, DENSE_ERR_CUDA, std::string("k_init: ") + cudaGetErrorString(e));
    h->uploaded = true;
    h->prim_slot = -1;
    int rc = dense::handle_ensure_prim(h, 0);
    if (rc) return rc;
    return dense_set_time(h, 0.0, 0);
}

int dense_vortex_error(dense_handle_t* h, double* l1, double* linf) {
    if (!h || !l1 || !linf) return err(h, DENSE_ERR_ARG, "null argument");
    if (h->cfg.benchmark != DENSE_BENCH_IVC_PERIODIC)
        return err(h, DENSE_ERR_BENCHMARK, "the exact solution is known for the translating vortex (11)");
    if (!h->uploaded) return err(h, DENSE_ERR_STATE, "dense_vortex_error before an upload");
    const dense_config_t& c = h->cfg;
    const dim3 b(32, 8), g((c.ni + 31) / 32, (c.nj + 7) / 8);
    const int nb = (int)(g.x * g.y);
    double t = 0.0;
    int step = 0;
    int rc = dense_get_time(h, &t, &step, nullptr);
    if (rc) return rc;
    double* part = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&part, (size_t)2 * nb * sizeof(double), h->stream);
    if (e != cudaSuccess) return err(h, DENSE_ERR_NOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    k_vortex_error<<<g, b, 0, h->stream>>>(h->prm, c.var_eps, c.var_xc, c.var_yc, t, part);
    h->launches += 1;
    std::vector<double> hp((size_t)2 * nb);
    e = cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(part, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return err(h, DENSE_ERR_CUDA, std::string("vortex error: ") + cudaGetErrorString(e));
    double s = 0.0, m = 0.0;
    for (int k = 0; k < nb; ++k) { s += hp[2 * k]; m = std::fmax(m, hp[2 * k + 1]); }
    *l1 = s / ((double)c.ni * c.nj);
    *linf = m;
    return DENSE_OK;
}

}  // extern "C"
