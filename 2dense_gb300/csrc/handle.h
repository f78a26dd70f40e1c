// handle.h — the single-block handle behind dense_handle_t (capi.cu), shared with the adjoint
// (adjoint.cu), which drives the same device buffers, kernels and step graph. Not part of the
// public interface.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "internal.h"

struct dense_handle {
    dense_config_t cfg;
    const dense::KernelTable* kt = nullptr;
    cudaStream_t stream = nullptr;
    int device = 0;
    double *cons = nullptr, *prim = nullptr, *cons0 = nullptr, *hx = nullptr, *he = nullptr;
    double *xbot = nullptr, *xtop = nullptr, *yleft = nullptr;
    double* theta = nullptr;  // AdaWENO indicators of the last stage, while if_save_theta
    dense::Scalars* sc = nullptr;
    dense::Params prm{};
    int NIp = 0, NJp = 0, P = 0;
    bool uploaded = false;
    int prim_slot = -1;  // stage slot whose max wave speeds match the current state, or -1
    cudaGraphExec_t step_graph = nullptr;
    int graph_nodes = 0;
    // the step graph runs a stage's eta sweep beside its xi sweep: the branch is captured on
    // `side` between the two events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    long long launches = 0;
    int count_branches = 0;
    std::string err;
};

namespace dense {
// get_primary of the current state into max-wave-speed slot `slot`, unless it is there already
int handle_ensure_prim(dense_handle* h, int slot);
// the CUDA graph of one time step (h->step_graph, h->graph_nodes), built on first use
int handle_step_graph(dense_handle* h);
// kernel launches of one stage (boundary, two sweeps, update)
int handle_stage_launches(dense_handle* h);
// the side stream and the fork/join events of a stage's two sweeps, created on first use
int handle_ensure_side(dense_handle* h);
}  // namespace dense
