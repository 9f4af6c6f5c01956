// lbm_handle.h -- the lattice handle behind the opaque lbm_t of include/lbm.h
// (internal to the library; shared by lbm_capi.cu and lbm_adjoint_host.cu).
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "lbm.h"

// State of an adjoint run (lbm_adjoint_forward / lbm_adjoint_backward).
struct lbm_adjoint_state {
    int iterations = 0;        // T of the last adjoint forward
    int every = 0;             // checkpoint interval c
    std::vector<void *> ckpt;  // Q_0, Q_c, Q_2c, ... (P buffers)
    std::vector<void *> seg;   // recomputed Q_{jc+1} .. Q_{jc+c-1} of one segment
    void *adj[2] = {nullptr, nullptr};  // adjoint ping-pong (post-stream layout)
    double *grad_lid = nullptr;         // dim*dim
    double *tau_acc = nullptr;          // per adjoint block
    double *loss_part = nullptr;        // per loss block (2 doubles)
    void *target = nullptr;             // dim*dim u_x target, adjoint type
    unsigned adj_grid = 0, loss_grid = 0;
    int plane_y = -1;
    bool init_state = false;   // Q_0 was made by the init kernel (lid-dependent)
    bool ready = false;        // a forward was recorded and Q_T is current
    int64_t it_end = -1;       // handle iteration count when the forward ended
    size_t bytes = 0;          // device bytes held by this state
    // graph replay of full segments: the staged first state, one graph per
    // adjoint-buffer parity, the parity flip of one segment, its length
    void *q0 = nullptr;
    cudaGraphExec_t seg_exec[2] = {nullptr, nullptr};
    int seg_flip[2] = {0, 0};
    int seg_graph_c = 0;
    bool seg_graph_macro = false;  // the graphs are of the stored-point sweep
    // stored-point sweep (no tau gradient): the linearisation point of every
    // iteration of one segment (3 planes each) and two state scratch buffers
    std::vector<void *> mseg;
    void *mtmp[2] = {nullptr, nullptr};
    // the points of the iterations tail_k0 .. T-1 (the last segments),
    // recorded by the adjoint forward into one allocation: those segments
    // are not recomputed
    void *tail_block = nullptr;
    size_t tail_bytes = 0;
    std::vector<void *> tpts;  // per iteration, into tail_block
    int tail_k0 = 0;
};

struct lbm_handle {
    lbm_config cfg;
    int dim = 0;
    size_t n = 0;
    int prec = 0;
    int V = 4;
    int sd = 0;             // log2 of the CSoA stride of F dumps
    double inv_tau = 0;     // 1/tau rounded to the compute precision
    float omega_f = 0;
    void *f[2] = {nullptr, nullptr};
    int cur = 0;            // f[cur] holds P_{t-1} (always 0 for the AA variant)
    int aa_phase = 0;       // AA variant (one lattice): 0 = A-form, next an A-step;
                            // 1 = B-form, next a B-step
    uint8_t *map = nullptr;
    void *rho = nullptr;
    void *u = nullptr;
    void *lid = nullptr;
    void *stage = nullptr;
    double *partials = nullptr;
    double *red_out = nullptr;
    int *status = nullptr;
    cudaStream_t stream = nullptr;
    // the iteration graphs' second branch (face-row launches beside the
    // interior-row launches) and its fork / join events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_first = nullptr, ev_last = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    std::vector<cudaEvent_t> spare;
    double kernels_ms = 0;
    int64_t it = 0;
    unsigned block = 128;
    unsigned nvec = 0;
    unsigned grid = 0;
    // staged variant (LBM_KERNEL_STAGED)
    int kernel = LBM_KERNEL_DIRECT;
    int rows = 1, gpp = 0, stages = 0;
    unsigned ngroups = 0, sgrid = 0, sblock = 0;
    size_t ssmem = 0;
    std::string device_name;
    int num_sms = 0;
    // lbm_step: graph_iters plain iterations captured once per starting
    // buffer parity and replayed (graph_iters = 1: no graphs)
    int graph_iters = 16;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    bool state_is_init = true;  // the populations are what lbm_init made
    size_t base_bytes = 0;      // device bytes lbm_init allocated
    lbm_adjoint_state adj;
};



namespace lbm {
// Makes the handle's device current for one entry point and restores the
// caller's device afterwards (handles of several devices may share a thread).
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev)
    {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};
// storage / macro / dump element sizes of a precision
inline size_t storage_bytes(int prec) { return prec == LBM_FP64 ? 8 : (prec == LBM_FP32 ? 4 : 2); }
inline size_t macro_bytes(int prec) { return prec == LBM_FP64 ? 8 : 4; }
// launch one iteration P_out = C(S(P_in)) with the handle's kernel variant
cudaError_t launch_iteration(const lbm_t *h, const void *fin, void *fout);
// the same iteration, also storing the adjoint's linearisation point of its
// input (MODE_STEP_ADJ: three planes of the compute type at `point`)
cudaError_t launch_iteration_adj(const lbm_t *h, const void *fin, void *fout, void *point);
// h->graph_iters iterations from h->f[h->cur] as one replayed CUDA graph
// (an even count: h->cur is unchanged)
cudaError_t replay_iterations(lbm_t *h);
// free the device memory of an adjoint state
void release_adjoint(lbm_t *h);
}  // namespace lbm
