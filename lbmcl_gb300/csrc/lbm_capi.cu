// lbm_capi.cu -- the extern "C" boundary (include/lbm.h): handle life cycle,
// device memory, the iteration loop, dumps, timing and reductions.
//
// Replaces the reference's OpenCL host plumbing of this path:
// buffer creation (lbmcl.hpp:403-417), the per-iteration kernel objects and
// the ping-pong argument swap (lbmcl.hpp:435-467), the enqueue loop
// (lbmcl.hpp:490-521), the blocking read-backs (lbmcl.hpp:159-277) and the
// event timing (lbmcl.hpp:548-593).  Failures return a status code and leave a
// message in lbm_last_error(); nothing here calls exit().
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "lbm.h"
#include "lbm_device.cuh"
#include "lbm_handle.h"
#include "lbm_launch.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define LBM_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            cudaGetLastError();                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA, "%s: %s", #call, \
                        cudaGetErrorString(e_));                                                \
        }                                                                                       \
    } while (0)

using lbm::macro_bytes;
using lbm::storage_bytes;
int vec_len(int prec) { return (int)(16 / storage_bytes(prec)); }
int dim_multiple(int prec) { return (prec == LBM_FP16 || prec == LBM_BF16) ? 8 : 4; }

constexpr size_t kStageElems = (size_t)1 << 25;  // dump / load staging, elements

__global__ void sum_partials_kernel(const double *__restrict__ partials, int nblocks, double *__restrict__ out)
{
    // one block of 256 threads, fixed summation order: deterministic
    double m = 0.0, e = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        m += partials[2 * i];
        e += partials[2 * i + 1];
    }
    __shared__ double sm[2][256];
    sm[0][threadIdx.x] = m;
    sm[1][threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sm[0][threadIdx.x] += sm[0][threadIdx.x + w];
            sm[1][threadIdx.x] += sm[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sm[0][0];
        out[1] = sm[1][0];
    }
}

}  // namespace

namespace lbm {
cudaError_t launch_sum_partials(const double *partials, int nblocks, double *out, cudaStream_t s)
{
    sum_partials_kernel<<<1, 256, 0, s>>>(partials, nblocks, out);
    return cudaGetLastError();
}

void set_last_error(const char *msg) { g_err = msg; }
}  // namespace lbm


namespace {

cudaError_t get_event(lbm_t *h, cudaEvent_t *ev)
{
    if (!h->spare.empty()) {
        *ev = h->spare.back();
        h->spare.pop_back();
        return cudaSuccess;
    }
    return cudaEventCreate(ev);
}

// Add the durations of finished event pairs to kernels_ms (in stream order).
int fold_events(lbm_t *h, bool wait)
{
    size_t k = 0;
    for (; k < h->pending.size(); ++k) {
        auto &p = h->pending[k];
        if (wait) {
            LBM_CUDA(cudaEventSynchronize(p.second));
        } else {
            cudaError_t q = cudaEventQuery(p.second);
            if (q == cudaErrorNotReady) break;
            LBM_CUDA(q);
        }
        float ms = 0;
        LBM_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
        h->kernels_ms += ms;
        h->spare.push_back(p.first);
        h->spare.push_back(p.second);
    }
    h->pending.erase(h->pending.begin(), h->pending.begin() + (ptrdiff_t)k);
    return LBM_OK;
}

void release(lbm_t *h)
{
    if (!h) return;
    const lbm::DeviceScope dev(h->cfg.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    lbm::release_adjoint(h);
    for (void *p : {h->f[0], h->f[1], (void *)h->map, h->rho, h->u, h->lid, h->stage, (void *)h->partials,
                    (void *)h->red_out, (void *)h->status})
        if (p) cudaFree(p);
    for (auto &p : h->pending) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    for (auto e : h->spare) cudaEventDestroy(e);
    for (cudaGraphExec_t &g : h->graph_exec)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    if (h->ev_first) cudaEventDestroy(h->ev_first);
    if (h->ev_last) cudaEventDestroy(h->ev_last);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

bool is_aa(const lbm_t *h) { return h->kernel == LBM_KERNEL_AA; }

// Iteration arguments from buffer `from` (two-lattice kernels) or of AA
// phase `phase` (the one lattice f[0]).
lbm::StepArgs step_args(const lbm_t *h, int from, int phase)
{
    lbm::StepArgs a;
    a.fin = is_aa(h) ? h->f[0] : h->f[from];
    a.fout = is_aa(h) ? h->f[0] : h->f[from ^ 1];
    a.aa_phase = phase;
    a.map = h->map;
    a.lid = h->lid;
    a.rho = h->rho;
    a.u = h->u;
    a.status = h->status;
    a.partials = h->partials;
    a.dim = h->dim;
    a.nvx = h->dim / h->V;
    a.nvec = h->nvec;
    a.n = h->n;
    a.inv_tau = h->inv_tau;
    a.omega_f = h->omega_f;
    a.rows = h->rows;
    a.gpp = h->gpp;
    a.ngroups = h->ngroups;
    a.stages = h->stages;
    a.sailfish = h->cfg.order == LBM_ORDER_SAILFISH ? 1 : 0;
    return a;
}
lbm::StepArgs step_args(const lbm_t *h, int from) { return step_args(h, from, h->aa_phase); }

// the buffer parity (two lattices) or phase (AA) of the current state, and
// its flip after one iteration
int parity(const lbm_t *h) { return is_aa(h) ? h->aa_phase : h->cur; }
void flip(lbm_t *h)
{
    if (is_aa(h)) h->aa_phase ^= 1;
    else h->cur ^= 1;
}
// layout of the current state for the dump / load kernels
int state_layout(const lbm_t *h)
{
    return is_aa(h) ? (h->aa_phase ? lbm::LAYOUT_AA_B : lbm::LAYOUT_AA_A) : lbm::LAYOUT_PULL;
}

const void *staged_ptr(int prec, int mode)
{
    switch (prec) {
    case LBM_FP32: return lbm::staged_kernel_ptr_f32(mode);
    case LBM_FP64: return lbm::staged_kernel_ptr_f64(mode);
    case LBM_FP16: return lbm::staged_kernel_ptr_f16(mode);
    default: return lbm::staged_kernel_ptr_bf16(mode);
    }
}

// Shape the staged variant: rows per group, ring depth, threads, persistent
// grid.  Returns false when the ring does not fit (the direct variant is used).
int setup_staged(lbm_t *h, int want_stages)
{
    const int dim = h->dim;
    const size_t sb = storage_bytes(h->prec);
    const int V = 4;
    const int nvx = dim / V;
    int rows = std::max(1, 512 / dim);
    rows = std::min(rows, dim - 2);
    const size_t stage_bytes = (size_t)lbm::Q * rows * dim * sb;
    int dev = 0, smem_optin = 0, nsm = 0;
    LBM_CUDA(cudaGetDevice(&dev));
    LBM_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    LBM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t cap = (size_t)smem_optin - 128;
    int stages = want_stages > 0 ? want_stages : (int)std::min<size_t>(8, std::max<size_t>(2, (110u << 10) / stage_bytes));
    while (stages > 2 && 128 + stages * stage_bytes > cap) --stages;
    if (stages < 2 || 128 + stages * stage_bytes > cap) return fail(LBM_EINVAL, "staged kernel: ring does not fit");
    const size_t smem = 128 + stages * stage_bytes;
    unsigned threads = (unsigned)std::min(256, ((rows * nvx + 31) / 32) * 32);
    int per_sm = 0;
    for (int mode : {lbm::MODE_STEP, lbm::MODE_STEP_MACRO}) {
        const void *k = staged_ptr(h->prec, mode);
        LBM_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    LBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, staged_ptr(h->prec, lbm::MODE_STEP),
                                                           (int)threads, smem));
    if (per_sm < 1) return fail(LBM_EINVAL, "staged kernel: no resident block");
    h->rows = rows;
    h->gpp = (dim - 2 + rows - 1) / rows;
    h->ngroups = (unsigned)h->gpp * (unsigned)(dim - 2);
    h->stages = stages;
    h->sblock = threads;
    h->ssmem = smem;
    h->sgrid = (unsigned)std::min<size_t>(h->ngroups, (size_t)per_sm * nsm);
    return LBM_OK;
}

cudaError_t launch_pull(const lbm_t *h, int mode, const lbm::StepArgs &a, unsigned *nparts = nullptr)
{
    if (h->kernel == LBM_KERNEL_AA) {
        switch (h->prec) {
        case LBM_FP32: return lbm::launch_aa_f32(mode, a, h->block, h->stream, nparts);
        case LBM_FP64: return lbm::launch_aa_f64(mode, a, h->block, h->stream, nparts);
        case LBM_FP16: return lbm::launch_aa_f16(mode, a, h->block, h->stream, nparts);
        default: return lbm::launch_aa_bf16(mode, a, h->block, h->stream, nparts);
        }
    }
    if (h->kernel == LBM_KERNEL_STAGED && (mode == lbm::MODE_STEP || mode == lbm::MODE_STEP_MACRO)) {
        switch (h->prec) {
        case LBM_FP32: return lbm::launch_staged_f32(mode, a, h->sgrid, h->sblock, h->ssmem, h->stream);
        case LBM_FP64: return lbm::launch_staged_f64(mode, a, h->sgrid, h->sblock, h->ssmem, h->stream);
        case LBM_FP16: return lbm::launch_staged_f16(mode, a, h->sgrid, h->sblock, h->ssmem, h->stream);
        default: return lbm::launch_staged_bf16(mode, a, h->sgrid, h->sblock, h->ssmem, h->stream);
        }
    }
    if (h->kernel == LBM_KERNEL_NARROW && mode != lbm::MODE_REDUCE) {
        switch (h->prec) {
        case LBM_FP32: return lbm::launch_narrow_f32(mode, a, h->block, h->stream);
        case LBM_FP16: return lbm::launch_narrow_f16(mode, a, h->block, h->stream);
        default: return lbm::launch_narrow_bf16(mode, a, h->block, h->stream);
        }
    }
    switch (h->prec) {
    case LBM_FP32: return lbm::launch_pull_f32(mode, a, h->block, h->stream, nparts);
    case LBM_FP64: return lbm::launch_pull_f64(mode, a, h->block, h->stream, nparts);
    case LBM_FP16: return lbm::launch_pull_f16(mode, a, h->block, h->stream, nparts);
    default: return lbm::launch_pull_bf16(mode, a, h->block, h->stream, nparts);
    }
}

size_t dump_elem(int prec) { return prec == LBM_FP64 ? 8 : 4; }

// true when one of the iterations it0 + 1 .. it0 + G stores the moments
bool macro_within(int64_t it0, int G, int macro_every)
{
    if (macro_every == 0) return false;
    const int64_t next = (it0 / macro_every + 1) * macro_every;  // first macro iteration after it0
    return next <= it0 + G;
}

bool splits(const lbm_t *h) { return h->kernel == LBM_KERNEL_DIRECT || h->kernel == LBM_KERNEL_NARROW; }

// One iteration (MODE_STEP or MODE_STEP_ADJ) of the direct / narrow variants
// with its face-row launch on the side stream, forked from and joined back
// into the handle's stream, so that (in a captured graph: as a second
// branch) it runs beside the interior-row launch; the two write disjoint rows
// of the output and read the same input.
cudaError_t split_iteration(const lbm_t *h, int mode, const lbm::StepArgs &a)
{
    cudaError_t e = cudaEventRecord(h->ev_fork, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->side, h->ev_fork, 0);
    if (e != cudaSuccess) return e;
    const int vb = h->kernel == LBM_KERNEL_NARROW ? 8 : 16;
    switch (h->prec) {
    case LBM_FP32: e = lbm::launch_split_f32(vb, mode, a, h->block, h->stream, h->side); break;
    case LBM_FP64: e = lbm::launch_split_f64(vb, mode, a, h->block, h->stream, h->side); break;
    case LBM_FP16: e = lbm::launch_split_f16(vb, mode, a, h->block, h->stream, h->side); break;
    default: e = lbm::launch_split_bf16(vb, mode, a, h->block, h->stream, h->side); break;
    }
    // join even after a failed launch, so the capture can end
    const cudaError_t ej = cudaEventRecord(h->ev_join, h->side);
    const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(h->stream, h->ev_join, 0) : ej;
    return e != cudaSuccess ? e : ew;
}

// Replay (capturing on first use) the graph of h->graph_iters plain
// iterations that starts from buffer h->cur.  The kernels' arguments are
// fixed per parity (the two buffers ping-pong), so two graphs cover every
// call.  With the direct / narrow kernels each iteration's face-row launch is
// a branch beside its interior-row launch.
cudaError_t replay_graph(lbm_t *h)
{
    cudaGraphExec_t &exec = h->graph_exec[parity(h)];
    if (!exec) {
        const bool split = splits(h);
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        int cur = h->cur, ph = h->aa_phase;
        for (int k = 0; k < h->graph_iters && e == cudaSuccess; ++k) {
            e = split ? split_iteration(h, lbm::MODE_STEP, step_args(h, cur, ph))
                      : launch_pull(h, lbm::MODE_STEP, step_args(h, cur, ph));
            if (is_aa(h)) ph ^= 1;
            else cur ^= 1;
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
        if (e == cudaSuccess) e = ec;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            exec = nullptr;
            return e;
        }
    }
    return cudaGraphLaunch(exec, h->stream);
}

}  // namespace

namespace lbm {
cudaError_t replay_iterations(lbm_t *h) { return replay_graph(h); }

cudaError_t launch_iteration(const lbm_t *h, const void *fin, void *fout)
{
    StepArgs a = step_args(h, h->cur);
    a.fin = fin;
    a.fout = fout;
    return splits(h) ? split_iteration(h, MODE_STEP, a) : launch_pull(h, MODE_STEP, a);
}

cudaError_t launch_iteration_adj(const lbm_t *h, const void *fin, void *fout, void *point)
{
    StepArgs a = step_args(h, h->cur);
    a.fin = fin;
    a.fout = fout;
    a.rho = nullptr;
    a.u = point;
    return splits(h) ? split_iteration(h, MODE_STEP_ADJ, a) : launch_pull(h, MODE_STEP_ADJ, a);
}
}  // namespace lbm

extern "C" {

void lbm_config_default(lbm_config *c)
{
    if (!c) return;
    memset(c, 0, sizeof *c);
    c->dim = 8;
    c->viscosity = 0.0089;
    c->velocity = 0.05;
    c->precision = LBM_FP32;
    c->stride = 32;
}

const char *lbm_last_error(void) { return g_err.c_str(); }

size_t lbm_size(const lbm_t *h, int what)
{
    if (!h) return 0;
    switch (what) {
    case LBM_DUMP_F: return (size_t)lbm::Q * h->n * dump_elem(h->prec);
    case LBM_DUMP_RHO: return h->n * macro_bytes(h->prec);
    case LBM_DUMP_U: return 3 * h->n * macro_bytes(h->prec);
    case LBM_DUMP_MAP: return h->n * sizeof(int32_t);
    case LBM_DUMP_MAP_U8: return h->n;
    case LBM_DUMP_F_RAW: return (size_t)lbm::Q * h->n * storage_bytes(h->prec);
    default: return 0;
    }
}

int lbm_init(lbm_t **out, const lbm_config *c)
{
    if (!out || !c) return fail(LBM_EINVAL, "lbm_init: NULL argument");
    *out = nullptr;
    if (c->precision < LBM_FP32 || c->precision > LBM_BF16)
        return fail(LBM_EINVAL, "lbm_init: unknown precision %d", c->precision);
    const int prec = c->precision;
    const int dim = c->dim;
    if (dim < 4 || dim % dim_multiple(prec) != 0 || dim > 2048)
        return fail(LBM_EINVAL, "lbm_init: dim %d must be in [4, 2048] and a multiple of %d for this precision", dim,
                    dim_multiple(prec));
    const size_t n = (size_t)dim * dim * dim;
    // CSoA stride of F dumps (kernels.cl:64): a power of two dividing dim^3;
    // 0 selects pure SoA, also for dims whose dim^3 is not a power of two
    // (sd = -1 then).
    const size_t stride = c->stride == 0 ? n : (size_t)c->stride;
    int sd = -1;
    if (c->stride < 0 || (c->stride > 0 && ((stride & (stride - 1)) != 0 || stride > n || n % stride != 0)))
        return fail(LBM_EINVAL, "lbm_init: stride %d must be a power of two dividing dim^3 (or 0 for SoA)",
                    c->stride);
    if ((stride & (stride - 1)) == 0) {
        sd = 0;
        while (((size_t)1 << sd) < stride) ++sd;
    }
    if (!(c->viscosity >= 0.0) && !(c->tau > 0.0))
        return fail(LBM_EINVAL, "lbm_init: viscosity must be >= 0");
    if (!std::isfinite(c->velocity)) return fail(LBM_EINVAL, "lbm_init: velocity must be finite");
    if (c->noise_sigma < 0.0 || !std::isfinite(c->noise_sigma))
        return fail(LBM_EINVAL, "lbm_init: noise_sigma must be finite and >= 0");
    if (c->kernel < LBM_KERNEL_AUTO || c->kernel > LBM_KERNEL_AA)
        return fail(LBM_EINVAL, "lbm_init: unknown kernel variant %d", c->kernel);
    if (c->stages < 0 || c->stages > 16) return fail(LBM_EINVAL, "lbm_init: stages %d out of range", c->stages);
    if (c->adjoint_steps < 0 || c->adjoint_steps > 2)
        return fail(LBM_EINVAL, "lbm_init: adjoint_steps %d out of range (0, 1, 2)", c->adjoint_steps);
    if (c->adjoint_max_states < 0)
        return fail(LBM_EINVAL, "lbm_init: adjoint_max_states %d must be >= 0", c->adjoint_max_states);
    if (c->adjoint_fp64 < 0 || c->adjoint_fp64 > 1)
        return fail(LBM_EINVAL, "lbm_init: adjoint_fp64 %d must be 0 or 1", c->adjoint_fp64);
    if (c->adjoint_full_states < 0 || c->adjoint_full_states > 1)
        return fail(LBM_EINVAL, "lbm_init: adjoint_full_states %d must be 0 or 1", c->adjoint_full_states);
    if (c->adjoint_kernel != LBM_KERNEL_AUTO && c->adjoint_kernel != LBM_KERNEL_DIRECT &&
        c->adjoint_kernel != LBM_KERNEL_STAGED)
        return fail(LBM_EINVAL, "lbm_init: adjoint_kernel %d must be 0, LBM_KERNEL_DIRECT or LBM_KERNEL_STAGED",
                    c->adjoint_kernel);
    if (c->adjoint_tail_segments < -1)
        return fail(LBM_EINVAL, "lbm_init: adjoint_tail_segments %d must be >= -1", c->adjoint_tail_segments);
    if (c->order < LBM_ORDER_REFERENCE || c->order > LBM_ORDER_SAILFISH)
        return fail(LBM_EINVAL, "lbm_init: unknown summation order %d", c->order);
    if (c->order == LBM_ORDER_SAILFISH && c->precision != LBM_FP32 && c->precision != LBM_FP64)
        return fail(LBM_EINVAL, "lbm_init: the Sailfish summation order needs FP32 or FP64 storage");
    if (c->graph_iterations < 0 || c->graph_iterations > 256 || (c->graph_iterations > 1 && c->graph_iterations % 2))
        return fail(LBM_EINVAL, "lbm_init: graph_iterations %d must be 0, 1 or an even number <= 256",
                    c->graph_iterations);
    if (c->block_threads < 0 || c->block_threads > 1024)
        return fail(LBM_EINVAL, "lbm_init: block_threads %d out of range", c->block_threads);
    if (c->lid_profile) {
        for (size_t k = 0; k < (size_t)dim * dim; ++k)
            if (!std::isfinite(c->lid_profile[k])) return fail(LBM_EINVAL, "lbm_init: lid_profile[%zu] not finite", k);
    }

    const int V = vec_len(prec);
    const size_t nvec = (size_t)(dim / V) * (size_t)(dim - 2) * (size_t)(dim - 2);
    unsigned block = c->block_threads > 0 ? (unsigned)(c->block_threads / 32 * 32) : 128u;
    if (block < 32) block = 32;
    // the iteration kernels' launch bounds: 128 threads for 16-bit storage
    const unsigned max_block = (prec == LBM_FP16 || prec == LBM_BF16) ? 128u : 256u;
    if (block > max_block) block = max_block;
    // reduction partials: one pair per block of the widest launch (the AA
    // variant's FP32 kernels use 8-byte vectors, twice the threads)
    const int Vr = (c->kernel == LBM_KERNEL_AA && prec == LBM_FP32) ? V / 2 : V;
    const size_t grid = ((size_t)(dim / Vr) * (size_t)(dim - 2) * (size_t)(dim - 2) + block - 1) / block;
    if (2 * nvec >= ((size_t)1 << 32)) return fail(LBM_EINVAL, "lbm_init: lattice too large");

    const size_t sb = storage_bytes(prec), mb = macro_bytes(prec);
    const size_t fbytes = (size_t)lbm::Q * n * sb;
    const size_t stage_elems = std::min(kStageElems, (size_t)lbm::Q * n);
    const bool aa = c->kernel == LBM_KERNEL_AA;  // one lattice
    const size_t need = (aa ? 1 : 2) * fbytes + n + 4 * n * mb + (size_t)dim * dim * mb + stage_elems * dump_elem(prec) +
                        (grid + 2) * 2 * sizeof(double) + 4 * sizeof(double) + sizeof(int);
    if (c->max_device_bytes > 0 && need > c->max_device_bytes)
        return fail(LBM_ENOMEM, "lbm_init: needs %zu device bytes, budget is %zu", need, c->max_device_bytes);

    lbm_t *h = new lbm_t();
    h->cfg = *c;
    h->cfg.lid_profile = nullptr;
    h->dim = dim;
    h->n = n;
    h->prec = prec;
    h->V = V;
    h->sd = sd;
    h->block = block;
    h->nvec = (unsigned)nvec;
    h->grid = (unsigned)grid;
    h->base_bytes = need;

    // tau = 3 nu + 0.5 and 1/tau in the compute precision (kernels.cl:61-62)
    if (prec == LBM_FP64) {
        const double tau = c->tau > 0 ? c->tau : (3.0 * c->viscosity) + 0.5;
        h->inv_tau = 1.0 / tau;
    } else {
        const float tau = c->tau > 0 ? (float)c->tau : (3.0f * (float)c->viscosity) + 0.5f;
        const float it = 1.0f / tau;
        h->inv_tau = (double)it;
    }
    h->omega_f = (float)h->inv_tau;
    if (!std::isfinite(h->inv_tau) || h->inv_tau <= 0)
        { release(h); return fail(LBM_EINVAL, "lbm_init: tau must be > 0"); }

    int rc = LBM_OK;
    auto setup = [&]() -> int {
        LBM_CUDA(cudaSetDevice(c->device));
        cudaDeviceProp prop;
        LBM_CUDA(cudaGetDeviceProperties(&prop, c->device));
        h->device_name = prop.name;
        h->num_sms = prop.multiProcessorCount;
        h->graph_iters = c->graph_iterations == 0 ? 16 : c->graph_iterations;
        LBM_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        LBM_CUDA(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        LBM_CUDA(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
        LBM_CUDA(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
        LBM_CUDA(cudaEventCreate(&h->ev_first));
        LBM_CUDA(cudaEventCreate(&h->ev_last));
        LBM_CUDA(cudaMalloc(&h->f[0], fbytes));
        if (!aa) LBM_CUDA(cudaMalloc(&h->f[1], fbytes));
        LBM_CUDA(cudaMalloc((void **)&h->map, n));
        LBM_CUDA(cudaMalloc(&h->rho, n * mb));
        LBM_CUDA(cudaMalloc(&h->u, 3 * n * mb));
        LBM_CUDA(cudaMalloc(&h->lid, (size_t)dim * dim * mb));
        LBM_CUDA(cudaMalloc(&h->stage, stage_elems * dump_elem(prec)));
        LBM_CUDA(cudaMalloc((void **)&h->partials, (grid + 2) * 2 * sizeof(double)));
        LBM_CUDA(cudaMalloc((void **)&h->red_out, 4 * sizeof(double)));
        LBM_CUDA(cudaMalloc((void **)&h->status, sizeof(int)));
        LBM_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), h->stream));

        // lid profile in the macro precision (the reference's VELOCITY is a
        // literal of the kernel's real type, lbmcl.hpp:141)
        std::vector<unsigned char> lidh((size_t)dim * dim * mb);
        for (size_t k = 0; k < (size_t)dim * dim; ++k) {
            const double v = c->lid_profile ? c->lid_profile[k] : c->velocity;
            if (mb == 8) memcpy(&lidh[k * 8], &v, 8);
            else { const float fv = (float)v; memcpy(&lidh[k * 4], &fv, 4); }
        }
        LBM_CUDA(cudaMemcpyAsync(h->lid, lidh.data(), lidh.size(), cudaMemcpyHostToDevice, h->stream));

        lbm::InitArgs ia;
        ia.f = h->f[0];
        ia.map = h->map;
        ia.lid = h->lid;
        ia.rho = h->rho;
        ia.u = h->u;
        ia.dim = dim;
        ia.n = n;
        ia.seed = c->seed;
        ia.noise_sigma = c->noise_sigma;
        ia.noise_sigma_f = (float)c->noise_sigma;
        ia.in_place = aa ? 1 : 0;
        LBM_CUDA(cudaEventRecord(h->ev_first, h->stream));
        switch (prec) {
        case LBM_FP32: LBM_CUDA(lbm::launch_init_f32(ia, h->stream)); break;
        case LBM_FP64: LBM_CUDA(lbm::launch_init_f64(ia, h->stream)); break;
        case LBM_FP16: LBM_CUDA(lbm::launch_init_f16(ia, h->stream)); break;
        default: LBM_CUDA(lbm::launch_init_bf16(ia, h->stream)); break;
        }
        LBM_CUDA(cudaEventRecord(h->ev_last, h->stream));
        // the copy source (lidh) must outlive the copy
        LBM_CUDA(cudaStreamSynchronize(h->stream));

        // iteration kernel: the fastest variant measured at 512^3 on GB300 --
        // 16-byte vectors for 16-bit storage and FP64, 8-byte vectors for FP32
        int want = c->kernel;
        if (want == LBM_KERNEL_AUTO) want = prec == LBM_FP32 ? LBM_KERNEL_NARROW : LBM_KERNEL_DIRECT;
        h->kernel = aa ? LBM_KERNEL_AA : LBM_KERNEL_DIRECT;
        if (want == LBM_KERNEL_NARROW && prec != LBM_FP64) {
            h->kernel = LBM_KERNEL_NARROW;
        }
        if (want == LBM_KERNEL_STAGED) {
            const int r = setup_staged(h, c->stages);
            if (r == LBM_OK) h->kernel = LBM_KERNEL_STAGED;
            else if (c->kernel == LBM_KERNEL_STAGED) return r;  // asked for explicitly
        }
        return LBM_OK;
    };
    rc = setup();
    if (rc != LBM_OK) {
        std::string msg = g_err;
        release(h);
        g_err = msg;
        return rc;
    }
    *out = h;
    return LBM_OK;
}

int lbm_step(lbm_t *h, int nsteps, int macro_every)
{
    if (!h) return fail(LBM_EINVAL, "lbm_step: NULL handle");
    const lbm::DeviceScope dev(h->cfg.device);
    if (nsteps < 0 || macro_every < 0) return fail(LBM_EINVAL, "lbm_step: nsteps and macro_every must be >= 0");
    if (nsteps == 0) return LBM_OK;
    h->state_is_init = false;
    h->adj.ready = false;
    int rc = fold_events(h, h->pending.size() > 4096);
    if (rc != LBM_OK) return rc;
    const bool per_step = h->cfg.profile_steps != 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!per_step) {
        LBM_CUDA(get_event(h, &e0));
        LBM_CUDA(get_event(h, &e1));
        LBM_CUDA(cudaEventRecord(e0, h->stream));
    }
    for (int k = 0; k < nsteps;) {
        // a run of graph_iters plain iterations (no macro output, no
        // per-iteration events) replays the captured graph of this parity
        const int G = h->graph_iters;
        if (!per_step && G > 1 && nsteps - k >= G && !macro_within(h->it, G, macro_every)) {
            LBM_CUDA(replay_graph(h));
            k += G;
            h->it += G;  // G is even: h->cur / h->aa_phase is unchanged
            continue;
        }
        ++k;
        const int64_t it = h->it + 1;
        const bool macro = macro_every != 0 && (it % macro_every) == 0;
        const lbm::StepArgs a = step_args(h, h->cur);
        cudaEvent_t s0 = nullptr, s1 = nullptr;
        if (per_step) {
            LBM_CUDA(get_event(h, &s0));
            LBM_CUDA(get_event(h, &s1));
            LBM_CUDA(cudaEventRecord(s0, h->stream));
        }
        LBM_CUDA(launch_pull(h, macro ? lbm::MODE_STEP_MACRO : lbm::MODE_STEP, a));
        if (per_step) {
            LBM_CUDA(cudaEventRecord(s1, h->stream));
            h->pending.emplace_back(s0, s1);
        }
        flip(h);
        h->it = it;
    }
    if (!per_step) {
        LBM_CUDA(cudaEventRecord(e1, h->stream));
        h->pending.emplace_back(e0, e1);
    }
    LBM_CUDA(cudaEventRecord(h->ev_last, h->stream));
    return LBM_OK;
}

int lbm_sync(lbm_t *h)
{
    if (!h) return fail(LBM_EINVAL, "lbm_sync: NULL handle");
    const lbm::DeviceScope dev(h->cfg.device);
    LBM_CUDA(cudaStreamSynchronize(h->stream));
    int st = 0;
    LBM_CUDA(cudaMemcpy(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st & 1) return fail(LBM_EDIVERGED, "lbm_sync: a density <= 0 or NaN was seen (simulation diverged)");
    if (st & 2) return fail(LBM_ETIMEOUT, "lbm_sync: a kernel's bounded wait expired; its results are not valid");
    return LBM_OK;
}

int lbm_dump(lbm_t *h, int what, void *dst, size_t bytes)
{
    if (!h || !dst) return fail(LBM_EINVAL, "lbm_dump: NULL argument");
    const lbm::DeviceScope dev(h->cfg.device);
    const size_t want = lbm_size(h, what);
    if (want == 0) return fail(LBM_EINVAL, "lbm_dump: unknown quantity %d", what);
    if (bytes != want) return fail(LBM_EINVAL, "lbm_dump: buffer is %zu bytes, quantity %d needs %zu", bytes, what, want);
    switch (what) {
    case LBM_DUMP_F: {
        const size_t te = dump_elem(h->prec);
        const size_t total = (size_t)lbm::Q * h->n;
        const size_t chunk = std::min(kStageElems, total);
        for (size_t o0 = 0; o0 < total; o0 += chunk) {
            lbm::DumpArgs a;
            a.f = h->f[h->cur];
            a.map = h->map;
            a.lid = h->lid;
            a.buf = h->stage;
            a.o0 = o0;
            a.count = std::min(chunk, total - o0);
            a.dim = h->dim;
            a.sd = h->sd;
            a.n = h->n;
            a.layout = state_layout(h);
            switch (h->prec) {
            case LBM_FP32: LBM_CUDA(lbm::launch_dump_f32(a, h->stream)); break;
            case LBM_FP64: LBM_CUDA(lbm::launch_dump_f64(a, h->stream)); break;
            case LBM_FP16: LBM_CUDA(lbm::launch_dump_f16(a, h->stream)); break;
            default: LBM_CUDA(lbm::launch_dump_bf16(a, h->stream)); break;
            }
            LBM_CUDA(cudaMemcpyAsync((char *)dst + o0 * te, h->stage, a.count * te, cudaMemcpyDeviceToHost, h->stream));
        }
        break;
    }
    case LBM_DUMP_RHO:
        LBM_CUDA(cudaMemcpyAsync(dst, h->rho, bytes, cudaMemcpyDeviceToHost, h->stream));
        break;
    case LBM_DUMP_U:
        LBM_CUDA(cudaMemcpyAsync(dst, h->u, bytes, cudaMemcpyDeviceToHost, h->stream));
        break;
    case LBM_DUMP_MAP_U8:
        LBM_CUDA(cudaMemcpyAsync(dst, h->map, bytes, cudaMemcpyDeviceToHost, h->stream));
        break;
    case LBM_DUMP_MAP: {
        std::vector<uint8_t> m(h->n);
        LBM_CUDA(cudaMemcpyAsync(m.data(), h->map, h->n, cudaMemcpyDeviceToHost, h->stream));
        LBM_CUDA(cudaStreamSynchronize(h->stream));
        int32_t *o = static_cast<int32_t *>(dst);
        for (size_t k = 0; k < h->n; ++k) o[k] = lbm::unpack_cell(m[k]);
        break;
    }
    case LBM_DUMP_F_RAW:
        LBM_CUDA(cudaMemcpyAsync(dst, h->f[h->cur], bytes, cudaMemcpyDeviceToHost, h->stream));
        break;
    }
    LBM_CUDA(cudaEventRecord(h->ev_last, h->stream));
    LBM_CUDA(cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

int lbm_load(lbm_t *h, int what, const void *src, size_t bytes)
{
    if (!h || !src) return fail(LBM_EINVAL, "lbm_load: NULL argument");
    const lbm::DeviceScope dev(h->cfg.device);
    if (what != LBM_DUMP_F && what != LBM_DUMP_F_RAW)
        return fail(LBM_EINVAL, "lbm_load: only LBM_DUMP_F and LBM_DUMP_F_RAW can be loaded");
    const size_t want = lbm_size(h, what);
    if (bytes != want) return fail(LBM_EINVAL, "lbm_load: buffer is %zu bytes, needs %zu", bytes, want);
    h->state_is_init = false;
    h->adj.ready = false;
    if (what == LBM_DUMP_F_RAW) {
        LBM_CUDA(cudaMemcpyAsync(h->f[h->cur], src, bytes, cudaMemcpyHostToDevice, h->stream));
    } else {
        const size_t te = dump_elem(h->prec);
        const size_t total = (size_t)lbm::Q * h->n;
        const size_t chunk = std::min(kStageElems, total);
        for (size_t o0 = 0; o0 < total; o0 += chunk) {
            lbm::DumpArgs a;
            a.f = h->f[h->cur];
            a.map = h->map;
            a.lid = h->lid;
            a.buf = h->stage;
            a.o0 = o0;
            a.count = std::min(chunk, total - o0);
            a.dim = h->dim;
            a.sd = h->sd;
            a.n = h->n;
            a.layout = state_layout(h);
            LBM_CUDA(cudaMemcpyAsync(h->stage, (const char *)src + o0 * te, a.count * te, cudaMemcpyHostToDevice,
                                     h->stream));
            switch (h->prec) {
            case LBM_FP32: LBM_CUDA(lbm::launch_load_f32(a, h->stream)); break;
            case LBM_FP64: LBM_CUDA(lbm::launch_load_f64(a, h->stream)); break;
            case LBM_FP16: LBM_CUDA(lbm::launch_load_f16(a, h->stream)); break;
            default: LBM_CUDA(lbm::launch_load_bf16(a, h->stream)); break;
            }
        }
    }
    LBM_CUDA(cudaEventRecord(h->ev_last, h->stream));
    LBM_CUDA(cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

int lbm_timing(lbm_t *h, double *total_ms, double *kernels_ms)
{
    if (!h) return fail(LBM_EINVAL, "lbm_timing: NULL handle");
    const lbm::DeviceScope dev(h->cfg.device);
    LBM_CUDA(cudaStreamSynchronize(h->stream));
    int rc = fold_events(h, true);
    if (rc != LBM_OK) return rc;
    float tot = 0;
    LBM_CUDA(cudaEventElapsedTime(&tot, h->ev_first, h->ev_last));
    if (total_ms) *total_ms = tot;
    if (kernels_ms) *kernels_ms = h->kernels_ms;
    return LBM_OK;
}

int lbm_iteration(const lbm_t *h, int64_t *it)
{
    if (!h || !it) return fail(LBM_EINVAL, "lbm_iteration: NULL argument");
    *it = h->it;
    return LBM_OK;
}

void *lbm_stream(lbm_t *h) { return h ? (void *)h->stream : nullptr; }

const char *lbm_device_name(const lbm_t *h) { return h ? h->device_name.c_str() : ""; }

int lbm_reduce(lbm_t *h, double out[3])
{
    if (!h || !out) return fail(LBM_EINVAL, "lbm_reduce: NULL argument");
    const lbm::DeviceScope dev(h->cfg.device);
    const lbm::StepArgs a = step_args(h, h->cur);
    unsigned nparts = 0;
    LBM_CUDA(launch_pull(h, lbm::MODE_REDUCE, a, &nparts));
    LBM_CUDA(lbm::launch_sum_partials(h->partials, (int)nparts, h->red_out, h->stream));
    double r[2];
    LBM_CUDA(cudaMemcpyAsync(r, h->red_out, sizeof r, cudaMemcpyDeviceToHost, h->stream));
    LBM_CUDA(cudaEventRecord(h->ev_last, h->stream));
    LBM_CUDA(cudaStreamSynchronize(h->stream));
    const double d4 = (double)(h->dim - 4);
    out[0] = r[0];
    out[1] = r[1];
    out[2] = d4 * d4 * d4 + d4 * d4;  // FLUID (dim-4)^3 + MOVING (dim-4)^2
    return LBM_OK;
}

void lbm_destroy(lbm_t *h) { release(h); }

}  // extern "C"
