// lbm_adjoint_host.cu -- gradients of a mid-plane velocity loss with respect
// to the lid-velocity profile, the relaxation time and the initial
// populations (lbm_adjoint_* in include/lbm.h).
//
// lbm_adjoint_forward runs T iterations from the handle's current state,
// keeping checkpoints Q_0, Q_c, Q_2c, ... of the P buffer (c = checkpoint
// interval; c = 1 keeps the whole trajectory).  lbm_adjoint_backward seeds
// a_T = dJ/dR_T, then walks the segments backwards: it restores a
// checkpoint, recomputes the segment's intermediate states with the forward
// kernel, and applies the adjoint step from the segment's last iteration to
// its first, two steps per launch for the FP32 adjoint (a segment of odd
// length ends with one single step).  When the segment's states do not fit
// in device memory, the segment itself is checkpointed and swept recursively
// (one more forward pass per level).  Memory: ceil(T/c) checkpoints + (c - 1) segment states, i.e.
// about 2 sqrt(T) states for c = sqrt(T); one extra forward iteration per
// iteration of the backward sweep.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include <cudaTypedefs.h>

#include "lbm.h"
#include "lbm_adjoint.cuh"
#include "lbm_handle.h"
#include "lbm_launch.h"

namespace {

constexpr unsigned kAdjBlock = 128;
constexpr unsigned kLossBlock = 256;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    lbm::set_last_error(buf);
    return code;
}

#define ADJ_CUDA(call)                                                                               \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            cudaGetLastError();                                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA, "%s: %s", #call,   \
                        cudaGetErrorString(e_));                                                     \
        }                                                                                            \
    } while (0)

// FP64 adjoint arithmetic: FP64 storage, or asked for (lbm_config.adjoint_fp64)
bool adj64(const lbm_t *h) { return h->prec == LBM_FP64 || h->cfg.adjoint_fp64 != 0; }
size_t adj_bytes(const lbm_t *h) { return adj64(h) ? 8 : 4; }
// adjoint kernels: 2 sites per thread (8-byte FP32 / 16-byte FP64 vectors)
constexpr int kAdjV = 2;

// blocks of the interior-row and face-row adjoint launches
void adj_grids(const lbm_t *h, unsigned &gi, unsigned &gf)
{
    const size_t nvx = (size_t)(h->dim / kAdjV);
    const size_t m = (size_t)(h->dim - 4);
    gi = (unsigned)((m * m * nvx + kAdjBlock - 1) / kAdjBlock);
    gf = (unsigned)((4 * (size_t)(h->dim - 3) * nvx + kAdjBlock - 1) / kAdjBlock);
}

lbm::AdjArgs adj_args(const lbm_t *h)
{
    lbm::AdjArgs a = {};
    a.map = h->map;
    a.lid = h->lid;
    a.grad_lid = h->adj.grad_lid;
    a.tau_acc = h->adj.tau_acc;
    a.target = h->adj.target;
    a.dim = h->dim;
    a.nvx = h->dim / kAdjV;
    a.nvec = (unsigned)((size_t)a.nvx * (size_t)(h->dim - 2) * (size_t)(h->dim - 2));
    a.n = h->n;
    a.omega = h->inv_tau;
    a.plane_y = h->adj.plane_y;
    return a;
}

template <class S, bool MACRO>
cudaError_t run_adjoint_step(const lbm::AdjArgs &a0, unsigned gi, unsigned gf, cudaStream_t s)
{
    using A = typename lbm::AdjType<S>::type;
    constexpr int VB = kAdjV * (int)sizeof(A);
    lbm::AdjArgs a = a0;
    if (gi > 0) {
        a.tau_base = 0;
        lbm::adjoint_kernel<S, A, VB, lbm::ROWS_INTERIOR, MACRO><<<gi, kAdjBlock, 0, s>>>(a);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    a.tau_base = gi;
    lbm::adjoint_kernel<S, A, VB, lbm::ROWS_FACES, MACRO><<<gf, kAdjBlock, 0, s>>>(a);
    return cudaGetLastError();
}
template <class S>
cudaError_t run_loss_seed(const lbm::AdjArgs &a, unsigned grid, cudaStream_t s)
{
    lbm::loss_seed_kernel<S, typename lbm::AdjType<S>::type><<<grid, kLossBlock, 0, s>>>(a);
    return cudaGetLastError();
}
template <class S>
cudaError_t run_lid_init_grad(const lbm::AdjArgs &a, cudaStream_t s)
{
    const int nc = a.dim * a.dim;
    lbm::lid_init_grad_kernel<S, typename lbm::AdjType<S>::type><<<(nc + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

// ---- two steps per launch (FP32 adjoint)
// z-planes per block (measured at 256^3: 16, 24, 32, 48 -> 24 best by 2%)
#ifndef LBM_ADJ2_CHUNK
#define LBM_ADJ2_CHUNK 24
#endif
constexpr int kAdj2Chunk = LBM_ADJ2_CHUNK;

// blocks of the two-step launch (macro: the stored-point kernel's taller tiles)
unsigned adj2_grid(const lbm_t *h, int &ntx, int &nty, bool macro)
{
    const int m = h->dim - 2;
    const int ty = (macro ? lbm::adj2_ey<true>() : lbm::adj2_ey<false>()) - 2;
    ntx = (m + lbm::ADJ2_TX - 1) / lbm::ADJ2_TX;
    nty = (m + ty - 1) / ty;
    const int ntz = (m + kAdj2Chunk - 1) / kAdj2Chunk;
    return (unsigned)ntx * (unsigned)nty * (unsigned)ntz;
}

// Two steps per launch for the FP32 adjoint (adjoint_steps 0 or 2), up to
// ADJ2_MAX_DIM.  By default only where its grid gives every SM two blocks or
// more: a small lattice (64^3: 66 blocks) runs faster one step at a time.
bool two_step(const lbm_t *h)
{
    if (adj64(h) || h->cfg.adjoint_steps == 1 || h->dim > lbm::ADJ2_MAX_DIM) return false;
    if (h->cfg.adjoint_steps == 2) return true;
    int ntx, nty;
    return adj2_grid(h, ntx, nty, false) >= 2u * (unsigned)std::max(h->num_sms, 1);
}

template <class S, bool MACRO>
cudaError_t run_adjoint2(const lbm::Adj2Args &a, unsigned grid, cudaStream_t s)
{
    lbm::adjoint2_kernel<S, MACRO>
        <<<grid, lbm::ADJ2_EX * lbm::adj2_ey<MACRO>(), lbm::adj2_smem_bytes<MACRO>(), s>>>(a);
    return cudaGetLastError();
}

template <class S>
cudaError_t set_adjoint2_smem()
{
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(lbm::adjoint2_kernel<S, false>, at, (int)lbm::adj2_smem_bytes<false>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(lbm::adjoint2_kernel<S, true>, at, (int)lbm::adj2_smem_bytes<true>());
    return e;
}

// ---- TMA-staged stored-point two-step kernel
// cuTensorMapEncodeTiled, looked up once through the runtime (the library
// does not link against the driver library)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A (dim, dim, dim, planes) float tensor at base with 40 x 8 x 1 x 1 boxes;
// coordinates outside it read as zeros.  Needs dim % 4 == 0 (row strides of
// 16-byte multiples) and a 16-byte aligned base.
bool adj2t_map(CUtensorMap *m, const void *base, int dim, int planes)
{
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t d = (cuuint64_t)dim;
    const cuuint64_t gdim[4] = {d, d, d, (cuuint64_t)planes};
    const cuuint64_t gstride[3] = {d * 4, d * d * 4, d * d * d * 4};
    const cuuint32_t box[4] = {(cuuint32_t)lbm::ADJ2T_BW, (cuuint32_t)lbm::ADJ2_EY, 1, 1};
    const cuuint32_t estride[4] = {1, 1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void *>(base), gdim, gstride, box, estride,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The staged kernel runs the stored-point pairs of steps when asked for
// (lbm_config.adjoint_kernel = LBM_KERNEL_STAGED); it needs dim % 4 == 0
// (always true of FP32 / FP16 / BF16 handles) and the driver's tensor maps.
// Not the default: at two blocks per SM (its shared memory) it measured 4%
// slower per backward iteration than the per-thread-load kernel at four
// (256^3 FP16: 0.651 against 0.625 ms), bound by its per-plane barrier.
bool adj2_staged(const lbm_t *h)
{
    return h->cfg.adjoint_kernel == LBM_KERNEL_STAGED && lbm::adj2_ey<true>() == lbm::ADJ2_EY && h->dim % 4 == 0 &&
           tensor_map_encoder() != nullptr;
}

// The two-step kernels' shared-memory size, set at the start of every
// backward sweep (outside any graph capture): the attribute belongs to the
// current device's context, and handles may live on different devices.
cudaError_t prepare_adjoint2(const lbm_t *h)
{
    if (h->prec != LBM_FP64) {
        const cudaError_t e = cudaFuncSetAttribute(lbm::adjoint2_tma_kernel<lbm::ADJ2T_NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)lbm::adj2t_smem_bytes());
        if (e != cudaSuccess) return e;
    }
    switch (h->prec) {
    case LBM_FP32: return set_adjoint2_smem<float>();
    case LBM_FP16: return set_adjoint2_smem<__half>();
    case LBM_BF16: return set_adjoint2_smem<__nv_bfloat16>();
    default: return cudaSuccess;
    }
}

// a_{k+1} -> a_{k-1} with Q_k (fwd_a) and Q_{k-1} (fwd_b), or with their
// stored linearisation points (macro)
cudaError_t adjoint_two_steps(const lbm_t *h, const void *fwd_a, const void *fwd_b, const void *ain, void *aout,
                              bool macro)
{
    lbm::Adj2Args a = {};
    a.fwd_a = fwd_a;
    a.fwd_b = fwd_b;
    a.ain = static_cast<const float *>(ain);
    a.aout = static_cast<float *>(aout);
    a.map = h->map;
    a.lid = h->lid;
    a.grad_lid = h->adj.grad_lid;
    a.tau_acc = h->adj.tau_acc;
    a.dim = h->dim;
    a.zc = kAdj2Chunk;
    for (int i = 0; i < lbm::Q; ++i) {
        const long long sh = lbm::ex_of(i) + (long long)lbm::ey_of(i) * h->dim +
                             (long long)lbm::ez_of(i) * h->dim * h->dim;
        const unsigned long long base = (unsigned long long)i * h->n;
        a.off_up[i] = (unsigned)(base + (unsigned long long)sh);
        a.off_down[i] = (unsigned)(base - (unsigned long long)sh);
        a.off_own[i] = (unsigned)base;
    }
    a.omega = (float)h->inv_tau;
    a.status = h->status;
    const unsigned grid = adj2_grid(h, a.ntx, a.nty, macro);
    if (macro && adj2_staged(h)) {
        CUtensorMap ma, mpa, mpb;
        if (!adj2t_map(&ma, ain, h->dim, lbm::Q) || !adj2t_map(&mpa, fwd_a, h->dim, 3) ||
            !adj2t_map(&mpb, fwd_b, h->dim, 3))
            return cudaErrorInvalidValue;
        lbm::adjoint2_tma_kernel<lbm::ADJ2T_NS><<<grid, lbm::ADJ2_EX * lbm::ADJ2_EY, lbm::adj2t_smem_bytes(), h->stream>>>(ma, mpa,
                                                                                                           mpb, a);
        return cudaGetLastError();
    }
    switch (h->prec) {
    case LBM_FP32: return macro ? run_adjoint2<float, true>(a, grid, h->stream) : run_adjoint2<float, false>(a, grid, h->stream);
    case LBM_FP16:
        return macro ? run_adjoint2<__half, true>(a, grid, h->stream) : run_adjoint2<__half, false>(a, grid, h->stream);
    default:
        return macro ? run_adjoint2<__nv_bfloat16, true>(a, grid, h->stream)
                     : run_adjoint2<__nv_bfloat16, false>(a, grid, h->stream);
    }
}

template <class S>
cudaError_t run_adjoint_step_any(const lbm::AdjArgs &a, unsigned gi, unsigned gf, cudaStream_t s, bool macro)
{
    return macro ? run_adjoint_step<S, true>(a, gi, gf, s) : run_adjoint_step<S, false>(a, gi, gf, s);
}

cudaError_t adjoint_step(const lbm_t *h, const lbm::AdjArgs &a, bool macro)
{
    unsigned gi, gf;
    adj_grids(h, gi, gf);
    if (adj64(h) && h->prec != LBM_FP64)
        return lbm::launch_adjoint_step_a64(h->prec, a, gi, gf, kAdjBlock, h->stream, macro);
    switch (h->prec) {
    case LBM_FP32: return run_adjoint_step_any<float>(a, gi, gf, h->stream, macro);
    case LBM_FP64: return run_adjoint_step_any<double>(a, gi, gf, h->stream, macro);
    case LBM_FP16: return run_adjoint_step_any<__half>(a, gi, gf, h->stream, macro);
    default: return run_adjoint_step_any<__nv_bfloat16>(a, gi, gf, h->stream, macro);
    }
}

cudaError_t loss_seed(const lbm_t *h, const lbm::AdjArgs &a)
{
    if (adj64(h) && h->prec != LBM_FP64)
        return lbm::launch_loss_seed_a64(h->prec, a, h->adj.loss_grid, kLossBlock, h->stream);
    switch (h->prec) {
    case LBM_FP32: return run_loss_seed<float>(a, h->adj.loss_grid, h->stream);
    case LBM_FP64: return run_loss_seed<double>(a, h->adj.loss_grid, h->stream);
    case LBM_FP16: return run_loss_seed<__half>(a, h->adj.loss_grid, h->stream);
    default: return run_loss_seed<__nv_bfloat16>(a, h->adj.loss_grid, h->stream);
    }
}

cudaError_t lid_init_grad(const lbm_t *h, const lbm::AdjArgs &a)
{
    if (adj64(h) && h->prec != LBM_FP64) return lbm::launch_lid_init_grad_a64(h->prec, a, h->stream);
    switch (h->prec) {
    case LBM_FP32: return run_lid_init_grad<float>(a, h->stream);
    case LBM_FP64: return run_lid_init_grad<double>(a, h->stream);
    case LBM_FP16: return run_lid_init_grad<__half>(a, h->stream);
    default: return run_lid_init_grad<__nv_bfloat16>(a, h->stream);
    }
}

// number of FLUID sites on the loss plane
double plane_sites(const lbm_t *h)
{
    const int y = h->adj.plane_y;
    if (y < 2 || y > h->dim - 3) return 0.0;
    const double m = (double)(h->dim - 4);
    return m * m;
}

// Device allocation counted against the handle's max_device_bytes budget.
int alloc_tracked(lbm_t *h, void **p, size_t bytes)
{
    const size_t cap = h->cfg.max_device_bytes;
    if (cap > 0 && h->base_bytes + h->adj.bytes + bytes > cap)
        return fail(LBM_ENOMEM, "adjoint: needs %zu more device bytes, budget is %zu", bytes, cap);
    ADJ_CUDA(cudaMalloc(p, bytes));
    h->adj.bytes += bytes;
    return LBM_OK;
}

// Device bytes the adjoint may still take: free memory less a margin for the
// runtime and other users, within the handle's budget.
size_t device_room(const lbm_t *h)
{
    size_t freeb = 0, totalb = 0;
    if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) return 0;
    const size_t margin = ((size_t)1 << 30) + totalb / 50;
    size_t r = freeb > margin ? freeb - margin : 0;
    const size_t cap = h->cfg.max_device_bytes;
    if (cap > 0) {
        const size_t used = h->base_bytes + h->adj.bytes;
        r = std::min(r, cap > used ? cap - used : (size_t)0);
    }
    return r;
}

void drop_segment_graphs(lbm_adjoint_state &s)
{
    for (cudaGraphExec_t &g : s.seg_exec)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    s.seg_graph_c = 0;
}

void free_tracked(lbm_t *h, void *p, size_t bytes)
{
    if (!p) return;
    cudaFree(p);
    h->adj.bytes -= bytes;
}

// the linearisation points the adjoint forward recorded for its last segments
void free_tail_points(lbm_t *h)
{
    free_tracked(h, h->adj.tail_block, h->adj.tail_bytes);
    h->adj.tail_block = nullptr;
    h->adj.tail_bytes = 0;
    h->adj.tpts.clear();
    h->adj.tail_k0 = h->adj.iterations;
}

// The adjoint steps k = start + len - 1 .. start with Q_k (or, macro, its
// stored linearisation point) given by state(k).
template <class State>
int adjoint_steps_down(lbm_t *h, int start, int len, State state, int &cur, bool macro = false)
{
    lbm_adjoint_state &s = h->adj;
    int k = start + len - 1;
    if (two_step(h)) {
        for (; k - 1 >= start; k -= 2) {
            ADJ_CUDA(adjoint_two_steps(h, state(k), state(k - 1), s.adj[cur], s.adj[cur ^ 1], macro));
            cur ^= 1;
        }
    }
    for (; k >= start; --k) {
        lbm::AdjArgs b = adj_args(h);
        b.fwd = state(k);
        b.ain = s.adj[cur];
        b.aout = s.adj[cur ^ 1];
        ADJ_CUDA(adjoint_step(h, b, macro));
        cur ^= 1;
    }
    return LBM_OK;
}

// Backward sweep over the iterations [start, start + len) from Q_start in q0,
// storing linearisation points only: len iterations recomputed from q0 (the
// states ping-pong through s.mtmp) write the point of each iteration k into
// s.mseg[k - start], then the adjoint steps read them.  Needs len <= mseg.
int sweep_macro(lbm_t *h, const void *q0, int start, int len, int &cur)
{
    lbm_adjoint_state &s = h->adj;
    const void *in = q0;
    for (int m = 0; m < len; ++m) {
        void *out = s.mtmp[m & 1];
        ADJ_CUDA(lbm::launch_iteration_adj(h, in, out, s.mseg[m]));
        in = out;
    }
    return adjoint_steps_down(h, start, len, [&](int k) -> const void * { return s.mseg[k - start]; }, cur, true);
}

// Backward sweep over the iterations [start, start + len), Q_start in q0,
// with the state buffers pool[p0, p1) free.  When len - 1 buffers are free
// the segment is recomputed and stored whole; otherwise the sweep keeps
// sub-checkpoints every c2 iterations (c2 = ceil(sqrt(len)), wider when the
// pool is short) and recurses into the sub-segments, last to first:
// multi-level checkpointing, one more forward pass per level.
int sweep(lbm_t *h, const void *q0, int start, int len, const std::vector<void *> &pool, int p0, int p1, int &cur)
{
    const int nfree = p1 - p0;
    if (len - 1 <= nfree) {
        for (int m = 1; m < len; ++m)
            ADJ_CUDA(lbm::launch_iteration(h, m == 1 ? q0 : pool[p0 + m - 2], pool[p0 + m - 1]));
        return adjoint_steps_down(h, start, len, [&](int k) -> const void * {
            return k == start ? q0 : pool[p0 + (k - start) - 1];
        }, cur);
    }
    if (nfree < 2)
        return fail(LBM_ENOMEM, "adjoint: %d free state buffers are too few for a segment of %d iterations", nfree,
                    len);
    if (nfree < 4) {
        // two buffers: every state recomputed from q0 (len^2 / 2 iterations)
        void *tmp[2] = {pool[p0], pool[p0 + 1]};
        auto advance = [&](int to, const void *&at, int &t) -> int {  // to >= t
            for (; t < to; ++t) {
                void *out = at == tmp[0] ? tmp[1] : tmp[0];
                ADJ_CUDA(lbm::launch_iteration(h, at, out));
                at = out;
            }
            return LBM_OK;
        };
        int k = start + len - 1;
        while (k >= start) {
            const void *at = q0;
            int t = start;
            const bool pair = two_step(h) && k - 1 >= start;
            int rc = advance(pair ? k - 1 : k, at, t);
            if (rc != LBM_OK) return rc;
            if (pair) {
                const void *prev = at;
                rc = advance(k, at, t);
                if (rc != LBM_OK) return rc;
                rc = adjoint_steps_down(h, k - 1, 2, [&](int i) -> const void * { return i == k ? at : prev; }, cur);
                k -= 2;
            } else {
                rc = adjoint_steps_down(h, k, 1, [&](int) -> const void * { return at; }, cur);
                k -= 1;
            }
            if (rc != LBM_OK) return rc;
        }
        return LBM_OK;
    }
    // m sub-checkpoints after q0, two buffers left for the sub-segments
    int c2 = (int)std::ceil(std::sqrt((double)len));
    int m = (len + c2 - 1) / c2 - 1;
    if (m > nfree - 2) {
        m = nfree - 2;
        c2 = (len + m) / (m + 1);
        m = (len + c2 - 1) / c2 - 1;
    }
    // advance from q0, writing sub-checkpoint i (iteration start + i c2) into
    // pool[p0 + i - 1] and the iterations between into two scratch buffers
    void *tmp[2] = {pool[p0 + m], pool[p0 + m + 1]};
    const void *at = q0;
    for (int t = 1; t <= m * c2; ++t) {
        void *out = (t % c2 == 0) ? pool[p0 + t / c2 - 1] : (at == tmp[0] ? tmp[1] : tmp[0]);
        ADJ_CUDA(lbm::launch_iteration(h, at, out));
        at = out;
    }
    for (int i = m; i >= 0; --i) {
        const void *q = i == 0 ? q0 : pool[p0 + i - 1];
        const int rc = sweep(h, q, start + i * c2, std::min(c2, len - i * c2), pool, p0 + m, p1, cur);
        if (rc != LBM_OK) return rc;
    }
    return LBM_OK;
}

// One full segment of the one-level sweep (c - 1 recomputed iterations
// from the staged first state s.q0, then its c adjoint steps) as a captured
// CUDA graph, replayed for every full segment: the launches of a launch-bound
// small lattice cost one graph launch.  One graph per adjoint-buffer parity.
int replay_segment(lbm_t *h, int c, int &cur, bool macro)
{
    lbm_adjoint_state &s = h->adj;
    cudaGraphExec_t &exec = s.seg_exec[cur];
    if (!exec) {
        ADJ_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int c2 = cur, rc = LBM_OK;
        if (macro) {
            rc = sweep_macro(h, s.q0, 0, c, c2);
        } else {
            for (int m = 1; m < c && rc == LBM_OK; ++m) {
                const cudaError_t e = lbm::launch_iteration(h, m == 1 ? s.q0 : s.seg[m - 2], s.seg[m - 1]);
                if (e != cudaSuccess) rc = fail(LBM_ECUDA, "segment capture: %s", cudaGetErrorString(e));
            }
            if (rc == LBM_OK)
                rc = adjoint_steps_down(h, 0, c, [&](int k) -> const void * { return k == 0 ? s.q0 : s.seg[k - 1]; },
                                        c2);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
        if (rc == LBM_OK && ec != cudaSuccess) rc = fail(LBM_ECUDA, "segment capture: %s", cudaGetErrorString(ec));
        if (rc == LBM_OK) {
            const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
            if (ei != cudaSuccess) {
                exec = nullptr;
                rc = fail(LBM_ECUDA, "segment graph: %s", cudaGetErrorString(ei));
            }
        }
        if (g) cudaGraphDestroy(g);
        if (rc != LBM_OK) return rc;
        s.seg_flip[cur] = c2 ^ cur;
    }
    ADJ_CUDA(cudaGraphLaunch(exec, h->stream));
    cur ^= s.seg_flip[cur];
    return LBM_OK;
}

}  // namespace

namespace lbm {
void release_adjoint(lbm_t *h)
{
    lbm_adjoint_state &s = h->adj;
    for (void *p : s.ckpt) cudaFree(p);
    for (void *p : s.seg) cudaFree(p);
    for (void *p : s.mseg) cudaFree(p);
    if (s.tail_block) cudaFree(s.tail_block);
    s.tail_block = nullptr;
    s.tail_bytes = 0;
    s.ckpt.clear();
    s.seg.clear();
    s.mseg.clear();
    s.tpts.clear();
    for (void *&p : s.mtmp) {
        if (p) cudaFree(p);
        p = nullptr;
    }
    for (void *&p : s.adj) {
        if (p) cudaFree(p);
        p = nullptr;
    }
    for (void *p : {(void *)s.grad_lid, (void *)s.tau_acc, (void *)s.loss_part, s.target, s.q0})
        if (p) cudaFree(p);
    s.q0 = nullptr;
    drop_segment_graphs(s);
    s.grad_lid = nullptr;
    s.tau_acc = nullptr;
    s.loss_part = nullptr;
    s.target = nullptr;
    s.bytes = 0;
    s.ready = false;
}
}  // namespace lbm

extern "C" {

int lbm_adjoint_set_loss(lbm_t *h, int plane_y, const double *target_ux)
{
    if (!h) return fail(LBM_EINVAL, "lbm_adjoint_set_loss: NULL handle");
    const lbm::DeviceScope dev(h->cfg.device);
    if (plane_y < 2 || plane_y > h->dim - 3)
        return fail(LBM_EINVAL, "lbm_adjoint_set_loss: plane_y %d must hold FLUID sites ([2, %d])", plane_y,
                    h->dim - 3);
    const size_t nc = (size_t)h->dim * h->dim;
    const size_t ab = adj_bytes(h);
    if (!h->adj.target) {
        int rc = alloc_tracked(h, &h->adj.target, nc * ab);
        if (rc != LBM_OK) return rc;
    }
    std::vector<unsigned char> buf(nc * ab);
    for (size_t k = 0; k < nc; ++k) {
        const double v = target_ux ? target_ux[k] : 0.0;
        if (ab == 8) memcpy(&buf[k * 8], &v, 8);
        else { const float f = (float)v; memcpy(&buf[k * 4], &f, 4); }
    }
    ADJ_CUDA(cudaMemcpyAsync(h->adj.target, buf.data(), buf.size(), cudaMemcpyHostToDevice, h->stream));
    ADJ_CUDA(cudaStreamSynchronize(h->stream));
    h->adj.plane_y = plane_y;
    // a new loss invalidates the recorded forward (its loss value belongs to
    // the old plane / target) and the captured segment graphs with it
    drop_segment_graphs(h->adj);
    h->adj.ready = false;
    return LBM_OK;
}

int lbm_adjoint_forward(lbm_t *h, int iterations, int checkpoint_every, double *loss)
{
    if (!h) return fail(LBM_EINVAL, "lbm_adjoint_forward: NULL handle");
    const lbm::DeviceScope dev(h->cfg.device);
    if (iterations < 1 || checkpoint_every < 1)
        return fail(LBM_EINVAL, "lbm_adjoint_forward: iterations and checkpoint_every must be >= 1");
    if (h->adj.plane_y < 0) return fail(LBM_ESTATE, "lbm_adjoint_forward: call lbm_adjoint_set_loss first");
    if (h->kernel == LBM_KERNEL_AA)
        return fail(LBM_ESTATE, "lbm_adjoint_forward: the adjoint needs the two-lattice kernels "
                                "(LBM_KERNEL_AA keeps one lattice in place)");
    if (h->cfg.order != LBM_ORDER_REFERENCE)
        return fail(LBM_ESTATE, "lbm_adjoint_forward: the adjoint is linearised in the reference summation "
                                "order (lbm_config.order = LBM_ORDER_REFERENCE)");
    lbm_adjoint_state &s = h->adj;
    const size_t fbytes = (size_t)lbm::Q * h->n * lbm::storage_bytes(h->prec);
    // drop the previous run's state buffers (the target and work buffers
    // stay) and the segment graphs that point at them
    for (void *p : s.ckpt) free_tracked(h, p, fbytes);
    for (void *p : s.seg) free_tracked(h, p, fbytes);
    s.ckpt.clear();
    s.seg.clear();
    free_tail_points(h);
    drop_segment_graphs(s);
    s.ready = false;
    const int c = std::min(checkpoint_every, iterations);
    const int nck = (iterations + c - 1) / c;
    for (int k = 0; k < nck; ++k) {
        void *p = nullptr;
        int rc = alloc_tracked(h, &p, fbytes);
        if (rc != LBM_OK) return rc;
        s.ckpt.push_back(p);
    }
    s.iterations = iterations;
    s.every = c;
    s.init_state = h->state_is_init;

    // The last mt segments record their linearisation points here (the
    // stored-point backward sweep then skips recomputing them): as many as
    // fit in the device memory left once the sweep's own buffers (c point
    // sets, two state scratch buffers, the staged checkpoint, the two adjoint
    // buffers) are set aside.
    const size_t mbytes = 3 * h->n * lbm::macro_bytes(h->prec);
    int mt = 0;
    if (h->cfg.adjoint_tail_segments >= 0) {
        const size_t abytes = (size_t)lbm::Q * h->n * adj_bytes(h);
        size_t reserve = ((size_t)1 << 30);
        if (s.mseg.size() < (size_t)c) reserve += ((size_t)c - s.mseg.size()) * mbytes;
        if (!s.mtmp[0]) reserve += 2 * fbytes;
        if (!s.q0) reserve += fbytes;
        if (!s.adj[0]) reserve += 2 * abytes + (size_t)h->dim * h->dim * sizeof(double);
        const size_t r = device_room(h);
        if (r > reserve) mt = (int)std::min<size_t>((size_t)nck, (r - reserve) / ((size_t)c * mbytes));
        if (h->cfg.adjoint_tail_segments > 0) mt = std::min(mt, h->cfg.adjoint_tail_segments);
    }
    s.tail_k0 = (nck - mt) * c;
    if (s.tail_k0 < iterations) {
        const size_t bytes = (size_t)(iterations - s.tail_k0) * mbytes;
        if (alloc_tracked(h, &s.tail_block, bytes) != LBM_OK) {
            // not after all: recompute every segment (not an error of this call)
            cudaGetLastError();
            lbm::set_last_error("");
            s.tail_block = nullptr;
            s.tail_k0 = iterations;
        } else {
            s.tail_bytes = bytes;
            for (int k = s.tail_k0; k < iterations; ++k)
                s.tpts.push_back(static_cast<char *>(s.tail_block) + (size_t)(k - s.tail_k0) * mbytes);
        }
    }

    // Q_0, then the iterations, copying Q_{jc} into checkpoint j; runs that
    // stay inside one checkpoint interval replay the step graph; the tail's
    // iterations also store their points
    ADJ_CUDA(cudaMemcpyAsync(s.ckpt[0], h->f[h->cur], fbytes, cudaMemcpyDeviceToDevice, h->stream));
    for (int k = 0; k < iterations;) {
        const int G = h->graph_iters, next_ck = (k / c + 1) * c;
        if (k >= s.tail_k0) {
            ADJ_CUDA(lbm::launch_iteration_adj(h, h->f[h->cur], h->f[h->cur ^ 1], s.tpts[k - s.tail_k0]));
            h->cur ^= 1;
            ++k;
        } else if (G > 1 && k + G <= iterations && k + G <= next_ck) {
            ADJ_CUDA(lbm::replay_iterations(h));
            k += G;
        } else {
            ADJ_CUDA(lbm::launch_iteration(h, h->f[h->cur], h->f[h->cur ^ 1]));
            h->cur ^= 1;
            ++k;
        }
        if (k < iterations && k % c == 0)
            ADJ_CUDA(cudaMemcpyAsync(s.ckpt[k / c], h->f[h->cur], fbytes, cudaMemcpyDeviceToDevice, h->stream));
    }
    h->it += iterations;
    h->state_is_init = false;

    // loss of R_T = S(Q_T)
    s.loss_grid = (unsigned)((h->n + kLossBlock - 1) / kLossBlock);
    if (!s.loss_part) {
        int rc = alloc_tracked(h, (void **)&s.loss_part, ((size_t)s.loss_grid + 1) * 2 * sizeof(double));
        if (rc != LBM_OK) return rc;
    }
    lbm::AdjArgs a = adj_args(h);
    a.fwd = h->f[h->cur];
    a.aout = nullptr;
    a.loss_part = s.loss_part;
    ADJ_CUDA(loss_seed(h, a));
    ADJ_CUDA(lbm::launch_sum_partials(s.loss_part, (int)s.loss_grid, s.loss_part + 2 * (size_t)s.loss_grid,
                                      h->stream));
    double sums[2];
    ADJ_CUDA(cudaMemcpyAsync(sums, s.loss_part + 2 * (size_t)s.loss_grid, sizeof sums, cudaMemcpyDeviceToHost,
                             h->stream));
    ADJ_CUDA(cudaEventRecord(h->ev_last, h->stream));
    ADJ_CUDA(cudaStreamSynchronize(h->stream));
    const double m = plane_sites(h);
    if (loss) *loss = m > 0 ? sums[0] / m : 0.0;
    s.ready = true;
    s.it_end = h->it;
    return LBM_OK;
}

int lbm_adjoint_backward(lbm_t *h, double dloss, double *grad_tau, double *grad_lid, void *grad_f0,
                         size_t grad_f0_bytes)
{
    if (!h) return fail(LBM_EINVAL, "lbm_adjoint_backward: NULL handle");
    const lbm::DeviceScope dev(h->cfg.device);
    lbm_adjoint_state &s = h->adj;
    if (!s.ready || s.it_end != h->it)
        return fail(LBM_ESTATE, "lbm_adjoint_backward: no adjoint forward recorded for the current state");
    const size_t ab = adj_bytes(h);
    const size_t abytes = (size_t)lbm::Q * h->n * ab;
    // grad_f0 comes in the F dump's element type (double for FP64 storage)
    const size_t db = h->prec == LBM_FP64 ? 8 : 4;
    const size_t dbytes = (size_t)lbm::Q * h->n * db;
    if (grad_f0 && grad_f0_bytes != dbytes)
        return fail(LBM_EINVAL, "lbm_adjoint_backward: grad_f0 is %zu bytes, needs %zu", grad_f0_bytes, dbytes);
    const size_t nc = (size_t)h->dim * h->dim;
    unsigned gi, gf;
    adj_grids(h, gi, gf);
    int ntx, nty;
    // tau partial slots: the one-step launch pair, or the two-step launch
    const unsigned agrid = std::max(gi + gf, two_step(h) ? adj2_grid(h, ntx, nty, false) : 0u);
    if (!s.adj[0]) {
        int rc = alloc_tracked(h, &s.adj[0], abytes);
        if (rc == LBM_OK) rc = alloc_tracked(h, &s.adj[1], abytes);
        if (rc == LBM_OK) rc = alloc_tracked(h, (void **)&s.grad_lid, nc * sizeof(double));
        if (rc != LBM_OK) return rc;
    }
    if (s.tau_acc && s.adj_grid != agrid) {
        free_tracked(h, s.tau_acc, (size_t)s.adj_grid * sizeof(double));
        s.tau_acc = nullptr;
        drop_segment_graphs(s);
    }
    if (!s.tau_acc) {
        int rc = alloc_tracked(h, (void **)&s.tau_acc, (size_t)agrid * sizeof(double));
        if (rc != LBM_OK) return rc;
    }
    s.adj_grid = agrid;
    cudaStream_t st = h->stream;
    ADJ_CUDA(cudaMemsetAsync(s.adj[0], 0, abytes, st));
    ADJ_CUDA(cudaMemsetAsync(s.adj[1], 0, abytes, st));
    ADJ_CUDA(cudaMemsetAsync(s.grad_lid, 0, nc * sizeof(double), st));
    ADJ_CUDA(cudaMemsetAsync(s.tau_acc, 0, (size_t)agrid * sizeof(double), st));

    // seed a_T
    int cur = 0;
    lbm::AdjArgs a = adj_args(h);
    const double m = plane_sites(h);
    a.fwd = h->f[h->cur];
    a.aout = s.adj[cur];
    a.loss_part = nullptr;
    a.dloss = m > 0 ? dloss * 2.0 / m : 0.0;
    ADJ_CUDA(loss_seed(h, a));

    const int T = s.iterations, c = s.every;
    const size_t fbytes = (size_t)lbm::Q * h->n * lbm::storage_bytes(h->prec);
    const size_t mbytes = 3 * h->n * lbm::macro_bytes(h->prec);
    // device bytes this sweep may still take
    auto room = [&]() -> size_t { return device_room(h); };

    // Without a tau gradient the adjoint needs only the velocity of the FLUID
    // sites and the density of the lid sites of each iteration: the segments
    // are recomputed storing those three planes (c of them, plus two state
    // scratch buffers) instead of c - 1 full states.
    bool macro = grad_tau == nullptr && !h->cfg.adjoint_full_states;
    // the recorded tail points serve the stored-point sweep only
    if (!macro) free_tail_points(h);
    if (macro) {
        // the full-state buffers of an earlier sweep make room first (and
        // the graphs that captured them go)
        if (!s.seg.empty()) drop_segment_graphs(s);
        for (void *p : s.seg) free_tracked(h, p, fbytes);
        s.seg.clear();
        const size_t need = (s.mseg.size() < (size_t)c ? (size_t)c - s.mseg.size() : 0) * mbytes +
                            (s.mtmp[0] ? 0 : 2 * fbytes);
        if (need > room()) {
            macro = false;  // does not fit: the full-state sweep (recursive when short)
            free_tail_points(h);
        } else {
            for (int k = 0; k < 2; ++k)
                if (!s.mtmp[k]) {
                    const int rc = alloc_tracked(h, &s.mtmp[k], fbytes);
                    if (rc != LBM_OK) return rc;
                }
            while ((int)s.mseg.size() < c) {
                void *p = nullptr;
                const int rc = alloc_tracked(h, &p, mbytes);
                if (rc != LBM_OK) return rc;
                s.mseg.push_back(p);
            }
        }
    }
    if (!macro) {
        if (!s.mseg.empty() || s.mtmp[0] || s.mtmp[1]) drop_segment_graphs(s);
        for (void *p : s.mseg) free_tracked(h, p, mbytes);
        s.mseg.clear();
        for (void *&p : s.mtmp) {
            free_tracked(h, p, fbytes);
            p = nullptr;
        }
    }

    // full-state sweep: c - 1 segment states when they fit (one-level sqrt
    // checkpointing), else as many as fit, and the sweep recurses.  Allocated
    // on the first backward sweep only, so a loss-only forward holds just its
    // checkpoints.
    if (!macro && (int)s.seg.size() < c - 1) {
        size_t fit = room() / fbytes;
        size_t want_total = (size_t)(c - 1);
        if (h->cfg.adjoint_max_states > 0) want_total = std::min(want_total, (size_t)h->cfg.adjoint_max_states);
        if (want_total > s.seg.size() + fit) {
            // a whole segment does not fit: take what the two-level schedule
            // uses (sub-checkpoints + one sub-segment + two), not all memory
            const size_t c2 = (size_t)std::ceil(std::sqrt((double)c));
            const size_t two_level = ((size_t)c + c2 - 1) / c2 - 1 + (c2 - 1) + 2;
            want_total = std::min(want_total, std::max<size_t>(two_level, 4));
        }
        const int want =
            want_total > s.seg.size() ? (int)std::min<size_t>(want_total - s.seg.size(), fit) : 0;
        for (int k = 0; k < want; ++k) {
            void *p = nullptr;
            const int rc = alloc_tracked(h, &p, fbytes);
            if (rc != LBM_OK) return rc;
            s.seg.push_back(p);
        }
    }
    // segments, last to first.  Full segments of the one-level sweep replay
    // a captured graph from a staged copy of their checkpoint (one state copy
    // per segment) when graphs are on and the copy buffer fits.
    ADJ_CUDA(prepare_adjoint2(h));
    const int nck = (T + c - 1) / c;
    bool graphs = h->graph_iters > 1 && c >= 2 && (macro || (int)s.seg.size() >= c - 1);
    if (graphs && (s.seg_graph_c != c || s.seg_graph_macro != macro)) {  // graphs of another sweep
        drop_segment_graphs(s);
        s.seg_graph_c = c;
        s.seg_graph_macro = macro;
    }
    if (graphs && !s.q0) {
        if (room() < fbytes || alloc_tracked(h, &s.q0, fbytes) != LBM_OK) graphs = false;
    }
    for (int j = nck - 1; j >= 0; --j) {
        const int start = j * c, len = std::min(T, start + c) - start;
        if (macro && start >= s.tail_k0) {
            // points recorded by the forward: the adjoint steps only
            const int rc = adjoint_steps_down(h, start, len,
                                              [&](int k) -> const void * { return s.tpts[k - s.tail_k0]; }, cur, true);
            if (rc != LBM_OK) return rc;
            continue;
        }
        if (graphs && len == c) {
            ADJ_CUDA(cudaMemcpyAsync(s.q0, s.ckpt[j], fbytes, cudaMemcpyDeviceToDevice, st));
            const int rc = replay_segment(h, c, cur, macro);
            if (rc != LBM_OK) return rc;
            continue;
        }
        const int rc = macro ? sweep_macro(h, s.ckpt[j], start, len, cur)
                             : sweep(h, s.ckpt[j], start, len, s.seg, 0, (int)s.seg.size(), cur);
        if (rc != LBM_OK) return rc;
    }
    // a_0 = dJ/dR_0; the init kernel's lid dependence of R_0
    if (s.init_state) {
        lbm::AdjArgs b = adj_args(h);
        b.ain = s.adj[cur];
        ADJ_CUDA(lid_init_grad(h, b));
    }
    std::vector<double> tau(agrid);
    ADJ_CUDA(cudaMemcpyAsync(tau.data(), s.tau_acc, agrid * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (grad_lid) ADJ_CUDA(cudaMemcpyAsync(grad_lid, s.grad_lid, nc * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (grad_f0) {
        const size_t total = (size_t)lbm::Q * h->n;
        const size_t chunk = std::min(total, (size_t)1 << 25);
        for (size_t o0 = 0; o0 < total; o0 += chunk) {
            const size_t cnt = std::min(chunk, total - o0);
            const unsigned g = (unsigned)((cnt + 255) / 256);
            if (ab == 8 && db == 8)
                lbm::export_adjoint_kernel<double, double><<<g, 256, 0, st>>>(
                    static_cast<const double *>(s.adj[cur]), static_cast<double *>(h->stage), o0, cnt, h->sd, h->n);
            else if (ab == 8)
                lbm::export_adjoint_kernel<double, float><<<g, 256, 0, st>>>(
                    static_cast<const double *>(s.adj[cur]), static_cast<float *>(h->stage), o0, cnt, h->sd, h->n);
            else
                lbm::export_adjoint_kernel<float, float><<<g, 256, 0, st>>>(
                    static_cast<const float *>(s.adj[cur]), static_cast<float *>(h->stage), o0, cnt, h->sd, h->n);
            ADJ_CUDA(cudaGetLastError());
            ADJ_CUDA(cudaMemcpyAsync((char *)grad_f0 + o0 * db, h->stage, cnt * db, cudaMemcpyDeviceToHost, st));
        }
    }
    ADJ_CUDA(cudaEventRecord(h->ev_last, st));
    ADJ_CUDA(cudaStreamSynchronize(st));
    int status = 0;
    ADJ_CUDA(cudaMemcpy(&status, h->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status & 2)
        return fail(LBM_ETIMEOUT, "lbm_adjoint_backward: a bounded wait of the two-step adjoint expired; "
                                  "the gradients are not valid");
    double dw = 0.0;
    for (double v : tau) dw += v;
    // omega = 1 / tau
    if (grad_tau) *grad_tau = -h->inv_tau * h->inv_tau * dw;
    return LBM_OK;
}

}  // extern "C"
