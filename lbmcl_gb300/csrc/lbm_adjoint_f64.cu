// lbm_adjoint_f64.cu -- the adjoint kernels in FP64 arithmetic over FP32,
// FP16 and BF16 population storage (lbm_config.adjoint_fp64): the same
// hand-written adjoint as the FP32 one, so that the two can be compared on
// one and the same trajectory.  A translation unit of its own so that these
// register-heavy instantiations compile in parallel with the rest.
#include "lbm.h"
#include "lbm_adjoint.cuh"

namespace lbm {
namespace {

template <class S, bool MACRO>
cudaError_t step_a64(const AdjArgs &a0, unsigned gi, unsigned gf, unsigned block, cudaStream_t s)
{
    AdjArgs a = a0;
    if (gi > 0) {
        a.tau_base = 0;
        adjoint_kernel<S, double, 16, ROWS_INTERIOR, MACRO><<<gi, block, 0, s>>>(a);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    a.tau_base = gi;
    adjoint_kernel<S, double, 16, ROWS_FACES, MACRO><<<gf, block, 0, s>>>(a);
    return cudaGetLastError();
}

template <class S>
cudaError_t step_any(const AdjArgs &a, unsigned gi, unsigned gf, unsigned block, cudaStream_t s, bool macro)
{
    return macro ? step_a64<S, true>(a, gi, gf, block, s) : step_a64<S, false>(a, gi, gf, block, s);
}

}  // namespace

cudaError_t launch_adjoint_step_a64(int prec, const AdjArgs &a, unsigned gi, unsigned gf, unsigned block,
                                    cudaStream_t s, bool macro)
{
    switch (prec) {
    case LBM_FP32: return step_any<float>(a, gi, gf, block, s, macro);
    case LBM_FP16: return step_any<__half>(a, gi, gf, block, s, macro);
    case LBM_BF16: return step_any<__nv_bfloat16>(a, gi, gf, block, s, macro);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_loss_seed_a64(int prec, const AdjArgs &a, unsigned grid, unsigned block, cudaStream_t s)
{
    switch (prec) {
    case LBM_FP32: loss_seed_kernel<float, double><<<grid, block, 0, s>>>(a); break;
    case LBM_FP16: loss_seed_kernel<__half, double><<<grid, block, 0, s>>>(a); break;
    case LBM_BF16: loss_seed_kernel<__nv_bfloat16, double><<<grid, block, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_lid_init_grad_a64(int prec, const AdjArgs &a, cudaStream_t s)
{
    const int nc = a.dim * a.dim;
    const unsigned grid = (unsigned)((nc + 255) / 256);
    switch (prec) {
    case LBM_FP32: lid_init_grad_kernel<float, double><<<grid, 256, 0, s>>>(a); break;
    case LBM_FP16: lid_init_grad_kernel<__half, double><<<grid, 256, 0, s>>>(a); break;
    case LBM_BF16: lid_init_grad_kernel<__nv_bfloat16, double><<<grid, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace lbm
