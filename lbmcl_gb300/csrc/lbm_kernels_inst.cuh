// lbm_kernels_inst.cuh -- instantiates the kernels of one storage type.
// Included by lbm_kernels_<type>.cu with LBM_S (element type), LBM_T (F-dump
// element type) and LBM_SFX (launcher suffix) defined.
#include "lbm_kernels.cuh"
#include "lbm_launch.h"

namespace lbm {

#define LBM_CAT2(a, b) a##b
#define LBM_CAT(a, b) LBM_CAT2(a, b)

cudaError_t LBM_CAT(launch_pull_, LBM_SFX)(int mode, const StepArgs &a, unsigned grid, unsigned block,
                                           cudaStream_t s)
{
    if (grid == 0) return cudaSuccess;
    switch (mode) {
    case MODE_STEP: pull_kernel<LBM_S, MODE_STEP><<<grid, block, 0, s>>>(a); break;
    case MODE_STEP_MACRO: pull_kernel<LBM_S, MODE_STEP_MACRO><<<grid, block, 0, s>>>(a); break;
    case MODE_REDUCE: pull_kernel<LBM_S, MODE_REDUCE><<<grid, block, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

const void *LBM_CAT(pull_kernel_ptr_, LBM_SFX)(int mode)
{
    switch (mode) {
    case MODE_STEP: return (const void *)pull_kernel<LBM_S, MODE_STEP>;
    case MODE_STEP_MACRO: return (const void *)pull_kernel<LBM_S, MODE_STEP_MACRO>;
    case MODE_REDUCE: return (const void *)pull_kernel<LBM_S, MODE_REDUCE>;
    default: return nullptr;
    }
}

cudaError_t LBM_CAT(launch_narrow_, LBM_SFX)(int mode, const StepArgs &a, unsigned grid, unsigned block,
                                             cudaStream_t s)
{
    if (grid == 0) return cudaSuccess;
    if constexpr (sizeof(LBM_S) < 8) {
        switch (mode) {
        case MODE_STEP: pull_kernel<LBM_S, MODE_STEP, 8><<<grid, block, 0, s>>>(a); break;
        case MODE_STEP_MACRO: pull_kernel<LBM_S, MODE_STEP_MACRO, 8><<<grid, block, 0, s>>>(a); break;
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    } else {
        return cudaErrorInvalidValue;  // one double per 8 bytes: no narrow variant
    }
}

cudaError_t LBM_CAT(launch_staged_, LBM_SFX)(int mode, const StepArgs &a, unsigned grid, unsigned block,
                                             size_t smem, cudaStream_t s)
{
    if (grid == 0) return cudaSuccess;
    switch (mode) {
    case MODE_STEP: pull_staged_kernel<LBM_S, MODE_STEP><<<grid, block, smem, s>>>(a); break;
    case MODE_STEP_MACRO: pull_staged_kernel<LBM_S, MODE_STEP_MACRO><<<grid, block, smem, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

const void *LBM_CAT(staged_kernel_ptr_, LBM_SFX)(int mode)
{
    switch (mode) {
    case MODE_STEP: return (const void *)pull_staged_kernel<LBM_S, MODE_STEP>;
    case MODE_STEP_MACRO: return (const void *)pull_staged_kernel<LBM_S, MODE_STEP_MACRO>;
    default: return nullptr;
    }
}

cudaError_t LBM_CAT(launch_init_, LBM_SFX)(const InitArgs &a, cudaStream_t s)
{
    const unsigned block = 256;
    const size_t grid = (a.n + block - 1) / block;
    init_kernel<LBM_S><<<(unsigned)grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t LBM_CAT(launch_dump_, LBM_SFX)(const DumpArgs &a, cudaStream_t s)
{
    const unsigned block = 256;
    const size_t grid = (a.count + block - 1) / block;
    if (grid == 0) return cudaSuccess;
    dump_f_kernel<LBM_S, LBM_T><<<(unsigned)grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t LBM_CAT(launch_load_, LBM_SFX)(const DumpArgs &a, cudaStream_t s)
{
    const unsigned block = 256;
    const size_t grid = (a.count + block - 1) / block;
    if (grid == 0) return cudaSuccess;
    load_f_kernel<LBM_S, LBM_T><<<(unsigned)grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace lbm
