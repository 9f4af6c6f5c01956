// lbm_launch.h -- host-side launchers of the kernels, one translation unit
// per storage type (lbm_kernels_<type>.cu) so they compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "lbm_device.cuh"

namespace lbm {

struct InitArgs;
struct DumpArgs;

// prec: 0 FP32, 1 FP64, 2 FP16, 3 BF16 (lbm_precision)
#define LBM_DECLARE_LAUNCHERS(SFX)                                                                   \
    cudaError_t launch_pull_##SFX(int mode, const StepArgs &a, unsigned block, cudaStream_t s,       \
                                  unsigned *nparts);                                                 \
    cudaError_t launch_narrow_##SFX(int mode, const StepArgs &a, unsigned block, cudaStream_t s);    \
    cudaError_t launch_split_##SFX(int vb, int mode, const StepArgs &a, unsigned block, cudaStream_t s,\
                                   cudaStream_t sf);                                                 \
    cudaError_t launch_aa_##SFX(int mode, const StepArgs &a, unsigned block, cudaStream_t s,         \
                                unsigned *nparts);                                                   \
    cudaError_t launch_staged_##SFX(int mode, const StepArgs &a, unsigned grid, unsigned block,      \
                                    size_t smem, cudaStream_t s);                                    \
    const void *staged_kernel_ptr_##SFX(int mode);                                                  \
    cudaError_t launch_init_##SFX(const InitArgs &a, cudaStream_t s);                               \
    cudaError_t launch_dump_##SFX(const DumpArgs &a, cudaStream_t s);                               \
    cudaError_t launch_load_##SFX(const DumpArgs &a, cudaStream_t s);

LBM_DECLARE_LAUNCHERS(f32)
LBM_DECLARE_LAUNCHERS(f64)
LBM_DECLARE_LAUNCHERS(f16)
LBM_DECLARE_LAUNCHERS(bf16)

cudaError_t launch_sum_partials(const double *partials, int nblocks, double *out, cudaStream_t s);

// Set the calling thread's lbm_last_error() text (for entry points defined
// outside lbm_capi.cu).
void set_last_error(const char *msg);

}  // namespace lbm
