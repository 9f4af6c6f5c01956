// lbm_kernels_bf16.cu -- kernels with __nv_bfloat16 population storage.
#define LBM_S __nv_bfloat16
#define LBM_T float
#define LBM_SFX bf16
#include "lbm_kernels_inst.cuh"
