// lbm_kernels_f16.cu -- kernels with __half population storage.
#define LBM_S __half
#define LBM_T float
#define LBM_SFX f16
#include "lbm_kernels_inst.cuh"
