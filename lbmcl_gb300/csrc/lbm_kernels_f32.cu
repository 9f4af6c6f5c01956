// lbm_kernels_f32.cu -- kernels with float population storage.
#define LBM_S float
#define LBM_T float
#define LBM_SFX f32
#include "lbm_kernels_inst.cuh"
