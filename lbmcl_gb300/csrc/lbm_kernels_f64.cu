// lbm_kernels_f64.cu -- kernels with double population storage.
#define LBM_S double
#define LBM_T double
#define LBM_SFX f64
#include "lbm_kernels_inst.cuh"
