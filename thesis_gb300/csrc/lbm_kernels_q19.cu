// D3Q19 instantiation of the step, init, residual and encode/decode launchers.
#include "lbm_kernels.cuh"

LBM_DEFINE_LAUNCHERS(19)
