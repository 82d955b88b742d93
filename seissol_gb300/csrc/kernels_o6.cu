// FP32 CUDA-core ADER-DG kernels, convergence order 6.
#include "common.cuh"
#include "tc.cuh"
#include "_gen/kernels_o6.cuh"
#define SEI_ORDER 6
#include "kernels_order.cuh"
