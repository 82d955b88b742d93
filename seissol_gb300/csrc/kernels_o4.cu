// FP32 CUDA-core ADER-DG kernels, convergence order 4.
#include "common.cuh"
#include "tc.cuh"
#include "_gen/kernels_o4.cuh"
#define SEI_ORDER 4
#include "kernels_order.cuh"
