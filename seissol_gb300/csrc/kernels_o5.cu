// FP32 CUDA-core ADER-DG kernels, convergence order 5.
#include "common.cuh"
#include "tc.cuh"
#include "_gen/kernels_o5.cuh"
#define SEI_ORDER 5
#include "kernels_order.cuh"
