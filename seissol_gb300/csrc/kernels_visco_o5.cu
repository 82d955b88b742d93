// Viscoelastic kernels, convergence order 5 (generated bodies + launchers).
#include "common.cuh"
#include "_gen/kernels_visco_o5.cuh"
#define SEI_VORDER 5
#include "kernels_visco.cuh"
