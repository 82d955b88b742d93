// Viscoelastic kernels, convergence order 4 (generated bodies + launchers).
#include "common.cuh"
#include "_gen/kernels_visco_o4.cuh"
#define SEI_VORDER 4
#include "kernels_visco.cuh"
