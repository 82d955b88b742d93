// Internal declarations shared by the host set-up, the C ABI and the kernel launchers.
#pragma once
#include <cstdint>
#include <vector>

#include "sei_gb300.h"

namespace sei {

inline int numBasis(int order) { return order * (order + 1) * (order + 2) / 6; }
inline int numFaceBasis(int order) { return order * (order + 1) / 2; }
inline int paddedBasis(int order) { return (numBasis(order) + 3) / 4 * 4; }
inline int derivativesSize(int order) {
  int s = 0;
  for (int i = 0; i < order; ++i) s += numBasis(order - i) * 9;
  return s;
}

// Non-zeros of the elastic star matrix (codegen/matrices/star.xml), column-major order over (q, p).
constexpr int kStarNnz = 24;
constexpr int kStarNz[kStarNnz][2] = {{6, 0}, {7, 0}, {8, 0}, {6, 1}, {7, 1}, {8, 1}, {6, 2}, {7, 2},
                                      {8, 2}, {6, 3}, {7, 3}, {7, 4}, {8, 4}, {6, 5}, {8, 5}, {0, 6},
                                      {3, 6}, {5, 6}, {1, 7}, {3, 7}, {4, 7}, {2, 8}, {4, 8}, {5, 8}};

struct HostMesh {
  int64_t n = 0;
  std::vector<int64_t> topo;     // [n][4] vertex ids (periodic identification applied)
  std::vector<double> coords;    // [n][4][3] unwrapped vertex coordinates
  std::vector<double> material;  // [n][3] rho, mu, lambda
  std::vector<int32_t> nbr;      // [n][4]
  std::vector<int8_t> side, orient, ftype;
};

void buildPeriodicCube(const sei_cube_params& p, HostMesh& m);
void computeFaceRelations(HostMesh& m);
void buildOperators(const HostMesh& m, std::vector<float>& star, std::vector<float>& aplus, std::vector<float>& aminus);
double cflTimestep(const HostMesh& m, int order, double cfl);
void seedDofs(int64_t n, int order, uint64_t seed, std::vector<float>& dofs);

// Kernel launchers (one translation unit per order).
struct DeviceArrays {
  int n;
  float* Q;
  float* I;
  float* derivs;  // nullable
  const float* star_nz;
  const float* aplus;
  const float* aminus;
  const int32_t* nbr;
  const uint8_t* rel;    // side | orient << 2
  const uint8_t* ftype;  // 0 regular, 1 dynamic rupture, 2 none
};

using LaunchLocalFn = int (*)(const DeviceArrays&, const float* coeffs, void* stream);
using LaunchNeighborFn = int (*)(const DeviceArrays&, void* stream);
using LaunchTaylorFn = int (*)(int n, const float* derivs, const float* coeffs, float* out, void* stream);

struct OrderKernels {
  LaunchLocalFn local;
  LaunchNeighborFn neighbor;
  LaunchTaylorFn taylor;
};

bool kernelsForOrder(int order, OrderKernels& out);

}  // namespace sei
