// Output path: receivers and the device -> host staging of output rows (output.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <vector>

#include "internal.h"

namespace sei {

// Rows written on the compute stream into one of two device halves; a full half (or a flush)
// is copied on the stager's own stream into its pinned twin, and a stream host function appends
// the rows to the host store.  Writes into a half wait for that half's previous copy.
class Stager {
 public:
  ~Stager();
  int init(size_t rowBytes, size_t rowsPerHalf);  // 0, or -1 when an allocation failed
  void release();
  bool ready() const { return stream_ != nullptr; }
  // Device memory for `rows` consecutive rows, written on `compute` (flushes a full half first);
  // *err -2 when rows exceed a half, -1 on a CUDA error.
  void* reserve(size_t rows, cudaStream_t compute, int* err);
  int flush(cudaStream_t compute);
  // Flushes, waits for the copies and moves up to maxRows rows (oldest first) to out.
  int drain(cudaStream_t compute, void* out, size_t maxRows, size_t* nrows);
  size_t pendingRows(cudaStream_t compute);  // flushes and waits; rows in the host store

 private:
  static void CUDART_CB appendHost(void* p);
  friend struct StagerAppend;
  cudaStream_t stream_ = nullptr;
  void* dev_[2] = {nullptr, nullptr};
  void* host_[2] = {nullptr, nullptr};
  cudaEvent_t done_[2] = {nullptr, nullptr}, full_[2] = {nullptr, nullptr};
  size_t rowBytes_ = 0, rowsPerHalf_ = 0, used_ = 0;
  int half_ = 0;
  std::mutex mu_;
  std::vector<char> store_;
};

constexpr int kRecvMaxSamples = 32;  // samples per evaluation launch

struct RecvEvalArgs {
  int nrecv;            // receivers of this launch
  const int32_t* list;  // [nrecv] their indices (the rows of slot, phi, dphi)
  const int32_t* slot;  // [receivers] row of derivs: the receiver's cell in the compact copy
  const float* derivs;  // [cells][derivativesSize]
  const float* phi;     // [nrecv][B] basis functions at the receiver
  const float* dphi;    // [nrecv][3][B] their gradients in global coordinates
  double time0;         // expansion point: the start of the step
  int nsamples;
  double offset[kRecvMaxSamples];  // sampling times minus time0
  unsigned qmask;                  // quantities written (bit q: quantity q)
  int derived;                     // SEI_RECV_ROTATION | SEI_RECV_STRAIN
  int ncols;
  int visco;    // derivatives of the viscoelastic kernels: [order][27][B] (every stage all rows)
  double* out;  // [nsamples][nrecv][ncols], receivers in list order
};

int launchGatherRows(int m, const int32_t* src, const float* in, float* out, int rowFloats, void* stream);
int launchRecvEval(int order, const RecvEvalArgs& a, void* stream);
// Basis functions (phi [B]) and their global gradients (dphi [3][B]) at reference point xez, with
// grad[r][x] = d xi_r / d x.
void basisAtPoint(int order, const double xez[3], const double grad[3][3], double* phi, double* dphi);
void locatePoints(const HostMesh& m, int64_t np, const double* xyz, std::vector<int64_t>& cell,
                  std::vector<double>& xez);

}  // namespace sei
