// sei_mlp_gradient_noalloc: the loss gradient of the warm-start network (same kernel and result
// as sei_mlp_gradient) without any device allocation.
//
// Who needs it: host codes that own all device memory through their own pool, reserved at
// start-up for the mesh and the time-stepping buffers, and that keep several streams of device
// work in flight.  A cudaMalloc from the library would take memory outside that pool (and can
// fail once the pool holds the device), and cudaFree synchronises the whole device, stalling the
// caller's streams.  This entry point therefore calls no cudaMalloc, cudaFree or allocating
// library routine: its device scratch (copies of the parameters, normalisation and samples, the
// gradient and loss accumulators) is one file-scope static device array of fixed size, which
// bounds the sample count at SEI_MLP_NOALLOC_MAX_SAMPLES.
//
// Set-up: the first call on a device (the device current at the call) looks up the array's device
// address with cudaGetSymbolAddress and keeps it for later calls on that device.  Make that first
// call before any stream capture on the device.  With lazy module loading (the CUDA default) that
// first look-up also loads this module, which is when the driver allocates the 421 KiB array, and a
// module load may synchronise the device: make the first call at start-up, before the pool takes
// the device and before streams are in flight (or load eagerly, CUDA_MODULE_LOADING=EAGER).
//
// Streams: the copies, the clears and the kernel run on the calling host thread's per-thread
// default stream (cudaStreamPerThread), which does not wait for the caller's other streams, and
// the call returns after that stream alone has finished.  It still orders with the legacy default
// stream (stream 0) if the caller uses that one.
//
// Sharing: every call on a device uses the same array.  The gradient and loss accumulators are
// cleared at the start of every call and the inputs overwritten, so consecutive calls are
// independent; calls that overlap on the GPU (for example from two host threads at once) race on
// the array and give wrong results.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"
#include "mlp.cuh"

namespace {

constexpr int kMaxSamples = SEI_MLP_NOALLOC_MAX_SAMPLES;
constexpr int kAlignFloats = 64;  // 256 bytes
constexpr int roundUp(int v) { return (v + kAlignFloats - 1) / kAlignFloats * kAlignFloats; }

// Scratch layout in floats, every region starting on a 256-byte boundary.
constexpr int kParams = sei_mlp::kHidden * 5 + sei_mlp::kHidden + sei_mlp::kHidden * sei_mlp::kHidden +
                        sei_mlp::kHidden + sei_mlp::kHidden + 1;
constexpr int kOffP = 0;                              // parameters [kParams]
constexpr int kOffN = kOffP + roundUp(kParams);       // normalisation [16]
constexpr int kOffG = kOffN + roundUp(sei_mlp::kNorm);  // gradient accumulator [kParams], zeroed per call
constexpr int kOffL = kOffG + roundUp(kParams);       // loss accumulator [1], zeroed per call
constexpr int kOffT = kOffL + kAlignFloats;           // targets [n]
constexpr int kOffX = kOffT + roundUp(kMaxSamples);   // inputs [n][5]
constexpr int kScratchFloats = kOffX + roundUp(5 * kMaxSamples);  // 107,776 floats = 421 KiB

static __device__ __align__(256) float g_mlpScratch[kScratchFloats];

constexpr int kMaxDevices = 64;
std::mutex g_setupMutex;
float* g_scratchPtr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
int scratchOnCurrentDevice(float** out, int* sms) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SEI_ERR_CUDA;
  if (cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SEI_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setupMutex);
  if (!g_scratchPtr[dev]) {
    float* ptr = nullptr;
    if (cudaGetSymbolAddress((void**)&ptr, g_mlpScratch) != cudaSuccess || !ptr) {
      cudaGetLastError();
      return SEI_ERR_CUDA;
    }
    g_scratchPtr[dev] = ptr;
  }
  *out = g_scratchPtr[dev];
  return SEI_OK;
}

}  // namespace

extern "C" int sei_mlp_gradient_noalloc(const float* params, const float* norm, const float* samples, int64_t n,
                                        float* grads, float* loss) {
  if (!params || !norm || !samples || !grads || !loss || n <= 0) return SEI_ERR_ARG;
  if (n > kMaxSamples) return SEI_ERR_CAPACITY;
  float* s = nullptr;
  int sms = 0;
  int rc = scratchOnCurrentDevice(&s, &sms);
  if (rc) return rc;
  float* P = s + kOffP;
  float* N = s + kOffN;
  float* G = s + kOffG;
  float* L = s + kOffL;
  float* T = s + kOffT;
  float* X = s + kOffX;
  const size_t rows = (size_t)n;
  // samples [n][6] -> inputs [n][5] and targets [n] by strided copies, all on the per-thread stream
  const cudaStream_t st = cudaStreamPerThread;
  if (cudaMemcpyAsync(P, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(N, norm, sizeof(float) * sei_mlp::kNorm, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpy2DAsync(X, 5 * sizeof(float), samples, 6 * sizeof(float), 5 * sizeof(float), rows,
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpy2DAsync(T, sizeof(float), samples + 5, 6 * sizeof(float), sizeof(float), rows, cudaMemcpyHostToDevice,
                        st) != cudaSuccess ||
      cudaMemsetAsync(G, 0, sizeof(float) * kParams, st) != cudaSuccess ||
      cudaMemsetAsync(L, 0, sizeof(float), st) != cudaSuccess ||
      sei::launchMlpGrad(P, N, X, T, (int)n, G, L, sms > 0 ? sms : 1, (void*)st) != 0 ||
      cudaMemcpyAsync(grads, G, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(loss, L, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    rc = SEI_ERR_CUDA;
  cudaGetLastError();
  return rc;
}
