// C ABI of the GB300 ADER-DG element update (declarations and reference mapping in include/sei_gb300.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "internal.h"

namespace sei {
OrderKernels orderKernels4();
OrderKernels orderKernels5();
OrderKernels orderKernels6();

bool kernelsForOrder(int order, OrderKernels& out) {
  switch (order) {
    case 4: out = orderKernels4(); return true;
    case 5: out = orderKernels5(); return true;
    case 6: out = orderKernels6(); return true;
    default: return false;
  }
}
}  // namespace sei

struct sei_ctx {
  sei_config cfg{};
  int B = 0, Bp = 0, F = 0;
  sei::OrderKernels k{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  int64_t n = 0;
  // device arrays
  float *Q = nullptr, *I = nullptr, *derivs = nullptr, *star_nz = nullptr, *aplus = nullptr, *aminus = nullptr;
  int32_t* nbr = nullptr;
  uint8_t *rel = nullptr, *ftype = nullptr;
  // host copies of what the context built (for sei_get_cells / sei_get_geometry)
  sei::HostMesh mesh;
  std::vector<float> h_star, h_aplus, h_aminus;
  bool has_mesh = false;
  // per-launch timing (sei_set_profiling): one event before every launch plus one at the end
  bool profiling = false;
  std::vector<cudaEvent_t> prof_events;
  std::vector<int> prof_kind;  // kind of the launch that starts at event i (0 local, 1 neighbour)
  size_t prof_used = 0;
};

namespace {

int fail(sei_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cudaFail(sei_ctx* c, cudaError_t e, const char* what) {
  return fail(c, SEI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SEI_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cudaFail(c, e_, #call); \
  } while (0)

void freeArrays(sei_ctx* c) {
  cudaFree(c->Q);
  cudaFree(c->I);
  cudaFree(c->derivs);
  cudaFree(c->star_nz);
  cudaFree(c->aplus);
  cudaFree(c->aminus);
  cudaFree(c->nbr);
  cudaFree(c->rel);
  cudaFree(c->ftype);
  c->Q = c->I = c->derivs = c->star_nz = c->aplus = c->aminus = nullptr;
  c->nbr = nullptr;
  c->rel = c->ftype = nullptr;
  c->n = 0;
}

int allocArrays(sei_ctx* c, int64_t n) {
  freeArrays(c);
  if (n <= 0 || n > (int64_t)0x7fffffff / 9) return fail(c, SEI_ERR_ARG, "cell count out of range");
  const size_t dof = (size_t)n * 9 * c->Bp * sizeof(float);
  auto alloc = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, bytes) == cudaSuccess; };
  bool ok = alloc((void**)&c->Q, dof) && alloc((void**)&c->I, dof) &&
            alloc((void**)&c->star_nz, (size_t)n * 3 * sei::kStarNnz * sizeof(float)) &&
            alloc((void**)&c->aplus, (size_t)n * 4 * 81 * sizeof(float)) &&
            alloc((void**)&c->aminus, (size_t)n * 4 * 81 * sizeof(float)) &&
            alloc((void**)&c->nbr, (size_t)n * 4 * sizeof(int32_t)) && alloc((void**)&c->rel, (size_t)n * 4) &&
            alloc((void**)&c->ftype, (size_t)n * 4);
  if (ok && c->cfg.store_derivatives)
    ok = alloc((void**)&c->derivs, (size_t)n * sei::derivativesSize(c->cfg.order) * sizeof(float));
  if (!ok) {
    cudaGetLastError();
    freeArrays(c);
    return fail(c, SEI_ERR_OOM, "device allocation failed");
  }
  c->n = n;
  if (cudaMemsetAsync(c->Q, 0, dof, c->stream) != cudaSuccess || cudaMemsetAsync(c->I, 0, dof, c->stream) != cudaSuccess)
    return fail(c, SEI_ERR_CUDA, "memset failed");
  return SEI_OK;
}

int uploadCells(sei_ctx* c, int64_t n, const float* star, const float* aplus, const float* aminus,
                const int32_t* nbr, const int8_t* side, const int8_t* orient, const int8_t* ftype) {
  std::vector<float> snz((size_t)n * 3 * sei::kStarNnz);
  for (int64_t i = 0; i < n; ++i)
    for (int e = 0; e < 3; ++e)
      for (int z = 0; z < sei::kStarNnz; ++z)
        snz[(i * 3 + e) * sei::kStarNnz + z] = star[(i * 3 + e) * 81 + sei::kStarNz[z][0] + 9 * sei::kStarNz[z][1]];
  std::vector<uint8_t> rel((size_t)n * 4), ft((size_t)n * 4);
  for (int64_t i = 0; i < n * 4; ++i) {
    if (ftype[i] < 0 || ftype[i] > 2) return fail(c, SEI_ERR_ARG, "face_type must be 0, 1 or 2");
    if (ftype[i] == 0) {
      if (nbr[i] < 0 || nbr[i] >= n) return fail(c, SEI_ERR_ARG, "regular face with neighbour out of range");
      if (side[i] < 0 || side[i] > 3 || orient[i] < 0 || orient[i] > 2)
        return fail(c, SEI_ERR_ARG, "face relation out of range (side 0..3, orientation 0..2)");
    }
    rel[i] = (uint8_t)((side[i] & 3) | ((orient[i] & 3) << 2));
    ft[i] = (uint8_t)ftype[i];
  }
  for (size_t i = 0; i < snz.size(); ++i)
    if (!std::isfinite(snz[i])) return fail(c, SEI_ERR_NAN, "non-finite star matrix entry");
  SEI_CUDA(cudaMemcpy(c->star_nz, snz.data(), snz.size() * sizeof(float), cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->aplus, aplus, (size_t)n * 4 * 81 * sizeof(float), cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->aminus, aminus, (size_t)n * 4 * 81 * sizeof(float), cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->nbr, nbr, (size_t)n * 4 * sizeof(int32_t), cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->rel, rel.data(), rel.size(), cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->ftype, ft.data(), ft.size(), cudaMemcpyHostToDevice));
  return SEI_OK;
}

sei::DeviceArrays arrays(sei_ctx* c) {
  return sei::DeviceArrays{(int)c->n, c->Q, c->I, c->derivs, c->star_nz, c->aplus, c->aminus, c->nbr, c->rel, c->ftype};
}

void taylorCoeffs(int order, double dt, float* out) {
  // MonomialBasis::integrate(0, dt): dt^{i+1} / (i+1)!
  double v = dt;
  for (int i = 0; i < order; ++i) {
    out[i] = (float)v;
    v *= dt / (i + 2);
  }
}

int checkReady(sei_ctx* c) {
  if (!c) return SEI_ERR_ARG;
  if (c->cfg.device < 0) return fail(c, SEI_ERR_STATE, "host-only context (device < 0) has no device data");
  if (c->n <= 0) return fail(c, SEI_ERR_STATE, "no cells uploaded");
  return SEI_OK;
}

int profMark(sei_ctx* c, int kind) {
  if (!c->profiling) return SEI_OK;
  if (c->prof_used == c->prof_events.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return fail(c, SEI_ERR_CUDA, "event creation failed");
    c->prof_events.push_back(e);
    c->prof_kind.push_back(kind);
  }
  c->prof_kind[c->prof_used] = kind;
  if (cudaEventRecord(c->prof_events[c->prof_used], c->stream) != cudaSuccess)
    return fail(c, SEI_ERR_CUDA, "event record failed");
  ++c->prof_used;
  return SEI_OK;
}

int launchLocal(sei_ctx* c, const sei::DeviceArrays& d, const float* coeffs) {
  int rc = profMark(c, 0);
  if (rc) return rc;
  if (c->k.local(d, coeffs, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "local kernel launch failed");
  return SEI_OK;
}

int launchNeighbor(sei_ctx* c, const sei::DeviceArrays& d) {
  int rc = profMark(c, 1);
  if (rc) return rc;
  if (c->k.neighbor(d, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "neighbour kernel launch failed");
  return SEI_OK;
}

int runKernel(sei_ctx* c, int kernel, double dt, int steps) {
  float coeffs[8];
  taylorCoeffs(c->cfg.order, dt, coeffs);
  sei::DeviceArrays d = arrays(c);
  c->prof_used = 0;
  int rc = SEI_OK;
  for (int s = 0; s < steps && rc == SEI_OK; ++s) {
    switch (kernel) {
      case SEI_KERNEL_ALL:
        rc = launchLocal(c, d, coeffs);
        if (!rc) rc = launchNeighbor(c, d);
        break;
      case SEI_KERNEL_LOCAL:
        rc = launchLocal(c, d, coeffs);
        break;
      case SEI_KERNEL_NEIGHBOR:
        rc = launchNeighbor(c, d);
        break;
      default:
        return fail(c, SEI_ERR_UNSUPPORTED, "kernel not supported by this build");
    }
  }
  if (!rc) rc = profMark(c, -1);
  return rc;
}

}  // namespace

extern "C" {

int sei_version(void) { return 1; }

int sei_create(const sei_config* cfg, sei_ctx** out) {
  if (!cfg || !out) return SEI_ERR_ARG;
  *out = nullptr;
  sei_ctx* c = new (std::nothrow) sei_ctx();
  if (!c) return SEI_ERR_OOM;
  c->cfg = *cfg;
  if (!sei::kernelsForOrder(cfg->order, c->k)) {
    delete c;
    return SEI_ERR_UNSUPPORTED;
  }
  if (cfg->precision != SEI_PREC_FP32) {
    delete c;
    return SEI_ERR_UNSUPPORTED;
  }
  c->B = sei::numBasis(cfg->order);
  c->Bp = sei::paddedBasis(cfg->order);
  c->F = sei::numFaceBasis(cfg->order);
  if (cfg->device < 0) {  // host-only context: set-up functions only, no CUDA calls
    *out = c;
    return SEI_OK;
  }
  if (cudaSetDevice(cfg->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    cudaGetLastError();
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return SEI_ERR_CUDA;
  }
  *out = c;
  return SEI_OK;
}

void sei_destroy(sei_ctx* c) {
  if (!c) return;
  if (c->cfg.device < 0) {
    delete c;
    return;
  }
  cudaSetDevice(c->cfg.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  freeArrays(c);
  for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* sei_last_error(const sei_ctx* c) { return c ? c->err.c_str() : "null context"; }

int sei_build_periodic_cube(sei_ctx* c, const sei_cube_params* p, int64_t* ncells) {
  if (!c || !p) return SEI_ERR_ARG;
  try {
    c->mesh = sei::HostMesh();
    sei::buildPeriodicCube(*p, c->mesh);
    sei::buildOperators(c->mesh, c->h_star, c->h_aplus, c->h_aminus);
  } catch (const std::invalid_argument& e) {
    return fail(c, SEI_ERR_ARG, e.what());
  } catch (const std::bad_alloc&) {
    return fail(c, SEI_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(c, SEI_ERR_ARG, e.what());
  }
  const int64_t n = c->mesh.n;
  if (c->cfg.device < 0) {  // host-only: keep the host copies
    c->has_mesh = true;
    if (ncells) *ncells = n;
    return SEI_OK;
  }
  int rc = allocArrays(c, n);
  if (rc) return rc;
  rc = uploadCells(c, n, c->h_star.data(), c->h_aplus.data(), c->h_aminus.data(), c->mesh.nbr.data(),
                   c->mesh.side.data(), c->mesh.orient.data(), c->mesh.ftype.data());
  if (rc) return rc;
  std::vector<float> dofs;
  sei::seedDofs(n, c->cfg.order, p->seed, dofs);
  SEI_CUDA(cudaMemcpy(c->Q, dofs.data(), dofs.size() * sizeof(float), cudaMemcpyHostToDevice));
  c->has_mesh = true;
  if (ncells) *ncells = n;
  return SEI_OK;
}

int sei_set_cells(sei_ctx* c, int64_t n, const float* star, const float* aplus, const float* aminus,
                  const int32_t* neighbor, const int8_t* side, const int8_t* orient, const int8_t* face_type) {
  if (!c || !star || !aplus || !aminus || !neighbor || !side || !orient || !face_type) return SEI_ERR_ARG;
  if (c->cfg.device < 0) return fail(c, SEI_ERR_STATE, "host-only context (device < 0) cannot hold cells");
  int rc = allocArrays(c, n);
  if (rc) return rc;
  c->has_mesh = false;
  return uploadCells(c, n, star, aplus, aminus, neighbor, side, orient, face_type);
}

int64_t sei_num_cells(const sei_ctx* c) { return c ? c->n : 0; }

int sei_get_cells(sei_ctx* c, float* star, float* aplus, float* aminus, int32_t* neighbor, int8_t* side, int8_t* orient,
                  int8_t* face_type) {
  if (!c) return SEI_ERR_ARG;
  if (!c->has_mesh) return fail(c, SEI_ERR_STATE, "no host-built mesh in this context");
  const size_t n = (size_t)c->mesh.n;
  if (star) std::memcpy(star, c->h_star.data(), n * 3 * 81 * sizeof(float));
  if (aplus) std::memcpy(aplus, c->h_aplus.data(), n * 4 * 81 * sizeof(float));
  if (aminus) std::memcpy(aminus, c->h_aminus.data(), n * 4 * 81 * sizeof(float));
  if (neighbor) std::memcpy(neighbor, c->mesh.nbr.data(), n * 4 * sizeof(int32_t));
  if (side) std::memcpy(side, c->mesh.side.data(), n * 4);
  if (orient) std::memcpy(orient, c->mesh.orient.data(), n * 4);
  if (face_type) std::memcpy(face_type, c->mesh.ftype.data(), n * 4);
  return SEI_OK;
}

int sei_get_geometry(sei_ctx* c, double* vertices, double* material, int64_t* topology) {
  if (!c) return SEI_ERR_ARG;
  if (!c->has_mesh) return fail(c, SEI_ERR_STATE, "no host-built mesh in this context");
  const size_t n = (size_t)c->mesh.n;
  if (vertices) std::memcpy(vertices, c->mesh.coords.data(), n * 12 * sizeof(double));
  if (material) std::memcpy(material, c->mesh.material.data(), n * 3 * sizeof(double));
  if (topology) std::memcpy(topology, c->mesh.topo.data(), n * 4 * sizeof(int64_t));
  return SEI_OK;
}

int sei_cfl_timestep(sei_ctx* c, double cfl, double* dt) {
  if (!c || !dt || !(cfl > 0)) return SEI_ERR_ARG;
  if (!c->has_mesh) return fail(c, SEI_ERR_STATE, "no host-built mesh in this context");
  *dt = sei::cflTimestep(c->mesh, c->cfg.order, cfl);
  return SEI_OK;
}

int sei_derivatives_size(int order) { return (order >= 2 && order <= 8) ? sei::derivativesSize(order) : 0; }

static int copyDofs(sei_ctx* c, float* dst_dev_or_host, const float* src, bool to_device) {
  // Host arrays are unpadded [n][9][B]; device arrays have column stride Bp.
  const size_t n = (size_t)c->n;
  if (c->B == c->Bp) {
    const size_t bytes = n * 9 * c->B * sizeof(float);
    SEI_CUDA(cudaMemcpyAsync(dst_dev_or_host, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                             c->stream));
  } else {
    SEI_CUDA(cudaMemcpy2DAsync(dst_dev_or_host, (to_device ? c->Bp : c->B) * sizeof(float), src,
                               (to_device ? c->B : c->Bp) * sizeof(float), c->B * sizeof(float), n * 9,
                               to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c->stream));
  }
  return SEI_OK;
}

int sei_set_dofs(sei_ctx* c, const float* dofs) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!dofs) return fail(c, SEI_ERR_ARG, "null dofs");
  rc = copyDofs(c, c->Q, dofs, true);
  if (rc) return rc;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_get_dofs(sei_ctx* c, float* dofs) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!dofs) return fail(c, SEI_ERR_ARG, "null dofs");
  rc = copyDofs(c, dofs, c->Q, false);
  if (rc) return rc;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_get_time_integrated(sei_ctx* c, float* tint) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!tint) return fail(c, SEI_ERR_ARG, "null output");
  rc = copyDofs(c, tint, c->I, false);
  if (rc) return rc;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_get_derivatives(sei_ctx* c, float* derivs) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->derivs) return fail(c, SEI_ERR_STATE, "context created without store_derivatives");
  SEI_CUDA(cudaMemcpyAsync(derivs, c->derivs, (size_t)c->n * sei::derivativesSize(c->cfg.order) * sizeof(float),
                           cudaMemcpyDeviceToHost, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_compute_ader_local(sei_ctx* c, double dt) {
  int rc = checkReady(c);
  if (rc) return rc;
  return runKernel(c, SEI_KERNEL_LOCAL, dt, 1);
}

int sei_compute_neighbors_integral(sei_ctx* c) {
  int rc = checkReady(c);
  if (rc) return rc;
  return runKernel(c, SEI_KERNEL_NEIGHBOR, 0.0, 1);
}

int sei_compute_ader(sei_ctx* c, double) { return fail(c, SEI_ERR_UNSUPPORTED, "ADER alone is not built yet"); }
int sei_compute_local_integral(sei_ctx* c) { return fail(c, SEI_ERR_UNSUPPORTED, "local alone is not built yet"); }

int sei_evaluate_taylor(sei_ctx* c, const double* coeffs, float* out_device) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->derivs) return fail(c, SEI_ERR_STATE, "context created without store_derivatives");
  if (!coeffs || !out_device) return fail(c, SEI_ERR_ARG, "null argument");
  float cf[8];
  for (int i = 0; i < c->cfg.order; ++i) cf[i] = (float)coeffs[i];
  if (c->k.taylor((int)c->n, c->derivs, cf, out_device, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "taylor launch failed");
  return SEI_OK;
}

int sei_run(sei_ctx* c, int kernel, double dt, int nsteps) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (nsteps < 0 || !(dt >= 0) || !std::isfinite(dt)) return fail(c, SEI_ERR_ARG, "invalid dt or step count");
  SEI_CUDA(cudaEventRecord(c->ev0, c->stream));
  rc = runKernel(c, kernel, dt, nsteps);
  if (rc) return rc;
  SEI_CUDA(cudaEventRecord(c->ev1, c->stream));
  return SEI_OK;
}

int sei_run_host(sei_ctx* c, int kernel, double dt, int nsteps, const float* dofs_in, float* dofs_out) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!dofs_in || !dofs_out) return fail(c, SEI_ERR_ARG, "null host buffer");
  rc = copyDofs(c, c->Q, dofs_in, true);
  if (rc) return rc;
  rc = sei_run(c, kernel, dt, nsteps);
  if (rc) return rc;
  rc = copyDofs(c, dofs_out, c->Q, false);
  if (rc) return rc;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_sync(sei_ctx* c) {
  if (!c) return SEI_ERR_ARG;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_last_run_ms(sei_ctx* c, double* ms) {
  if (!c || !ms) return SEI_ERR_ARG;
  float f = 0;
  SEI_CUDA(cudaEventElapsedTime(&f, c->ev0, c->ev1));
  *ms = f;
  return SEI_OK;
}

int sei_set_profiling(sei_ctx* c, int on) {
  if (!c) return SEI_ERR_ARG;
  c->profiling = on != 0;
  c->prof_used = 0;
  return SEI_OK;
}

int sei_kernel_times_ms(sei_ctx* c, double* local_ms, double* neighbor_ms, int* launches) {
  if (!c || !local_ms || !neighbor_ms || !launches) return SEI_ERR_ARG;
  *local_ms = *neighbor_ms = 0.0;
  *launches = 0;
  if (!c->profiling || c->prof_used < 2) return fail(c, SEI_ERR_STATE, "profiling off or nothing recorded");
  SEI_CUDA(cudaEventSynchronize(c->prof_events[c->prof_used - 1]));
  for (size_t i = 0; i + 1 < c->prof_used; ++i) {
    float ms = 0;
    SEI_CUDA(cudaEventElapsedTime(&ms, c->prof_events[i], c->prof_events[i + 1]));
    if (c->prof_kind[i] == 0) *local_ms += ms;
    if (c->prof_kind[i] == 1) *neighbor_ms += ms;
    ++*launches;
  }
  return SEI_OK;
}

int sei_metrics(const sei_ctx* c, int kernel, sei_perf* out) {
  if (!c || !out) return SEI_ERR_ARG;
  (void)kernel;
  std::memset(out, 0, sizeof(*out));
  return SEI_ERR_UNSUPPORTED;
}

}  // extern "C"
