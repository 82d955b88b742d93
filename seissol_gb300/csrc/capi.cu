// C ABI of the GB300 ADER-DG element update (declarations and reference mapping in include/sei_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <limits>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "internal.h"
#include "output.h"
#include "mlp.cuh"

namespace sei {
OrderKernels orderKernels4();
OrderKernels orderKernels5();
OrderKernels orderKernels6();
ViscoKernels viscoKernels4();
ViscoKernels viscoKernels5();
bool viscoKernelsForOrder(int order, ViscoKernels& out) {
  switch (order) {
    case 4: out = viscoKernels4(); return true;
    case 5: out = viscoKernels5(); return true;
    default: return false;
  }
}

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
  int32_t* dslot = nullptr;  // derivative slots (dynamic rupture): only fault cells store derivatives
  uint8_t *rel = nullptr, *ftype = nullptr;
  // host copies of what the context built (for sei_get_cells / sei_get_geometry)
  sei::HostMesh mesh;
  std::vector<float> h_star, h_aplus, h_aminus;
  bool has_mesh = false;
  // dynamic rupture
  sei::HostFault fault;
  bool has_fault = false, dr_ready = false;
  int64_t nslots = 0;  // rows of the derivative buffer
  sei_rs_params rs{};
  int npts = 0;
  int32_t *d_pc = nullptr, *d_mc = nullptr, *d_pslot = nullptr, *d_mslot = nullptr, *d_iters = nullptr;
  uint8_t *d_ps = nullptr, *d_ms = nullptr, *d_rel = nullptr;
  float *d_tinvt = nullptr, *d_fsp = nullptr, *d_fsm = nullptr, *d_isp = nullptr, *d_ism = nullptr;
  double *d_imp = nullptr, *d_state = nullptr;  // state: SEI_DR_NUM_FIELDS fields x [nf][npts]
  double* d_time = nullptr;                       // fault time at the start of the next step
  int dr_law = SEI_LAW_FVW;
  sei_lsw_params lsw{};
  bool dr_nucleate = false;
  bool dr_tp = false;  // thermal pressurisation
  sei_tp_params tp{};
  double* d_tp = nullptr;  // modes [2][60][nf][npts]: temperature, then pressure
  double dr_t0 = 0.0, dr_s0 = 0.0;  // nucleation duration / start (t0 also ramps the forced rupture)
  float* d_mlp = nullptr;  // trained warm-start network (nullptr: none)
  float mlp_norm[sei_mlp::kNorm] = {0};
  bool warm_start = false;
  bool dr_refine32 = false;  // SEI_OPT_DR_REFINE32
  // receivers: the cells in a compact copy (unique cells), basis values at the points
  double sim_time = 0.0;  // start of the next global step (receiver clock)
  int64_t nrecv = 0, nrecv_cells = 0;
  std::vector<int64_t> recv_cell;
  int32_t *d_recv_ucell = nullptr, *d_recv_slot = nullptr;
  float *d_recv_q = nullptr, *d_recv_i = nullptr, *d_recv_star = nullptr, *d_recv_derivs = nullptr;
  float *d_recv_phi = nullptr, *d_recv_dphi = nullptr;
  float *d_recv_grad = nullptr, *d_recv_theta = nullptr;  // viscoelastic: the cells' gradients and attenuation
  double recv_interval = 0.0;
  unsigned recv_qmask = 0;
  int recv_derived = 0, recv_ncols = 0;
  sei::Stager recv_stage;
  // receiver groups: every receiver (global steps), then one per LTS cluster; each group samples
  // the shared time sequence t_0, t_0 + interval, ... (repeated addition) with its own cursor
  std::vector<double> recv_xyz;
  int32_t* d_recv_list = nullptr;    // [2 nrecv]: all receivers in order, then grouped by cluster
  std::vector<int32_t> h_recv_list;
  std::vector<int64_t> recv_gstart;  // [ncl + 1] group offsets into the grouped half
  std::vector<int64_t> recv_next;    // next sample index per group: clusters, then global steps
  std::vector<double> recv_times;
  struct RecvLaunch {
    int64_t k0, first, count;  // rows: m samples x count receivers h_recv_list[first ...]
    int m;
  };
  std::vector<RecvLaunch> recv_log;
  std::map<int64_t, std::pair<std::vector<double>, int64_t>> recv_pending;  // sample -> rows, receivers done
  int64_t recv_emit = 0;
  // fault snapshots every fault_every full steps
  int fault_every = 0;
  int64_t fault_steps = 0;
  std::vector<int> fault_fields;
  sei::Stager fault_stage;
  // off-fault plasticity (sei_plasticity_setup): per-cell parameters at the nodes, current cell order
  bool plast = false;
  double plast_tv = 0.0;
  float* d_plmats = nullptr;  // V, Vinv [2][B][Bp]
  float *d_pls0 = nullptr, *d_plccos = nullptr, *d_plssin = nullptr, *d_plmu = nullptr, *d_pstrain = nullptr;
  unsigned long long* d_plyield = nullptr;
  std::vector<float> pl_s0, pl_ccos, pl_ssin;  // host copies [n][6][B], [n][B], [n][B]
  int tune_fail_at = -1;     // SEI_OPT_TUNE_FAIL_AT: candidate the autotuner fails on the host (tests)
  float* d_rec = nullptr;  // recorded training samples [rec_cap][6]
  unsigned* d_rec_count = nullptr;
  unsigned rec_cap = 0;
  // per-launch timing (sei_set_profiling): one event before every launch plus one at the end
  bool profiling = false;
  bool fused_local = false;  // SEI_OPT_FUSED_LOCAL: ADER and local integral in one launch
  int sms = 0;               // multiprocessors of the device (persistent tensor-core grids)
  int* d_status = nullptr;   // device error word: 1 = a bounded wait in a kernel gave up
  // tensor-core path (SEI_PREC_F16X3): face traces fMrT_f I of every cell, written by the local
  // integral and read by the neighbour kernel; valid while I has not changed since
  float* d_trace = nullptr;
  bool trace_valid = false;
  int tc_local = 0;       // SEI_OPT_TC_LOCAL: 0 FP32 CUDA cores, 1 transposed tensor-core kernel, 2 rows form
  cudaStream_t copy_stream = nullptr;      // host <-> device copies of sei_run_host, beside the compute stream
  std::vector<cudaEvent_t> pipe_events;    // chunk events of the pipelined sei_run_host
  int nb_ctas = 3;        // SEI_OPT_NB_CTAS: persistent CTAs per SM of the rows-form tensor-core neighbour kernel
  int nb_form = 2;        // SEI_OPT_NB_FORM: 2 transposed with the local flux fused in, 1 transposed, 0 rows form
  std::vector<cudaEvent_t> prof_events;
  std::vector<int> prof_kind;  // kind of the launch starting at event i: 0 ADER (or fused ADER + local),
                               // 1 neighbour, 2 fault, 3 local integral, 4 LTS gather / buffer, -1 end of run
  size_t prof_used = 0;
  // local time stepping (sei_lts_setup): cells sorted by cluster; the time-integrated array I is a
  // pool of 9 x Bp blocks: [0, n) the cells' own I, then one integration buffer per cell with a
  // coarser neighbour, then one block per face whose neighbour is coarser (its Taylor integral)
  bool lts = false;
  int ncl = 0;
  double lts_dt0 = 0.0;
  std::vector<int64_t> cl_start, b_start, g_start;  // [ncl + 1] each
  std::vector<int64_t> lts_perm;                    // new cell -> cell before sei_lts_setup
  int64_t npool = 0;                                // pool blocks (cells, buffers, half-step blocks)
  bool lts_trace = false;  // SEI_PREC_F16X3 under LTS: face traces of every pool block, [4][npool][9][FP]
  int32_t* d_src = nullptr;                         // [n][4] pool block read through each face (even sub-step)
  int32_t* d_src1 = nullptr;                        // the same for the odd sub-step of a coarser neighbour's step
  int32_t *d_bcell = nullptr, *d_bdst = nullptr;    // buffer entries, grouped by cluster
  int32_t *d_gsrc = nullptr, *d_gdst = nullptr;     // half-step entries: derivative slot -> first-half block
  int32_t* d_gdst1 = nullptr;                       // second-half block
  int32_t* d_fidx = nullptr;                        // fault faces grouped by cluster
  std::vector<int64_t> f_start;                     // [ncl + 1] ranges of d_fidx
  // viscoelastic (sei_visco_setup): 27 quantities per cell in Q and I
  int nq = 9;
  bool visco = false;
  sei::ViscoKernels vk{};
  float omega[3] = {0, 0, 0};
  double visco_params[4] = {0, 0, 0, 0};  // Qp, Qs, central frequency, frequency ratio
  float *d_grad = nullptr, *d_theta = nullptr, *d_wplus = nullptr, *d_wminus = nullptr;
  std::vector<float> h_grad, h_theta, h_wplus, h_wminus;  // host copies (sei_visco_operators)
  bool lts_graph = false;                           // SEI_OPT_LTS_GRAPH
  bool capturing = false;                           // recording the cycle graph: no profiling events
  cudaGraphExec_t lts_exec = nullptr;               // one recorded cycle
};

namespace {

int fail(sei_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// Named NVTX range for timeline tools (Nsight Systems); host-side, a no-op without a tool.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

int cudaFail(sei_ctx* c, cudaError_t e, const char* what) {
  return fail(c, SEI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// A recorded LTS cycle graph holds the fault kernel's arguments (network, sample buffer); calls
// that change them drop the graph, which the next sei_lts_run records again.
void dropLtsGraph(sei_ctx* c) {
  if (c->lts_exec) cudaGraphExecDestroy(c->lts_exec);
  c->lts_exec = nullptr;
}

#define SEI_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cudaFail(c, e_, #call); \
  } while (0)

void freeFault(sei_ctx* c) {
  for (void* p : {(void*)c->d_pc, (void*)c->d_mc, (void*)c->d_pslot, (void*)c->d_mslot, (void*)c->d_iters, (void*)c->d_ps,
                  (void*)c->d_ms, (void*)c->d_rel, (void*)c->d_tinvt, (void*)c->d_fsp, (void*)c->d_fsm, (void*)c->d_isp,
                  (void*)c->d_ism, (void*)c->d_imp, (void*)c->d_state, (void*)c->d_time, (void*)c->d_tp})
    cudaFree(p);
  c->d_tp = nullptr;
  c->dr_tp = false;
  c->d_pc = c->d_mc = c->d_pslot = c->d_mslot = c->d_iters = nullptr;
  c->d_ps = c->d_ms = c->d_rel = nullptr;
  c->d_tinvt = c->d_fsp = c->d_fsm = c->d_isp = c->d_ism = nullptr;
  c->d_imp = c->d_state = c->d_time = nullptr;
  c->dr_ready = false;
  c->dr_law = SEI_LAW_FVW;
  c->dr_nucleate = false;
  c->dr_t0 = c->dr_s0 = 0.0;
  c->fault_every = 0;  // snapshots describe the fault that is gone
  c->fault_fields.clear();
  c->fault_stage.release();
}

void freePlasticity(sei_ctx* c) {
  for (void* p : {(void*)c->d_plmats, (void*)c->d_pls0, (void*)c->d_plccos, (void*)c->d_plssin, (void*)c->d_plmu,
                  (void*)c->d_pstrain, (void*)c->d_plyield})
    cudaFree(p);
  c->d_plmats = c->d_pls0 = c->d_plccos = c->d_plssin = c->d_plmu = c->d_pstrain = nullptr;
  c->d_plyield = nullptr;
  c->pl_s0.clear();
  c->pl_ccos.clear();
  c->pl_ssin.clear();
  c->plast = false;
  // a recorded LTS cycle holds the plasticity launches (or lacks them): record it again
  if (c->lts_exec) cudaGraphExecDestroy(c->lts_exec);
  c->lts_exec = nullptr;
}

void freeOutput(sei_ctx* c) {
  for (void* p : {(void*)c->d_recv_ucell, (void*)c->d_recv_slot, (void*)c->d_recv_q, (void*)c->d_recv_i,
                  (void*)c->d_recv_star, (void*)c->d_recv_derivs, (void*)c->d_recv_phi, (void*)c->d_recv_dphi,
                  (void*)c->d_recv_list, (void*)c->d_recv_grad, (void*)c->d_recv_theta})
    cudaFree(p);
  c->d_recv_ucell = c->d_recv_slot = c->d_recv_list = nullptr;
  c->d_recv_q = c->d_recv_i = c->d_recv_star = c->d_recv_derivs = c->d_recv_phi = c->d_recv_dphi = nullptr;
  c->d_recv_grad = c->d_recv_theta = nullptr;
  c->nrecv = c->nrecv_cells = 0;
  c->recv_cell.clear();
  c->recv_xyz.clear();
  c->recv_log.clear();
  c->recv_pending.clear();
  c->recv_stage.release();
  c->fault_every = 0;
  c->fault_fields.clear();
  c->fault_stage.release();
}

void freeArrays(sei_ctx* c) {
  freeOutput(c);
  freePlasticity(c);
  cudaFree(c->Q);
  cudaFree(c->I);
  cudaFree(c->derivs);
  cudaFree(c->star_nz);
  cudaFree(c->aplus);
  cudaFree(c->aminus);
  cudaFree(c->nbr);
  cudaFree(c->rel);
  cudaFree(c->ftype);
  cudaFree(c->dslot);
  cudaFree(c->d_trace);
  c->d_trace = nullptr;
  c->trace_valid = false;
  for (void* p : {(void*)c->d_src, (void*)c->d_src1, (void*)c->d_bcell, (void*)c->d_bdst, (void*)c->d_gsrc,
                  (void*)c->d_gdst, (void*)c->d_gdst1, (void*)c->d_fidx,
                  (void*)c->d_grad, (void*)c->d_theta, (void*)c->d_wplus, (void*)c->d_wminus})
    cudaFree(p);
  c->d_grad = c->d_theta = c->d_wplus = c->d_wminus = nullptr;
  c->visco = false;
  c->nq = 9;
  c->d_src = c->d_src1 = c->d_bcell = c->d_bdst = c->d_gsrc = c->d_gdst = c->d_gdst1 = c->d_fidx = nullptr;
  if (c->lts_exec) cudaGraphExecDestroy(c->lts_exec);
  c->lts_exec = nullptr;
  c->lts = false;
  c->lts_trace = false;
  c->npool = 0;
  c->ncl = 0;
  freeFault(c);
  c->dslot = nullptr;
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
  if (ok && c->cfg.store_derivatives) {
    ok = alloc((void**)&c->derivs, (size_t)n * sei::derivativesSize(c->cfg.order) * sizeof(float));
    c->nslots = n;
  }
  const size_t trace_bytes = (size_t)n * sei::traceFloatsPerCell(c->cfg.order) * sizeof(float);
  if (ok && c->cfg.precision == SEI_PREC_F16X3) ok = alloc((void**)&c->d_trace, trace_bytes);
  if (!ok) {
    cudaGetLastError();
    freeArrays(c);
    return fail(c, SEI_ERR_OOM, "device allocation failed");
  }
  c->n = n;
  if (cudaMemsetAsync(c->Q, 0, dof, c->stream) != cudaSuccess || cudaMemsetAsync(c->I, 0, dof, c->stream) != cudaSuccess ||
      (c->d_trace && cudaMemsetAsync(c->d_trace, 0, trace_bytes, c->stream) != cudaSuccess))
    return fail(c, SEI_ERR_CUDA, "memset failed");
  return SEI_OK;
}

// The checks of a caller's cell data, made before anything of the context changes: face types,
// neighbours and relations in range, the used star entries finite.
int validateCells(sei_ctx* c, int64_t n, const float* star, const int32_t* nbr, const int8_t* side, const int8_t* orient,
                  const int8_t* ftype) {
  if (n <= 0 || n > INT32_MAX) return fail(c, SEI_ERR_ARG, "cell count out of range");
  for (int64_t i = 0; i < n * 4; ++i) {
    if (ftype[i] < 0 || ftype[i] > 2) return fail(c, SEI_ERR_ARG, "face_type must be 0, 1 or 2");
    if (ftype[i] == 0) {
      if (nbr[i] < 0 || nbr[i] >= n) return fail(c, SEI_ERR_ARG, "regular face with neighbour out of range");
      if (side[i] < 0 || side[i] > 3 || orient[i] < 0 || orient[i] > 2)
        return fail(c, SEI_ERR_ARG, "face relation out of range (side 0..3, orientation 0..2)");
    }
  }
  for (int64_t i = 0; i < n; ++i)
    for (int e = 0; e < 3; ++e)
      for (int z = 0; z < sei::kStarNnz; ++z)
        if (!std::isfinite(star[(i * 3 + e) * 81 + sei::kStarNz[z][0] + 9 * sei::kStarNz[z][1]]))
          return fail(c, SEI_ERR_NAN, "non-finite star matrix entry");
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
  sei::DeviceArrays d{(int)c->n, c->Q, c->I, c->derivs, c->dslot, c->star_nz, c->aplus, c->aminus, c->nbr, c->rel, c->ftype};
  d.status = c->d_status;
  return d;
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
  if (!c->profiling || c->capturing) return SEI_OK;
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

int launchAderOnly(sei_ctx* c, const sei::DeviceArrays& d, const float* coeffs) {
  int rc = profMark(c, 0);
  if (rc) return rc;
  c->trace_valid = false;
  if (c->k.ader(d, coeffs, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "ADER kernel launch failed");
  return SEI_OK;
}

// True when a step of kernel 'all' runs the local flux inside the tensor-core neighbour kernel
// (SEI_OPT_NB_FORM 2): the local integral then computes the volume term and the traces only.
bool fusedFlux(const sei_ctx* c) {
  return c->cfg.precision == SEI_PREC_F16X3 && c->nb_form == 2 && (c->tc_local == 0 || c->lts) &&
         (!c->lts || c->lts_trace) && c->d_trace;
}

// The tensor-core neighbour path with stored face traces is on: global stepping, or local time
// stepping whose cycle keeps the traces of every pool block.
bool traceNeighbor(const sei_ctx* c) {
  return c->cfg.precision == SEI_PREC_F16X3 && c->d_trace && (!c->lts || c->lts_trace);
}

int launchLintOnly(sei_ctx* c, const sei::DeviceArrays& d, bool volumeOnly = false) {
  int rc = profMark(c, 3);
  if (rc) return rc;
  // the traces cover every cell only outside local time stepping (whose kernels run per cluster);
  // a view of a range of cells writes its part ([4][n][9][FP], face-major)
  float* trace = traceNeighbor(c)
                     ? c->d_trace + (size_t)d.first * 9 * ((sei::numFaceBasis(c->cfg.order) + 3) / 4 * 4)
                     : nullptr;
  if (c->cfg.precision == SEI_PREC_F16X3 && c->tc_local && !c->lts) {
    const int lrc = c->tc_local == 1 ? sei::launchLintTransposed(c->cfg.order, d, trace, 0, c->d_status, c->sms, c->stream)
                                     : sei::launchLintTensorCore(c->cfg.order, d, trace, 0, c->d_status, c->sms, c->stream);
    if (lrc != 0) return fail(c, SEI_ERR_CUDA, "tensor-core local-integral kernel launch failed");
  } else {
    sei::DeviceArrays dt = d;
    dt.trace = trace;
    const bool vol = volumeOnly && trace != nullptr;
    if ((vol ? c->k.lintVol(dt, c->stream) : c->k.lint(dt, c->stream)) != 0)
      return fail(c, SEI_ERR_CUDA, "local-integral kernel launch failed");
  }
  c->trace_valid = trace != nullptr && d.n == c->n;
  return SEI_OK;
}

// ADER followed by the local integral: two launches (default) or one fused launch.
int launchLocal(sei_ctx* c, const sei::DeviceArrays& d, const float* coeffs, bool volumeOnly = false) {
  if (volumeOnly && c->fused_local) {
    // fused-flux path: ADER, volume and face traces in one launch, I stays on chip
    int rc = profMark(c, 0);
    if (rc) return rc;
    sei::DeviceArrays dt = d;
    dt.trace = c->d_trace + (size_t)d.first * 9 * ((sei::numFaceBasis(c->cfg.order) + 3) / 4 * 4);
    if (c->k.localVol(dt, coeffs, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "ADER-volume-trace kernel launch failed");
    c->trace_valid = d.n == c->n;
    return SEI_OK;
  }
  if (!c->fused_local || c->cfg.precision != SEI_PREC_FP32) {
    int rc = launchAderOnly(c, d, coeffs);
    return rc ? rc : launchLintOnly(c, d, volumeOnly);
  }
  int rc = profMark(c, 0);
  if (rc) return rc;
  if (c->k.local(d, coeffs, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "local kernel launch failed");
  return SEI_OK;
}

int launchNeighbor(sei_ctx* c, const sei::DeviceArrays& d, bool withLocal = false) {
  int rc = profMark(c, 1);
  if (rc) return rc;
  if (traceNeighbor(c)) {
    // tensor-core path: the neighbour flux reads the stored face traces of I; they are
    // recomputed first when I changed after the last local integral (under local time stepping
    // the cycle keeps the traces of every pool block current)
    if (!c->lts && !c->trace_valid) {
      if (sei::launchLintTransposed(c->cfg.order, d, c->d_trace, 1, c->d_status, c->sms, c->stream) != 0)
        return fail(c, SEI_ERR_CUDA, "tensor-core trace kernel launch failed");
      c->trace_valid = true;
    }
    const int lrc = (c->nb_form || c->lts)
                        ? sei::launchNeighborTransposed(c->cfg.order, d, c->d_trace, c->d_status, c->sms, c->stream,
                                                        withLocal && c->nb_form == 2)
                               : sei::launchNeighborTensorCore(c->cfg.order, d, c->d_trace, c->d_status, c->sms,
                                                               c->nb_ctas, c->stream);
    if (lrc != 0) return fail(c, SEI_ERR_CUDA, "tensor-core neighbour kernel launch failed");
    return SEI_OK;
  }
  if (c->k.neighbor(d, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "neighbour kernel launch failed");
  return SEI_OK;
}

sei::DrArgs drArgs(sei_ctx* c, double dt) {
  sei::DrArgs a{};
  const int64_t nf = c->fault.nf, np = c->npts;
  a.nfaces = (int)nf;
  a.fidx = nullptr;
  a.face_begin = 0;
  a.face_count = (int)nf;
  a.plus_cell = c->d_pc;
  a.minus_cell = c->d_mc;
  a.plus_side = c->d_ps;
  a.minus_side = c->d_ms;
  a.rel = c->d_rel;
  a.plus_slot = c->d_pslot;
  a.minus_slot = c->d_mslot;
  a.derivs = c->derivs;
  a.tinvt = c->d_tinvt;
  a.fsp = c->d_fsp;
  a.fsm = c->d_fsm;
  a.imp = c->d_imp;
  double* st = c->d_state;
  auto field = [&](int k) { return st + (size_t)k * nf * np; };
  a.psi = field(SEI_DR_PSI);
  a.v1 = field(SEI_DR_SLIP_RATE1);
  a.v2 = field(SEI_DR_SLIP_RATE2);
  a.slip1 = field(SEI_DR_SLIP1);
  a.slip2 = field(SEI_DR_SLIP2);
  a.slip = field(SEI_DR_SLIP);
  a.mu = field(SEI_DR_MU);
  a.trac1 = field(SEI_DR_TRACTION1);
  a.trac2 = field(SEI_DR_TRACTION2);
  a.a = field(SEI_DR_A);
  a.init = field(SEI_DR_SN0);  // sn0, tau1_0, tau2_0 are consecutive fields: [3][nf][npts]
  a.isp = c->d_isp;
  a.ism = c->d_ism;
  a.newton_iters = c->d_iters;
  a.Q = c->Q;
  const sei_rs_params& r = c->rs;
  a.f0 = r.f0;
  a.b = r.b;
  a.v0 = r.v0;
  a.l = r.l;
  a.muw = r.muw;
  a.vw = r.vw;
  a.newton_tol = r.newton_tol;
  a.state_tol = r.state_tol;
  a.max_newton = r.max_newton;
  a.max_outer = r.max_outer;
  a.refine32 = c->dr_refine32 ? 1 : 0;
  // Gauss-Legendre time points on [0, dt] (TimeCluster.cpp:236-241), sub-steps (FrictionSolver.cpp:20-37)
  const int N = c->cfg.order;
  double x[8], w[8];
  sei::gaussLegendre01(N, x, w);
  for (int s = 0; s < N; ++s) {
    const double t = x[s] * dt;
    a.tweights[s] = w[s] * dt;
    a.deltat[s] = s == 0 ? t : t - x[s - 1] * dt;
    double v = 1.0;
    for (int p = 0; p < N; ++p) {
      a.coll[s][p] = (float)v;  // t^p / p!
      v *= t / (p + 1);
    }
  }
  a.deltat[N - 1] += x[0] * dt;
  a.mlp = c->warm_start && c->dr_law == SEI_LAW_FVW ? c->d_mlp : nullptr;
  for (int i = 0; i < sei_mlp::kNorm; ++i) a.mlp_norm[i] = c->mlp_norm[i];
  a.rec = c->d_rec;
  a.rec_count = c->d_rec_count;
  a.rec_cap = c->rec_cap;
  a.law = c->dr_law;
  a.time = c->d_time;
  a.time_offset = 0.0;
  a.t0 = c->dr_t0;
  a.s0 = c->dr_s0;
  a.nucleate = c->dr_nucleate ? 1 : 0;
  a.nuc = field(SEI_DR_NUC_SN);  // nucleation sn, tau1, tau2: consecutive fields
  a.peak = field(SEI_DR_PEAK_SLIP_RATE);
  a.trup = field(SEI_DR_RUPTURE_TIME);
  a.tdyn = field(SEI_DR_DYN_STRESS_TIME);
  a.mu_s = field(SEI_DR_MU_S);
  a.mu_d = field(SEI_DR_MU_D);
  a.d_c = field(SEI_DR_D_C);
  a.cohesion = field(SEI_DR_COHESION);
  a.t_forced = field(SEI_DR_FORCED_RUPTURE_TIME);
  a.reg = field(SEI_DR_REG_STRENGTH);
  a.healing = c->lsw.healing_threshold;
  a.v_star = c->lsw.v_star;
  a.prakash_length = c->lsw.prakash_length > 0 ? c->lsw.prakash_length : 1.0;
  a.tp_exponent = c->lsw.tp_proxy_exponent;
  a.tp = c->dr_tp ? 1 : 0;
  a.tp_alpha = c->tp.thermal_diffusivity;
  a.tp_rhoc = c->tp.heat_capacity;
  a.tp_lambda = c->tp.undrained_tp_response;
  a.tp_t0 = c->tp.initial_temperature;
  a.tp_p0 = c->tp.initial_pressure;
  a.tp_hw = field(SEI_DR_TP_HALF_WIDTH);
  a.tp_hyd = field(SEI_DR_TP_HYDRAULIC_DIFFUSIVITY);
  a.tp_temp = field(SEI_DR_TP_TEMPERATURE);
  a.tp_pres = field(SEI_DR_TP_PRESSURE);
  a.tp_theta = c->d_tp;
  a.tp_sigma = c->d_tp ? c->d_tp + (size_t)sei::kTpModes * nf * np : nullptr;
  a.dir1 = field(SEI_DR_SLIP_DIR1);
  a.dir2 = field(SEI_DR_SLIP_DIR2);
  a.onset = field(SEI_DR_ONSET_TIME);
  a.taus = field(SEI_DR_TAU_S);
  a.taur = field(SEI_DR_TAU_R);
  return a;
}

int launchDr(sei_ctx* c, double dt) {
  NvtxRange range("sei fault step");
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up (sei_dr_setup)");
  int rc = profMark(c, 2);
  if (rc) return rc;
  if (sei::launchDrFaces(c->cfg.order, drArgs(c, dt), c->stream) != 0) return fail(c, SEI_ERR_CUDA, "fault kernel launch failed");
  if (sei::launchDrAdvanceTime(c->d_time, dt, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "fault time launch failed");
  return SEI_OK;
}

sei::ViscoArrays viscoArrays(sei_ctx* c) {
  sei::ViscoArrays v{};
  v.n = (int)c->n;
  v.Q = c->Q;
  v.I = c->I;
  v.star_nz = c->star_nz;
  v.grad = c->d_grad;
  v.theta = c->d_theta;
  v.aplus = c->aplus;
  v.wplus = c->d_wplus;
  v.aminus = c->aminus;
  v.wminus = c->d_wminus;
  v.nbr = c->nbr;
  v.rel = c->rel;
  v.ftype = c->ftype;
  for (int i = 0; i < 3; ++i) v.omega[i] = c->omega[i];
  return v;
}

int recordReceivers(sei_ctx* c, int g, double T, double dt, int64_t first, int64_t count);

// Viscoelastic steps: ADER, volume + local flux, neighbour flux (kernel kinds 0, 3, 1).
int runVisco(sei_ctx* c, int kernel, double dt, int steps, const double* given = nullptr) {
  float coeffs[8];
  taylorCoeffs(c->cfg.order, dt, coeffs);
  if (given)
    for (int i = 0; i < c->cfg.order; ++i) coeffs[i] = (float)given[i];
  const sei::ViscoArrays v = viscoArrays(c);
  const bool ader = kernel == SEI_KERNEL_ALL || kernel == SEI_KERNEL_LOCAL || kernel == SEI_KERNEL_ADER;
  const bool lint = kernel == SEI_KERNEL_ALL || kernel == SEI_KERNEL_LOCAL || kernel == SEI_KERNEL_LOCAL_WO_ADER;
  const bool nbr = kernel == SEI_KERNEL_ALL || kernel == SEI_KERNEL_NEIGHBOR;
  if (!ader && !lint && !nbr) return fail(c, SEI_ERR_UNSUPPORTED, "kernel not built for the viscoelastic equations");
  c->prof_used = 0;
  int rc = SEI_OK;
  for (int s = 0; s < steps && rc == SEI_OK; ++s) {
    if (kernel == SEI_KERNEL_ALL && c->nrecv &&
        (rc = recordReceivers(c, (int)c->recv_next.size() - 1, c->sim_time, dt, 0, c->nrecv)))
      break;
    if (ader && !(rc = profMark(c, 0)) && c->vk.ader(v, coeffs, c->stream)) rc = fail(c, SEI_ERR_CUDA, "viscoelastic ADER launch failed");
    if (!rc && lint && !(rc = profMark(c, 3)) && c->vk.lint(v, c->stream))
      rc = fail(c, SEI_ERR_CUDA, "viscoelastic local-integral launch failed");
    if (!rc && nbr && !(rc = profMark(c, 1)) && c->vk.neighbor(v, c->stream))
      rc = fail(c, SEI_ERR_CUDA, "viscoelastic neighbour launch failed");
    if (!rc && kernel == SEI_KERNEL_ALL) c->sim_time += dt;
  }
  if (!rc) rc = profMark(c, -1);
  return rc;
}

// given: time-basis coefficients of the predictor's time integral (nullptr: MonomialBasis::integrate(0, dt))
double recvTime(sei_ctx* c, int64_t k) {
  while ((int64_t)c->recv_times.size() <= k) c->recv_times.push_back(c->recv_times.back() + c->recv_interval);
  return c->recv_times[k];
}

// Receiver samples of group g for the step [T, T + dt) from the DOFs at its start
// (Receiver.cpp:118-214): the CK derivatives of the receiver cells (ADER on their compact copy),
// then the group's receivers h_recv_list[first, first + count) at every sampling time inside the
// step, in batches of kRecvMaxSamples; each batch is logged for the host-side assembly.
int recordReceivers(sei_ctx* c, int g, double T, double dt, int64_t first, int64_t count) {
  NvtxRange range("sei receivers");
  if (c->nrecv == 0 || count == 0) return SEI_OK;
  int64_t& k = c->recv_next[g];
  if (!(recvTime(c, k) < T + dt)) return SEI_OK;
  const int blk = c->nq * c->Bp;
  if (sei::launchGatherRows((int)c->nrecv_cells, c->d_recv_ucell, c->Q, c->d_recv_q, blk, c->stream))
    return fail(c, SEI_ERR_CUDA, "receiver gather launch failed");
  float co[8];
  taylorCoeffs(c->cfg.order, dt, co);
  if (c->visco) {
    sei::ViscoArrays v{};
    v.n = (int)c->nrecv_cells;
    v.Q = c->d_recv_q;
    v.I = c->d_recv_i;
    v.star_nz = c->d_recv_star;
    v.grad = c->d_recv_grad;
    v.theta = c->d_recv_theta;
    for (int i = 0; i < 3; ++i) v.omega[i] = c->omega[i];
    v.derivs = c->d_recv_derivs;
    v.dslot = nullptr;
    if (c->vk.ader(v, co, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "receiver ADER launch failed");
  } else {
    sei::DeviceArrays d{};
    d.n = (int)c->nrecv_cells;
    d.Q = c->d_recv_q;
    d.I = c->d_recv_i;
    d.derivs = c->d_recv_derivs;
    d.dslot = nullptr;
    d.star_nz = c->d_recv_star;
    if (c->k.ader(d, co, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "receiver ADER launch failed");
  }
  sei::RecvEvalArgs a{};
  a.nrecv = (int)count;
  a.list = c->d_recv_list + first;
  a.slot = c->d_recv_slot;
  a.derivs = c->d_recv_derivs;
  a.phi = c->d_recv_phi;
  a.dphi = c->d_recv_dphi;
  a.time0 = T;
  a.qmask = c->recv_qmask;
  a.derived = c->recv_derived;
  a.ncols = c->recv_ncols;
  a.visco = c->visco ? 1 : 0;
  while (recvTime(c, k) < T + dt) {
    const int64_t k0 = k;
    a.nsamples = 0;
    while (a.nsamples < sei::kRecvMaxSamples && recvTime(c, k) < T + dt) a.offset[a.nsamples++] = recvTime(c, k++) - T;
    int err = 0;
    a.out = static_cast<double*>(c->recv_stage.reserve((size_t)a.nsamples * count, c->stream, &err));
    if (!a.out) return fail(c, SEI_ERR_CUDA, "receiver staging failed");
    if (sei::launchRecvEval(c->cfg.order, a, c->stream)) return fail(c, SEI_ERR_CUDA, "receiver evaluation launch failed");
    c->recv_log.push_back({k0, first, count, a.nsamples});
  }
  return SEI_OK;
}

// A snapshot of the selected fault fields after every fault_every-th full step: the fault time,
// then each field [nf][npts], copied on the device into the staging ring.
int recordFault(sei_ctx* c) {
  if (c->fault_every <= 0 || !c->dr_ready || ++c->fault_steps % c->fault_every) return SEI_OK;
  int err = 0;
  double* row = static_cast<double*>(c->fault_stage.reserve(1, c->stream, &err));
  if (!row) return fail(c, SEI_ERR_CUDA, "fault output staging failed");
  const size_t plane = (size_t)c->fault.nf * c->npts;
  SEI_CUDA(cudaMemcpyAsync(row, c->d_time, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  for (size_t i = 0; i < c->fault_fields.size(); ++i)
    SEI_CUDA(cudaMemcpyAsync(row + 1 + i * plane, c->d_state + (size_t)c->fault_fields[i] * plane, plane * sizeof(double),
                             cudaMemcpyDeviceToDevice, c->stream));
  return SEI_OK;
}

// Plasticity of cells [s, e) after their neighbour integral over a step of dt
// (TimeCluster.cpp:966-975, Plasticity::computeRelaxTime).
int launchPlast(sei_ctx* c, int64_t s, int64_t e, double dt) {
  if (!c->plast || e <= s) return SEI_OK;
  int rc = profMark(c, 4);  // not one of the four reported kinds
  if (rc) return rc;
  sei::PlasticityArgs a{};
  a.Q = c->Q;
  a.mats = c->d_plmats;
  a.s0 = c->d_pls0;
  a.ccos = c->d_plccos;
  a.ssin = c->d_plssin;
  a.mufac = c->d_plmu;
  a.pstrain = c->d_pstrain;
  a.yield = c->d_plyield;
  a.begin = s;
  a.end = e;
  const double r = sei_plasticity_relax_factor(c->plast_tv, dt);
  a.relax = (float)r;
  a.inv_tvr = (float)(1.0 / (c->plast_tv * r));
  a.dt = (float)dt;
  if (sei::launchPlasticity(c->cfg.order, a, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "plasticity launch failed");
  return SEI_OK;
}

int runKernel(sei_ctx* c, int kernel, double dt, int steps, const double* given = nullptr) {
  if (c->visco) return runVisco(c, kernel, dt, steps, given);
  float coeffs[8];
  taylorCoeffs(c->cfg.order, dt, coeffs);
  if (given)
    for (int i = 0; i < c->cfg.order; ++i) coeffs[i] = (float)given[i];
  sei::DeviceArrays d = arrays(c);
  c->prof_used = 0;
  int rc = SEI_OK;
  const bool fullStep = kernel == SEI_KERNEL_ALL || kernel == SEI_KERNEL_ALL_DR;
  for (int s = 0; s < steps && rc == SEI_OK; ++s) {
    NvtxRange range("sei step");
    if (fullStep && c->nrecv &&
        (rc = recordReceivers(c, (int)c->recv_next.size() - 1, c->sim_time, dt, 0, c->nrecv)))
      return rc;
    switch (kernel) {
      case SEI_KERNEL_ALL:
        rc = launchLocal(c, d, coeffs, fusedFlux(c));
        if (!rc) rc = launchNeighbor(c, d, fusedFlux(c));
        if (!rc) rc = launchPlast(c, 0, c->n, dt);
        break;
      case SEI_KERNEL_LOCAL:
        rc = launchLocal(c, d, coeffs);
        break;
      case SEI_KERNEL_ADER:
        rc = launchAderOnly(c, d, coeffs);
        break;
      case SEI_KERNEL_LOCAL_WO_ADER:
        rc = launchLintOnly(c, d);
        break;
      case SEI_KERNEL_NEIGHBOR:
      case SEI_KERNEL_NEIGHBOR_DR:
        rc = launchNeighbor(c, d);
        break;
      case SEI_KERNEL_GODUNOV_DR:
        rc = launchDr(c, dt);
        break;
      case SEI_KERNEL_ALL_DR:
        rc = launchLocal(c, d, coeffs, fusedFlux(c));
        if (!rc) rc = launchDr(c, dt);
        if (!rc) rc = launchNeighbor(c, d, fusedFlux(c));
        if (!rc) rc = launchPlast(c, 0, c->n, dt);
        break;
      default:
        return fail(c, SEI_ERR_UNSUPPORTED, "kernel not supported by this build");
    }
    if (fullStep && rc == SEI_OK) {
      c->sim_time += dt;
      rc = recordFault(c);
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
  if (cfg->precision != SEI_PREC_FP32 && cfg->precision != SEI_PREC_F16X3) {
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
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess ||
      cudaMalloc(&c->d_status, sizeof(int)) != cudaSuccess || cudaMemset(c->d_status, 0, sizeof(int)) != cudaSuccess) {
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
  cudaFree(c->d_status);
  cudaFree(c->d_rec);
  cudaFree(c->d_rec_count);
  cudaFree(c->d_mlp);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t e : c->pipe_events) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* sei_last_error(const sei_ctx* c) { return c ? c->err.c_str() : "null context"; }

int sei_build_periodic_cube(sei_ctx* c, const sei_cube_params* p, int64_t* ncells) {
  if (!c || !p) return SEI_ERR_ARG;
  try {
    c->mesh = sei::HostMesh();
    sei::buildPeriodicCube(*p, c->mesh);
    c->has_fault = false;
    if (p->fault_plane >= 0) {
      if (p->fault_plane < 1 || p->fault_plane > p->nx - 1)
        throw std::invalid_argument("fault_plane must lie in 1..nx-1 (or -1 for no fault)");
      sei::buildPlanarFault(c->mesh, c->mesh.fault_x, p->h, c->fault);
      sei::faultFaceData(c->mesh, c->fault);
      c->has_fault = true;
    }
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

int sei_set_mesh(sei_ctx* c, const sei_mesh* p, int64_t* ncells, int64_t* nfaults) {
  if (!c || !p) return SEI_ERR_ARG;
  sei::HostMesh mesh;
  sei::HostFault fault;
  std::vector<float> star, aplus, aminus;
  try {
    sei::ingestMesh(*p, mesh, fault);
    sei::buildOperators(mesh, star, aplus, aminus);
  } catch (const std::domain_error& e) {
    return fail(c, SEI_ERR_UNSUPPORTED, e.what());
  } catch (const std::bad_alloc&) {
    return fail(c, SEI_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(c, SEI_ERR_ARG, e.what());
  }
  const int64_t n = mesh.n;
  if (c->cfg.device >= 0) {
    int rc = allocArrays(c, n);
    if (rc) return rc;
    rc = uploadCells(c, n, star.data(), aplus.data(), aminus.data(), mesh.nbr.data(), mesh.side.data(),
                     mesh.orient.data(), mesh.ftype.data());
    if (rc) return rc;
    SEI_CUDA(cudaMemset(c->Q, 0, (size_t)n * c->nq * c->Bp * sizeof(float)));
  }
  c->mesh = std::move(mesh);
  c->fault = std::move(fault);
  c->h_star = std::move(star);
  c->h_aplus = std::move(aplus);
  c->h_aminus = std::move(aminus);
  c->has_fault = c->fault.nf > 0;
  c->has_mesh = true;
  if (ncells) *ncells = n;
  if (nfaults) *nfaults = c->fault.nf;
  return SEI_OK;
}

int sei_set_cells(sei_ctx* c, int64_t n, const float* star, const float* aplus, const float* aminus,
                  const int32_t* neighbor, const int8_t* side, const int8_t* orient, const int8_t* face_type) {
  if (!c || !star || !aplus || !aminus || !neighbor || !side || !orient || !face_type) return SEI_ERR_ARG;
  if (c->cfg.device < 0) return fail(c, SEI_ERR_STATE, "host-only context (device < 0) cannot hold cells");
  int rc = validateCells(c, n, star, neighbor, side, orient, face_type);  // a rejected call changes nothing
  if (rc) return rc;
  rc = allocArrays(c, n);
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
  // Host arrays are unpadded [n][nq][B]; device arrays have column stride Bp.
  const size_t n = (size_t)c->n;
  if (c->B == c->Bp) {
    const size_t bytes = n * c->nq * c->B * sizeof(float);
    SEI_CUDA(cudaMemcpyAsync(dst_dev_or_host, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                             c->stream));
  } else {
    SEI_CUDA(cudaMemcpy2DAsync(dst_dev_or_host, (to_device ? c->Bp : c->B) * sizeof(float), src,
                               (to_device ? c->B : c->Bp) * sizeof(float), c->B * sizeof(float), n * c->nq,
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
  SEI_CUDA(cudaMemcpyAsync(derivs, c->derivs, (size_t)c->nslots * sei::derivativesSize(c->cfg.order) * sizeof(float),
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

int sei_compute_ader(sei_ctx* c, const double* coeffs, double dt) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (coeffs)
    for (int i = 0; i < c->cfg.order; ++i)
      if (!std::isfinite(coeffs[i])) return fail(c, SEI_ERR_ARG, "non-finite time-basis coefficient");
  if (!coeffs && !(dt > 0)) return fail(c, SEI_ERR_ARG, "dt > 0 needed when no coefficients are given");
  return runKernel(c, SEI_KERNEL_ADER, dt, 1, coeffs);
}

int sei_compute_local_integral(sei_ctx* c) {
  int rc = checkReady(c);
  if (rc) return rc;
  return runKernel(c, SEI_KERNEL_LOCAL_WO_ADER, 0.0, 1);
}

int sei_set_option(sei_ctx* c, int option, int value) {
  if (!c) return SEI_ERR_ARG;
  switch (option) {
    case SEI_OPT_FUSED_LOCAL:
      c->fused_local = value != 0;
      return SEI_OK;
    case SEI_OPT_LTS_GRAPH:
      c->lts_graph = value != 0;
      return SEI_OK;
    case SEI_OPT_TC_LOCAL:
      if (value < 0 || value > 2) return fail(c, SEI_ERR_ARG, "SEI_OPT_TC_LOCAL takes 0, 1 or 2");
      c->tc_local = value;
      c->trace_valid = false;
      return SEI_OK;
    case SEI_OPT_NB_CTAS:
      if (value < 1 || value > 3) return fail(c, SEI_ERR_ARG, "SEI_OPT_NB_CTAS takes 1, 2 or 3");
      c->nb_ctas = value;
      return SEI_OK;
    case SEI_OPT_NB_FORM:
      if (value < 0 || value > 2) return fail(c, SEI_ERR_ARG, "SEI_OPT_NB_FORM takes 0, 1 or 2");
      c->nb_form = value;
      return SEI_OK;
    case SEI_OPT_DR_REFINE32:
      c->dr_refine32 = value != 0;
      dropLtsGraph(c);  // a recorded cycle holds the fault kernel's arguments
      return SEI_OK;
    case SEI_OPT_TUNE_FAIL_AT:
      c->tune_fail_at = value;
      return SEI_OK;
    default:
      return fail(c, SEI_ERR_ARG, "unknown option");
  }
}

int sei_get_option(sei_ctx* c, int option, int* value) {
  if (!c || !value) return SEI_ERR_ARG;
  switch (option) {
    case SEI_OPT_FUSED_LOCAL: *value = c->fused_local ? 1 : 0; return SEI_OK;
    case SEI_OPT_LTS_GRAPH: *value = c->lts_graph ? 1 : 0; return SEI_OK;
    case SEI_OPT_TC_LOCAL: *value = c->tc_local; return SEI_OK;
    case SEI_OPT_NB_CTAS: *value = c->nb_ctas; return SEI_OK;
    case SEI_OPT_NB_FORM: *value = c->nb_form; return SEI_OK;
    case SEI_OPT_DR_REFINE32: *value = c->dr_refine32 ? 1 : 0; return SEI_OK;
    case SEI_OPT_TUNE_FAIL_AT: *value = c->tune_fail_at; return SEI_OK;
    default: return fail(c, SEI_ERR_ARG, "unknown option");
  }
}

int sei_evaluate_taylor(sei_ctx* c, const double* coeffs, float* out_device) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->derivs || c->dslot) return fail(c, SEI_ERR_STATE, "derivatives of all cells are not stored (store_derivatives off or fault slots)");
  if (!coeffs || !out_device) return fail(c, SEI_ERR_ARG, "null argument");
  float cf[8];
  for (int i = 0; i < c->cfg.order; ++i) cf[i] = (float)coeffs[i];
  if (c->k.taylor((int)c->n, c->derivs, cf, out_device, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "taylor launch failed");
  return SEI_OK;
}

int sei_run(sei_ctx* c, int kernel, double dt, int nsteps) {
  NvtxRange range("sei_run");
  int rc = checkReady(c);
  if (rc) return rc;
  if (nsteps < 0 || !(dt >= 0) || !std::isfinite(dt)) return fail(c, SEI_ERR_ARG, "invalid dt or step count");
  SEI_CUDA(cudaEventRecord(c->ev0, c->stream));
  rc = runKernel(c, kernel, dt, nsteps);
  if (rc) return rc;
  SEI_CUDA(cudaEventRecord(c->ev1, c->stream));
  return SEI_OK;
}

// A range [s, e) of the cells for global stepping: the cell-indexed arrays start at s, the
// neighbour flux reads the time-integrated DOFs (and traces) of the whole mesh.
static sei::DeviceArrays gtsRange(sei_ctx* c, int64_t s, int64_t e, bool neighbour) {
  const size_t blk = (size_t)9 * c->Bp;
  sei::DeviceArrays d = arrays(c);
  d.n = (int)(e - s);
  d.ntotal = (int)c->n;
  d.first = (int)s;
  d.Q = c->Q + s * blk;
  d.I = neighbour ? c->I : c->I + s * blk;
  d.derivs = c->derivs ? (c->dslot ? c->derivs : c->derivs + s * (size_t)sei::derivativesSize(c->cfg.order)) : nullptr;
  d.dslot = c->dslot ? c->dslot + s : nullptr;
  d.star_nz = c->star_nz + s * 3 * sei::kStarNnz;
  d.aplus = c->aplus + s * 4 * 81;
  d.aminus = c->aminus + s * 4 * 81;
  d.nbr = c->nbr + s * 4;
  d.rel = c->rel + s * 4;
  d.ftype = c->ftype + s * 4;
  return d;
}

// sei_run_host of kernel 'all' on global steps, pipelined in chunks of cells: the host -> device
// copy of chunk k runs on the copy stream while ADER and the local integral work on the chunks
// that have arrived; the last step's neighbour flux runs chunk by chunk and each finished chunk
// is copied back while the next one is computed.  (Two copy streams with alternating chunks
// measured slower on GB300: 41 vs 46 M cell-updates/s.)
static int runHostPipelined(sei_ctx* c, double dt, int nsteps, const float* in, float* out) {
  constexpr int kChunks = 8;
  const int64_t n = c->n;
  const int nch = (int)(n < kChunks ? n : kChunks);
  if (!c->copy_stream && cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(c, SEI_ERR_CUDA, "copy stream creation failed");
  while (c->pipe_events.size() < (size_t)(2 * kChunks + 2)) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(c, SEI_ERR_CUDA, "event creation");
    c->pipe_events.push_back(e);
  }
  cudaEvent_t* ev = c->pipe_events.data();
  const size_t blk = (size_t)9 * c->Bp;
  std::vector<int64_t> b(nch + 1);
  for (int k = 0; k <= nch; ++k) b[k] = n * k / nch;
  float co[8];
  taylorCoeffs(c->cfg.order, dt, co);
  c->prof_used = 0;
  // the copy stream starts after everything queued on the compute stream (Q may be in use)
  SEI_CUDA(cudaEventRecord(ev[2 * kChunks], c->stream));
  SEI_CUDA(cudaStreamWaitEvent(c->copy_stream, ev[2 * kChunks], 0));
  int rc = SEI_OK;
  for (int k = 0; k < nch && !rc; ++k) {
    SEI_CUDA(cudaMemcpyAsync(c->Q + b[k] * blk, in + b[k] * blk, (b[k + 1] - b[k]) * blk * sizeof(float),
                             cudaMemcpyHostToDevice, c->copy_stream));
    SEI_CUDA(cudaEventRecord(ev[k], c->copy_stream));
    SEI_CUDA(cudaStreamWaitEvent(c->stream, ev[k], 0));
    const sei::DeviceArrays d = gtsRange(c, b[k], b[k + 1], false);
    rc = launchLocal(c, d, co, fusedFlux(c));
  }
  if (rc) return rc;
  c->trace_valid = c->cfg.precision == SEI_PREC_F16X3 && c->d_trace;
  if (nsteps > 1) {
    const sei::DeviceArrays all = arrays(c);
    if ((rc = launchNeighbor(c, all, fusedFlux(c))) || (rc = launchPlast(c, 0, c->n, dt))) return rc;
    if (nsteps > 2 && (rc = runKernel(c, SEI_KERNEL_ALL, dt, nsteps - 2))) return rc;
    if ((rc = launchLocal(c, all, co, fusedFlux(c)))) return rc;
  }
  for (int k = 0; k < nch && !rc; ++k) {
    rc = launchNeighbor(c, gtsRange(c, b[k], b[k + 1], true), fusedFlux(c));
    if (!rc) rc = launchPlast(c, b[k], b[k + 1], dt);
    if (rc) return rc;
    SEI_CUDA(cudaEventRecord(ev[kChunks + k], c->stream));
    SEI_CUDA(cudaStreamWaitEvent(c->copy_stream, ev[kChunks + k], 0));
    SEI_CUDA(cudaMemcpyAsync(out + b[k] * blk, c->Q + b[k] * blk, (b[k + 1] - b[k]) * blk * sizeof(float),
                             cudaMemcpyDeviceToHost, c->copy_stream));
  }
  // later work on the compute stream waits for the last copy
  SEI_CUDA(cudaEventRecord(ev[2 * kChunks + 1], c->copy_stream));
  SEI_CUDA(cudaStreamWaitEvent(c->stream, ev[2 * kChunks + 1], 0));
  return profMark(c, -1);
}

int sei_run_host(sei_ctx* c, int kernel, double dt, int nsteps, const float* dofs_in, float* dofs_out) {
  NvtxRange range("sei_run_host");
  int rc = checkReady(c);
  if (rc) return rc;
  if (!dofs_in || !dofs_out) return fail(c, SEI_ERR_ARG, "null host buffer");
  if (kernel == SEI_KERNEL_ALL && nsteps >= 1 && !c->lts && !c->visco && c->B == c->Bp && c->nrecv == 0 &&
      !(c->fused_local && c->cfg.precision == SEI_PREC_FP32)) {
    rc = runHostPipelined(c, dt, nsteps, dofs_in, dofs_out);
    if (rc) return rc;
    SEI_CUDA(cudaStreamSynchronize(c->stream));
    return SEI_OK;
  }
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
  if (c->cfg.device < 0) return SEI_OK;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  int st = 0;
  SEI_CUDA(cudaMemcpy(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st) {
    cudaMemset(c->d_status, 0, sizeof(int));
    return fail(c, SEI_ERR_TIMEOUT, "a bounded wait inside a tensor-core kernel gave up");
  }
  return SEI_OK;
}

int sei_device_clock_khz(int device, int* khz) {
  if (!khz || device < 0) return SEI_ERR_ARG;
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrClockRate, device) != cudaSuccess) {
    cudaGetLastError();
    return SEI_ERR_CUDA;
  }
  *khz = v;
  return SEI_OK;
}

int sei_check_wait_timeout(sei_ctx* c, int polls, int arrive) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (polls < 1 || polls > (1 << 20) || (arrive != 0 && arrive != 1))
    return fail(c, SEI_ERR_ARG, "1 <= polls <= 2^20, arrive 0 or 1");
  if (sei::launchWaitProbe((uint32_t)polls, arrive, c->d_status, c->stream) != 0)
    return fail(c, SEI_ERR_CUDA, "wait probe launch failed");
  return SEI_OK;
}

int sei_last_run_ms(sei_ctx* c, double* ms) {
  if (!c || !ms) return SEI_ERR_ARG;
  float f = 0;
  SEI_CUDA(cudaEventElapsedTime(&f, c->ev0, c->ev1));
  *ms = f;
  return SEI_OK;
}

int sei_receivers_setup(sei_ctx* c, int64_t n, const double* xyz, double interval, unsigned qmask, int derived,
                        int64_t* cells) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->has_mesh) return fail(c, SEI_ERR_STATE, "receivers need a mesh built by the context");
  if (n < 0 || (n > 0 && !xyz) || !(interval > 0) || !std::isfinite(interval) || qmask > 0x1FFu ||
      (derived & ~(SEI_RECV_ROTATION | SEI_RECV_STRAIN)))
    return fail(c, SEI_ERR_ARG, "receivers: n >= 0, points, interval > 0, quantity mask of 9 bits, derived flags");
  std::vector<int64_t> cell;
  std::vector<double> xez;
  sei::locatePoints(c->mesh, n, xyz, cell, xez);
  for (int64_t r = 0; r < n; ++r)
    if (cell[r] < 0) return fail(c, SEI_ERR_ARG, "receiver " + std::to_string(r) + " lies outside the mesh");
  // a rejected call changes nothing: the old receivers go only now
  std::vector<double> points(xyz, xyz + 3 * n);
  for (void* p : {(void*)c->d_recv_ucell, (void*)c->d_recv_slot, (void*)c->d_recv_q, (void*)c->d_recv_i,
                  (void*)c->d_recv_star, (void*)c->d_recv_derivs, (void*)c->d_recv_phi, (void*)c->d_recv_dphi,
                  (void*)c->d_recv_list})
    cudaFree(p);
  c->d_recv_ucell = c->d_recv_slot = c->d_recv_list = nullptr;
  c->d_recv_q = c->d_recv_i = c->d_recv_star = c->d_recv_derivs = c->d_recv_phi = c->d_recv_dphi = nullptr;
  c->recv_stage.release();
  c->nrecv = c->nrecv_cells = 0;
  c->recv_cell.clear();
  c->recv_xyz.clear();
  c->recv_log.clear();
  c->recv_pending.clear();
  if (n == 0) return SEI_OK;
  const int order = c->cfg.order, B = sei::numBasis(order);
  std::vector<int32_t> ucell, slot(n);
  std::vector<int64_t> index(c->n, -1);
  std::vector<float> phi((size_t)n * B), dphi((size_t)n * 3 * B);
  std::vector<double> p(B), dp(3 * B);
  for (int64_t r = 0; r < n; ++r) {
    const int64_t cl = cell[r];
    if (index[cl] < 0) {
      index[cl] = (int64_t)ucell.size();
      ucell.push_back((int32_t)cl);
    }
    slot[r] = (int32_t)index[cl];
    // d xi_r / d x: rows of the inverse of [v1 - v0, v2 - v0, v3 - v0]
    const double* v = &c->mesh.coords[cl * 12];
    double e[3][3];
    for (int k = 0; k < 3; ++k)
      for (int x = 0; x < 3; ++x) e[k][x] = v[(k + 1) * 3 + x] - v[x];
    auto cross = [](const double* a, const double* b, double* o) {
      o[0] = a[1] * b[2] - a[2] * b[1];
      o[1] = a[2] * b[0] - a[0] * b[2];
      o[2] = a[0] * b[1] - a[1] * b[0];
    };
    double g[3][3];
    cross(e[1], e[2], g[0]);
    cross(e[2], e[0], g[1]);
    cross(e[0], e[1], g[2]);
    const double det = e[0][0] * g[0][0] + e[0][1] * g[0][1] + e[0][2] * g[0][2];
    for (int k = 0; k < 3; ++k)
      for (int x = 0; x < 3; ++x) g[k][x] /= det;
    sei::basisAtPoint(order, &xez[r * 3], g, p.data(), dp.data());
    for (int l = 0; l < B; ++l) phi[(size_t)r * B + l] = (float)p[l];
    for (int k = 0; k < 3 * B; ++k) dphi[(size_t)r * 3 * B + k] = (float)dp[k];
  }
  const int64_t m = (int64_t)ucell.size();
  // groups: every receiver in order, then the receivers of each LTS cluster
  const int ncl = c->lts ? c->ncl : 0;
  std::vector<int32_t> list(2 * n);
  std::vector<int64_t> gstart(ncl + 1, 0);
  std::vector<int> grp(n, 0);
  for (int64_t r = 0; r < n; ++r) {
    list[r] = (int32_t)r;
    if (ncl) {
      int g = 0;
      while (g + 1 < ncl && cell[r] >= c->cl_start[g + 1]) ++g;
      grp[r] = g;
      ++gstart[g + 1];
    }
  }
  for (int g = 0; g < ncl; ++g) gstart[g + 1] += gstart[g];
  {
    std::vector<int64_t> fillp(gstart.begin(), gstart.end());
    for (int64_t r = 0; r < n; ++r) list[n + (ncl ? fillp[grp[r]]++ : r)] = (int32_t)r;
  }
  const size_t blk = (size_t)c->nq * c->Bp;
  const size_t dsz = c->visco ? (size_t)c->vk.derivSize : (size_t)sei::derivativesSize(order);
  auto dalloc = [&](void** ptr, size_t bytes) { return cudaMalloc(ptr, bytes) == cudaSuccess; };
  bool ok = dalloc((void**)&c->d_recv_ucell, m * 4) && dalloc((void**)&c->d_recv_slot, n * 4) &&
            dalloc((void**)&c->d_recv_q, m * blk * 4) && dalloc((void**)&c->d_recv_i, m * blk * 4) &&
            dalloc((void**)&c->d_recv_star, m * 3 * sei::kStarNnz * 4) && dalloc((void**)&c->d_recv_derivs, m * dsz * 4) &&
            dalloc((void**)&c->d_recv_phi, phi.size() * 4) && dalloc((void**)&c->d_recv_dphi, dphi.size() * 4) &&
            dalloc((void**)&c->d_recv_list, list.size() * 4) &&
            (!c->visco || (dalloc((void**)&c->d_recv_grad, m * 9 * 4) && dalloc((void**)&c->d_recv_theta, m * 9 * 4)));
  if (!ok) {
    cudaGetLastError();
    return fail(c, SEI_ERR_OOM, "device allocation for the receivers failed");
  }
  SEI_CUDA(cudaMemcpy(c->d_recv_ucell, ucell.data(), m * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_recv_slot, slot.data(), n * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_recv_phi, phi.data(), phi.size() * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_recv_dphi, dphi.data(), dphi.size() * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_recv_list, list.data(), list.size() * 4, cudaMemcpyHostToDevice));
  if (sei::launchGatherRows((int)m, c->d_recv_ucell, c->star_nz, c->d_recv_star, 3 * sei::kStarNnz, c->stream) ||
      (c->visco && (sei::launchGatherRows((int)m, c->d_recv_ucell, c->d_grad, c->d_recv_grad, 9, c->stream) ||
                    sei::launchGatherRows((int)m, c->d_recv_ucell, c->d_theta, c->d_recv_theta, 9, c->stream))))
    return fail(c, SEI_ERR_CUDA, "receiver gather launch failed");
  c->recv_qmask = qmask;
  c->recv_derived = derived;
  c->recv_ncols = 1 + __builtin_popcount(qmask) + ((derived & SEI_RECV_ROTATION) ? 3 : 0) +
                  ((derived & SEI_RECV_STRAIN) ? 6 : 0);
  const size_t rowBytes = (size_t)c->recv_ncols * sizeof(double);
  const size_t rows = std::max<size_t>((size_t)n * sei::kRecvMaxSamples,
                                       std::min<size_t>((size_t)n * 1024, ((size_t)64 << 20) / rowBytes));
  if (c->recv_stage.init(rowBytes, rows) != 0) return fail(c, SEI_ERR_OOM, "receiver staging allocation failed");
  c->nrecv = n;
  c->nrecv_cells = m;
  c->recv_cell = cell;
  c->recv_interval = interval;
  c->recv_xyz = std::move(points);
  c->h_recv_list = std::move(list);
  c->recv_gstart = std::move(gstart);
  c->recv_next.assign(ncl + 1, 0);
  c->recv_times.assign(1, c->sim_time);
  c->recv_emit = 0;
  if (cells) std::copy(cell.begin(), cell.end(), cells);
  return SEI_OK;
}

double sei_plasticity_relax_factor(double tv, double dt) { return tv > 0.0 ? -std::expm1(-dt / tv) : 1.0; }

int sei_plasticity_nodes(int order, double* nodes) {
  if (order < 2 || order > 8 || !nodes) return SEI_ERR_ARG;
  sei::latticeNodes(order, nodes);
  return SEI_OK;
}

namespace {
int uploadF(sei_ctx* c, float** dst, const std::vector<float>& src) {
  cudaFree(*dst);
  *dst = nullptr;
  if (src.empty()) return SEI_OK;
  if (cudaMalloc(dst, src.size() * sizeof(float)) != cudaSuccess) return fail(c, SEI_ERR_OOM, "plasticity allocation");
  SEI_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(float), cudaMemcpyHostToDevice));
  return SEI_OK;
}

// Per-node arrays [n][K][B] <-> the device's tiled layout [n / 32][K][B][32] (cell c in tile
// c / 32, lane c % 32), in which a warp's 32 cells read one node's values as one 128-byte run.
std::vector<float> plastTile(const std::vector<float>& a, int64_t n, int K, int B) {
  const int64_t tiles = (n + 31) / 32;
  std::vector<float> t((size_t)tiles * K * B * 32, 0.f);
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < K * B; ++k) t[((size_t)(i >> 5) * K * B + k) * 32 + (i & 31)] = a[(size_t)i * K * B + k];
  return t;
}
std::vector<float> plastUntile(const std::vector<float>& t, int64_t n, int K, int B) {
  std::vector<float> a((size_t)n * K * B);
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < K * B; ++k) a[(size_t)i * K * B + k] = t[((size_t)(i >> 5) * K * B + k) * 32 + (i & 31)];
  return a;
}

// Device copies of the plasticity parameters in the current cell order (tiled), 1 / (2 mu) from
// the mesh's materials, and a zero plastic strain when reset.
int plastUpload(sei_ctx* c, bool resetStrain) {
  const int64_t n = c->n;
  const int B = sei::numBasis(c->cfg.order);
  std::vector<float> mu((size_t)n);
  for (int64_t i = 0; i < n; ++i) mu[i] = (float)(1.0 / (2.0 * c->mesh.material[(size_t)i * 3 + 1]));
  int rc;
  if ((rc = uploadF(c, &c->d_pls0, plastTile(c->pl_s0, n, 6, B))) ||
      (rc = uploadF(c, &c->d_plccos, plastTile(c->pl_ccos, n, 1, B))) ||
      (rc = uploadF(c, &c->d_plssin, plastTile(c->pl_ssin, n, 1, B))) || (rc = uploadF(c, &c->d_plmu, mu)))
    return rc;
  if (resetStrain) {
    const size_t bytes = (size_t)((n + 31) / 32) * 32 * 7 * B * sizeof(float);
    cudaFree(c->d_pstrain);
    c->d_pstrain = nullptr;
    if (cudaMalloc(&c->d_pstrain, bytes) != cudaSuccess) return fail(c, SEI_ERR_OOM, "plastic strain allocation failed");
    SEI_CUDA(cudaMemset(c->d_pstrain, 0, bytes));
  }
  return SEI_OK;
}

// After sei_lts_setup reordered the cells (new cell i = old cell order[i]).
int plastPermute(sei_ctx* c, const std::vector<int64_t>& order) {
  const int64_t n = c->n;
  const int B = sei::numBasis(c->cfg.order);
  auto perm = [&](std::vector<float>& a, size_t per) {
    std::vector<float> b(a.size());
    for (int64_t i = 0; i < n; ++i)
      std::copy(a.begin() + order[i] * per, a.begin() + (order[i] + 1) * per, b.begin() + i * per);
    a.swap(b);
  };
  perm(c->pl_s0, (size_t)6 * B);
  perm(c->pl_ccos, B);
  perm(c->pl_ssin, B);
  std::vector<float> pt((size_t)((n + 31) / 32) * 32 * 7 * B);
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  SEI_CUDA(cudaMemcpy(pt.data(), c->d_pstrain, pt.size() * sizeof(float), cudaMemcpyDeviceToHost));
  std::vector<float> ps = plastUntile(pt, n, 7, B);
  perm(ps, (size_t)7 * B);
  pt = plastTile(ps, n, 7, B);
  SEI_CUDA(cudaMemcpy(c->d_pstrain, pt.data(), pt.size() * sizeof(float), cudaMemcpyHostToDevice));
  return plastUpload(c, false);
}
}  // namespace

int sei_plasticity_setup(sei_ctx* c, const double* nodes, double tv, const double* bulk_friction,
                         const double* plast_co, const double* s0, int per_node) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (c->visco) return fail(c, SEI_ERR_UNSUPPORTED, "plasticity with the viscoelastic equations is not supported");
  const int order = c->cfg.order;
  if (order < 4 || order > 6) return fail(c, SEI_ERR_UNSUPPORTED, "plasticity kernels exist for orders 4-6");
  if (!bulk_friction || !plast_co || !s0) return fail(c, SEI_ERR_ARG, "null plasticity parameters");
  if (!(tv > 0.0) || !std::isfinite(tv))
    return fail(c, SEI_ERR_ARG, "relaxation time T_v must be positive (the plastic strain rate divides by it)");
  if (per_node != 0 && per_node != 1) return fail(c, SEI_ERR_ARG, "per_node must be 0 or 1");
  const int B = sei::numBasis(order), Bp = c->Bp;
  std::vector<double> nd((size_t)3 * B);
  if (nodes)
    std::copy(nodes, nodes + 3 * B, nd.begin());
  else
    sei::latticeNodes(order, nd.data());
  for (double x : nd)
    if (!std::isfinite(x)) return fail(c, SEI_ERR_ARG, "non-finite plasticity node");
  std::vector<double> v, vi;
  if (!sei::plasticityMatrices(order, nd.data(), v, vi))
    return fail(c, SEI_ERR_ARG, "the plasticity nodes are not unisolvent for the basis");
  const int64_t n = c->n;
  std::vector<float> ps0((size_t)n * 6 * B), pcos((size_t)n * B), psin((size_t)n * B);
  for (int64_t i = 0; i < n; ++i)
    for (int j = 0; j < B; ++j) {
      const size_t p = per_node ? (size_t)i * B + j : (size_t)i;
      const double phi = std::atan(bulk_friction[p]), co = plast_co[p];
      if (!std::isfinite(phi) || !std::isfinite(co)) return fail(c, SEI_ERR_ARG, "non-finite plasticity parameter");
      pcos[(size_t)i * B + j] = (float)(co * std::cos(phi));
      psin[(size_t)i * B + j] = (float)std::sin(phi);
      for (int x = 0; x < 6; ++x) {
        const double sv = s0[p * 6 + x];
        if (!std::isfinite(sv)) return fail(c, SEI_ERR_ARG, "non-finite initial stress");
        ps0[((size_t)i * 6 + x) * B + j] = (float)sv;
      }
    }
  std::vector<float> mats((size_t)2 * B * Bp, 0.f);
  for (int a = 0; a < B; ++a)
    for (int b = 0; b < B; ++b) {
      mats[(size_t)a * Bp + b] = (float)v[(size_t)a * B + b];            // V[node][basis]
      mats[(size_t)(B + a) * Bp + b] = (float)vi[(size_t)a * B + b];     // Vinv[basis][node]
    }
  freePlasticity(c);
  c->pl_s0.swap(ps0);
  c->pl_ccos.swap(pcos);
  c->pl_ssin.swap(psin);
  c->plast_tv = tv;
  if ((rc = uploadF(c, &c->d_plmats, mats)) || (rc = plastUpload(c, true))) {
    freePlasticity(c);
    return rc;
  }
  if (cudaMalloc(&c->d_plyield, sizeof(unsigned long long)) != cudaSuccess) {
    freePlasticity(c);
    return fail(c, SEI_ERR_OOM, "plasticity counter allocation failed");
  }
  SEI_CUDA(cudaMemset(c->d_plyield, 0, sizeof(unsigned long long)));
  c->plast = true;
  return SEI_OK;
}

int sei_plasticity_disable(sei_ctx* c) {
  if (!c) return SEI_ERR_ARG;
  if (c->n > 0) cudaStreamSynchronize(c->stream);
  freePlasticity(c);
  return SEI_OK;
}

int sei_plasticity_get_strain(sei_ctx* c, float* out) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!out) return fail(c, SEI_ERR_ARG, "null output");
  if (!c->plast) return fail(c, SEI_ERR_STATE, "plasticity not set up (sei_plasticity_setup)");
  const int B = sei::numBasis(c->cfg.order);
  std::vector<float> pt((size_t)((c->n + 31) / 32) * 32 * 7 * B);
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  SEI_CUDA(cudaMemcpy(pt.data(), c->d_pstrain, pt.size() * sizeof(float), cudaMemcpyDeviceToHost));
  const std::vector<float> ps = plastUntile(pt, c->n, 7, B);
  std::copy(ps.begin(), ps.end(), out);
  return SEI_OK;
}

int sei_plasticity_yield_count(sei_ctx* c, int64_t* count) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!count) return fail(c, SEI_ERR_ARG, "null output");
  if (!c->plast) return fail(c, SEI_ERR_STATE, "plasticity not set up (sei_plasticity_setup)");
  unsigned long long v = 0;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  SEI_CUDA(cudaMemcpy(&v, c->d_plyield, sizeof(v), cudaMemcpyDeviceToHost));
  *count = (int64_t)v;
  return SEI_OK;
}

int sei_basis_functions(int order, const double* xez, double* phi, double* dphi) {
  if (order < 1 || order > 8 || !xez || !phi) return SEI_ERR_ARG;
  const double identity[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  std::vector<double> d((size_t)3 * sei::numBasis(order));
  sei::basisAtPoint(order, xez, identity, phi, d.data());
  if (dphi) std::copy(d.begin(), d.end(), dphi);
  return SEI_OK;
}

int sei_receivers_columns(const sei_ctx* c) { return (c && c->nrecv > 0) ? c->recv_ncols : 0; }

int sei_receivers_read(sei_ctx* c, double* out, int64_t max_samples, int64_t* nsamples) {
  if (!c || !nsamples || max_samples < 0) return SEI_ERR_ARG;
  *nsamples = 0;
  if (c->nrecv == 0) return SEI_OK;
  // every staged row, then each logged launch's rows into their samples
  const size_t nc = (size_t)c->recv_ncols;
  size_t total = 0;
  for (const auto& L : c->recv_log) total += (size_t)L.m * L.count;
  std::vector<double> rows(total * nc);
  size_t got = 0;
  if (c->recv_stage.drain(c->stream, rows.data(), total, &got) != 0 || got != total)
    return fail(c, SEI_ERR_CUDA, "receiver staging copy failed");
  size_t pos = 0;
  for (const auto& L : c->recv_log)
    for (int sm = 0; sm < L.m; ++sm) {
      auto& P = c->recv_pending[L.k0 + sm];
      if (P.first.empty()) P.first.assign((size_t)c->nrecv * nc, 0.0);
      for (int64_t j = 0; j < L.count; ++j, ++pos) {
        const int32_t r = c->h_recv_list[L.first + j];
        std::copy_n(&rows[pos * nc], nc, &P.first[(size_t)r * nc]);
      }
      P.second += L.count;
    }
  c->recv_log.clear();
  // complete samples, in order
  int64_t done = 0;
  while (done < max_samples) {
    auto it = c->recv_pending.find(c->recv_emit);
    if (it == c->recv_pending.end() || it->second.second < c->nrecv) break;
    if (out) std::copy(it->second.first.begin(), it->second.first.end(), out + (size_t)done * c->nrecv * nc);
    c->recv_pending.erase(it);
    ++c->recv_emit;
    ++done;
  }
  *nsamples = done;
  return SEI_OK;
}

int sei_get_time(const sei_ctx* c, double* t) {
  if (!c || !t) return SEI_ERR_ARG;
  *t = c->sim_time;
  return SEI_OK;
}

int sei_set_time(sei_ctx* c, double t) {
  if (!c || !std::isfinite(t) || t < 0) return c ? fail(c, SEI_ERR_ARG, "time must be finite and >= 0") : SEI_ERR_ARG;
  c->sim_time = t;
  if (c->nrecv > 0) {
    // the receivers sample from t on: set them up again (samples not yet read are dropped)
    const std::vector<double> pts = c->recv_xyz;
    return sei_receivers_setup(c, (int64_t)pts.size() / 3, pts.data(), c->recv_interval, c->recv_qmask,
                               c->recv_derived, nullptr);
  }
  return SEI_OK;
}

int sei_fault_output_setup(sei_ctx* c, int every, const int* fields, int nfields) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  if (every < 0 || nfields < 0 || (every > 0 && (nfields == 0 || !fields)))
    return fail(c, SEI_ERR_ARG, "fault output: every >= 0 and at least one field");
  for (int i = 0; i < nfields && every > 0; ++i)
    if (fields[i] < 0 || fields[i] >= SEI_DR_NUM_FIELDS) return fail(c, SEI_ERR_ARG, "unknown friction-state field");
  c->fault_stage.release();
  c->fault_every = 0;
  c->fault_fields.clear();
  if (every == 0) return SEI_OK;
  const size_t rowBytes = (1 + (size_t)nfields * c->fault.nf * c->npts) * sizeof(double);
  const size_t rows = std::max<size_t>(1, std::min<size_t>(64, ((size_t)256 << 20) / rowBytes));
  if (c->fault_stage.init(rowBytes, rows) != 0) return fail(c, SEI_ERR_OOM, "fault output staging allocation failed");
  c->fault_fields.assign(fields, fields + nfields);
  c->fault_every = every;
  c->fault_steps = 0;
  dropLtsGraph(c);
  return SEI_OK;
}

int sei_fault_output_read(sei_ctx* c, double* out, int64_t max_snapshots, int64_t* nsnapshots) {
  if (!c || !nsnapshots || max_snapshots < 0) return SEI_ERR_ARG;
  *nsnapshots = 0;
  if (c->fault_every == 0) return SEI_OK;
  size_t rows = 0;
  if (c->fault_stage.drain(c->stream, out, (size_t)max_snapshots, &rows) != 0)
    return fail(c, SEI_ERR_CUDA, "fault output staging copy failed");
  *nsnapshots = (int64_t)rows;
  return SEI_OK;
}

int sei_dr_num_points(int order) { return (order >= 2 && order <= 6) ? sei::drNumPoints(order) : 0; }

int64_t sei_dr_num_faces(const sei_ctx* c) { return (c && c->has_fault) ? c->fault.nf : 0; }

namespace {
// Seeded uniform numbers for the initial fault state (splitmix64).
struct FaultRng {
  uint64_t z;
  double operator()(double lo, double hi) {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return lo + (hi - lo) * ((x >> 11) * (1.0 / 9007199254740992.0));
  }
};

// Fault arrays on the device from the host initial state st [SEI_DR_NUM_FIELDS][nf][npts]
// (replaces any earlier fault set-up of the context).
int drInstall(sei_ctx* c, const std::vector<double>& st) {
  const int64_t nf = c->fault.nf;
  const int np = c->npts;
  freeFault(c);
  // derivative slots: one per fault cell, in order of first appearance (plus, then minus side of
  // each face: slots 2f and 2f + 1 when no cell has two fault faces)
  std::vector<int32_t> slot(c->n, -1), ps(nf), ms(nf);
  int32_t nslots = 0;
  for (int64_t f = 0; f < nf; ++f) {
    for (int sd = 0; sd < 2; ++sd) {
      const int32_t cell = sd ? c->fault.minus_cell[f] : c->fault.plus_cell[f];
      if (slot[cell] < 0) slot[cell] = nslots++;
      (sd ? ms : ps)[f] = slot[cell];
    }
  }
  auto dalloc = [&](void** ptr, size_t bytes) { return cudaMalloc(ptr, bytes) == cudaSuccess; };
  const size_t dsz = (size_t)sei::derivativesSize(c->cfg.order) * sizeof(float);
  cudaFree(c->derivs);
  c->derivs = nullptr;
  cudaFree(c->dslot);
  c->dslot = nullptr;
  bool ok = dalloc((void**)&c->derivs, nslots * dsz) && dalloc((void**)&c->dslot, c->n * 4) &&
            dalloc((void**)&c->d_pc, nf * 4) && dalloc((void**)&c->d_mc, nf * 4) && dalloc((void**)&c->d_pslot, nf * 4) &&
            dalloc((void**)&c->d_mslot, nf * 4) && dalloc((void**)&c->d_iters, 3 * nf * np * 4) &&
            dalloc((void**)&c->d_ps, nf) && dalloc((void**)&c->d_ms, nf) && dalloc((void**)&c->d_rel, nf) &&
            dalloc((void**)&c->d_tinvt, nf * 81 * 4) && dalloc((void**)&c->d_fsp, nf * 81 * 4) &&
            dalloc((void**)&c->d_fsm, nf * 81 * 4) && dalloc((void**)&c->d_isp, nf * 9 * np * 4) &&
            dalloc((void**)&c->d_ism, nf * 9 * np * 4) && dalloc((void**)&c->d_imp, nf * 8 * 8) &&
            dalloc((void**)&c->d_state, st.size() * 8) && dalloc((void**)&c->d_time, sizeof(double));
  if (!ok) {
    cudaGetLastError();
    return fail(c, SEI_ERR_OOM, "device allocation for the fault failed");
  }
  const sei::HostFault& F = c->fault;
  SEI_CUDA(cudaMemcpy(c->dslot, slot.data(), c->n * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_pc, F.plus_cell.data(), nf * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_mc, F.minus_cell.data(), nf * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_pslot, ps.data(), nf * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_mslot, ms.data(), nf * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_ps, F.plus_side.data(), nf, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_ms, F.minus_side.data(), nf, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_rel, F.rel.data(), nf, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_tinvt, F.tinvt.data(), nf * 81 * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_fsp, F.fsp.data(), nf * 81 * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_fsm, F.fsm.data(), nf * 81 * 4, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_imp, F.imp.data(), nf * 8 * 8, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemcpy(c->d_state, st.data(), st.size() * 8, cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemset(c->d_iters, 0, 3 * nf * np * 4));
  SEI_CUDA(cudaMemset(c->d_isp, 0, nf * 9 * np * 4));
  SEI_CUDA(cudaMemset(c->d_ism, 0, nf * 9 * np * 4));
  SEI_CUDA(cudaMemset(c->derivs, 0, nslots * dsz));
  SEI_CUDA(cudaMemset(c->d_time, 0, sizeof(double)));
  c->dr_ready = true;
  c->nslots = nslots;
  return SEI_OK;
}

// Host initial state with the fields both laws share: rupture and dynamic-stress times pending
// (negative), no forced rupture, zero nucleation stresses and peak slip rate.
std::vector<double> drInitialState(int64_t nf, int np) {
  std::vector<double> st((size_t)SEI_DR_NUM_FIELDS * nf * np, 0.0);
  const size_t pl = (size_t)nf * np;
  std::fill_n(st.data() + SEI_DR_RUPTURE_TIME * pl, pl, -1.0);
  std::fill_n(st.data() + SEI_DR_DYN_STRESS_TIME * pl, pl, -1.0);
  std::fill_n(st.data() + SEI_DR_FORCED_RUPTURE_TIME * pl, pl, std::numeric_limits<double>::max());
  return st;
}

int drSetupCheck(sei_ctx* c, const void* p) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!p) return fail(c, SEI_ERR_ARG, "null parameters");
  if (!c->has_fault) return fail(c, SEI_ERR_STATE, "mesh has no fault (fault_plane < 0)");
  if (c->lts) return fail(c, SEI_ERR_STATE, "set up dynamic rupture before local time stepping");
  return SEI_OK;
}
}  // namespace

int sei_dr_setup(sei_ctx* c, const sei_rs_params* p, int64_t* nfaces) {
  return sei_dr_setup_rate_state(c, p, SEI_LAW_FVW, nfaces);
}

int sei_dr_setup_rate_state(sei_ctx* c, const sei_rs_params* p, int law, int64_t* nfaces) {
  int rc = drSetupCheck(c, p);
  if (rc) return rc;
  if (law != SEI_LAW_FVW && law != SEI_LAW_RS_AGING && law != SEI_LAW_RS_SLIP && law != SEI_LAW_RS_SEVERE)
    return fail(c, SEI_ERR_ARG, "law must be a rate-and-state law (SEI_LAW_FVW, _RS_AGING, _RS_SLIP, _RS_SEVERE)");
  if (!(p->a_min > 0) || p->a_max < p->a_min || !(p->v0 > 0) || !(p->l > 0) || !(p->vw > 0) || !(p->v_init > 0) ||
      p->max_newton <= 0 || p->max_outer <= 0 || !(p->newton_tol > 0) || !(p->state_tol > 0) || p->sn_max > 0)
    return fail(c, SEI_ERR_ARG, "invalid rate-and-state parameters");
  c->rs = *p;
  const int64_t nf = c->fault.nf;
  const int np = sei::drNumPoints(c->cfg.order);
  c->npts = np;
  std::vector<double> st = drInitialState(nf, np);
  auto field = [&](int k) { return st.data() + (size_t)k * nf * np; };
  FaultRng uni{p->seed};
  for (int64_t i = 0; i < nf * np; ++i) {
    const double a = uni(p->a_min, p->a_max);
    field(SEI_DR_A)[i] = a;
    field(SEI_DR_SN0)[i] = uni(p->sn_min, p->sn_max);
    field(SEI_DR_TAU1_0)[i] = uni(p->tau_min, p->tau_max);
    field(SEI_DR_TAU2_0)[i] = 0.0;
    field(SEI_DR_SLIP_RATE1)[i] = p->v_init;
    // the state at steady sliding at v_init: psi of the fast law, theta = L / V (aging, slip),
    // theta = V L / V0 (severe velocity weakening)
    field(SEI_DR_PSI)[i] = law == SEI_LAW_FVW      ? sei::fvwSteadyState(p->v_init, a, p->b, p->f0, p->v0, p->muw, p->vw)
                           : law == SEI_LAW_RS_SEVERE ? p->v_init * p->l / p->v0
                                                      : p->l / p->v_init;
  }
  if ((rc = drInstall(c, st))) return rc;
  c->dr_law = law;
  if (nfaces) *nfaces = nf;
  return SEI_OK;
}

int sei_dr_setup_lsw(sei_ctx* c, const sei_lsw_params* p, int64_t* nfaces) {
  int rc = drSetupCheck(c, p);
  if (rc) return rc;
  if (p->law != SEI_LAW_LSW && p->law != SEI_LAW_LSW_BIMATERIAL && p->law != SEI_LAW_LSW_TP_PROXY)
    return fail(c, SEI_ERR_ARG, "law must be SEI_LAW_LSW, SEI_LAW_LSW_BIMATERIAL or SEI_LAW_LSW_TP_PROXY");
  if (!(p->d_c > 0) || !std::isfinite(p->mu_s) || !std::isfinite(p->mu_d) || !std::isfinite(p->cohesion) ||
      !(p->t0 >= 0) || p->sn_max > 0 || p->sn_min > p->sn_max || p->tau_min > p->tau_max ||
      (p->law == SEI_LAW_LSW_BIMATERIAL && !(p->prakash_length > 0)) ||
      (p->law == SEI_LAW_LSW_TP_PROXY && !(p->tp_proxy_exponent > 0)))
    return fail(c, SEI_ERR_ARG, "invalid linear-slip-weakening parameters");
  c->rs = sei_rs_params{};
  c->lsw = *p;
  const int64_t nf = c->fault.nf;
  const int np = sei::drNumPoints(c->cfg.order);
  c->npts = np;
  std::vector<double> st = drInitialState(nf, np);
  auto field = [&](int k) { return st.data() + (size_t)k * nf * np; };
  FaultRng uni{p->seed};
  for (int64_t i = 0; i < nf * np; ++i) {
    const double sn = uni(p->sn_min, p->sn_max);
    field(SEI_DR_SN0)[i] = sn;
    field(SEI_DR_TAU1_0)[i] = uni(p->tau_min, p->tau_max);
    field(SEI_DR_MU_S)[i] = p->mu_s;
    field(SEI_DR_MU_D)[i] = p->mu_d;
    field(SEI_DR_D_C)[i] = p->d_c;
    field(SEI_DR_COHESION)[i] = p->cohesion;
    field(SEI_DR_FORCED_RUPTURE_TIME)[i] = p->forced_rupture_time;
    field(SEI_DR_MU)[i] = p->mu_s;  // LinearSlipWeakeningInitializer.cpp:43
    // LinearSlipWeakeningInitializer.cpp:82-85
    field(SEI_DR_REG_STRENGTH)[i] = -p->cohesion - p->mu_s * std::min(0.0, sn);
  }
  if ((rc = drInstall(c, st))) return rc;
  c->dr_law = p->law;
  c->dr_t0 = p->t0;
  if (nfaces) *nfaces = nf;
  return SEI_OK;
}

int sei_dr_setup_imposed(sei_ctx* c, const sei_isr_params* p, int64_t* nfaces) {
  int rc = drSetupCheck(c, p);
  if (rc) return rc;
  if (p->law != SEI_LAW_ISR_YOFFE && p->law != SEI_LAW_ISR_GAUSSIAN && p->law != SEI_LAW_ISR_DELTA)
    return fail(c, SEI_ERR_ARG, "law must be SEI_LAW_ISR_YOFFE, SEI_LAW_ISR_GAUSSIAN or SEI_LAW_ISR_DELTA");
  if (!std::isfinite(p->slip_dir1) || !std::isfinite(p->slip_dir2) || !std::isfinite(p->onset_time) ||
      !std::isfinite(p->sn0) || !std::isfinite(p->tau1_0) ||
      (p->law == SEI_LAW_ISR_YOFFE && !(p->tau_s > 0 && p->tau_r > 0)) || (p->law == SEI_LAW_ISR_GAUSSIAN && !(p->tau_s > 0)))
    return fail(c, SEI_ERR_ARG, "invalid imposed-slip-rate parameters");
  c->rs = sei_rs_params{};
  const int64_t nf = c->fault.nf;
  const int np = sei::drNumPoints(c->cfg.order);
  c->npts = np;
  std::vector<double> st = drInitialState(nf, np);
  auto fill = [&](int k, double v) { std::fill_n(st.data() + (size_t)k * nf * np, (size_t)nf * np, v); };
  fill(SEI_DR_SN0, p->sn0);
  fill(SEI_DR_TAU1_0, p->tau1_0);
  fill(SEI_DR_SLIP_DIR1, p->slip_dir1);
  fill(SEI_DR_SLIP_DIR2, p->slip_dir2);
  fill(SEI_DR_ONSET_TIME, p->onset_time);
  fill(SEI_DR_TAU_S, p->tau_s);
  fill(SEI_DR_TAU_R, p->tau_r);
  if ((rc = drInstall(c, st))) return rc;
  c->dr_law = p->law;
  if (nfaces) *nfaces = nf;
  return SEI_OK;
}

int sei_dr_set_thermal_pressurization(sei_ctx* c, int on, const sei_tp_params* p) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  if (c->dr_law != SEI_LAW_FVW && c->dr_law != SEI_LAW_RS_AGING && c->dr_law != SEI_LAW_RS_SLIP &&
      c->dr_law != SEI_LAW_RS_SEVERE)
    return fail(c, SEI_ERR_STATE, "thermal pressurisation needs a rate-and-state law");
  dropLtsGraph(c);
  cudaFree(c->d_tp);
  c->d_tp = nullptr;
  c->dr_tp = false;
  if (!on) return SEI_OK;
  if (!p || !(p->thermal_diffusivity > 0) || !(p->heat_capacity > 0) || !std::isfinite(p->undrained_tp_response) ||
      !std::isfinite(p->initial_temperature) || !std::isfinite(p->initial_pressure) || !(p->half_width_shear_zone > 0) ||
      !(p->hydraulic_diffusivity > 0) || p->hydraulic_diffusivity == p->thermal_diffusivity)
    return fail(c, SEI_ERR_ARG, "invalid thermal-pressurisation parameters");
  const size_t plane = (size_t)c->fault.nf * c->npts;
  if (cudaMalloc(&c->d_tp, 2 * sei::kTpModes * plane * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    c->d_tp = nullptr;
    return fail(c, SEI_ERR_OOM, "device allocation for thermal pressurisation failed");
  }
  SEI_CUDA(cudaMemsetAsync(c->d_tp, 0, 2 * sei::kTpModes * plane * sizeof(double), c->stream));
  std::vector<double> v(plane);
  const double init[4] = {p->half_width_shear_zone, p->hydraulic_diffusivity, p->initial_temperature, p->initial_pressure};
  for (int f = 0; f < 4; ++f) {
    std::fill(v.begin(), v.end(), init[f]);
    SEI_CUDA(cudaMemcpy(c->d_state + (size_t)(SEI_DR_TP_HALF_WIDTH + f) * plane, v.data(), plane * sizeof(double),
                        cudaMemcpyHostToDevice));
  }
  if (sei::launchTpTables(c->stream) != 0) return fail(c, SEI_ERR_CUDA, "thermal-pressurisation table launch failed");
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  c->tp = *p;
  c->dr_tp = true;
  return SEI_OK;
}

int sei_dr_law(const sei_ctx* c) { return (c && c->dr_ready) ? c->dr_law : -1; }

int sei_dr_set_nucleation(sei_ctx* c, int on, double t0, double s0) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  if (on && (!(t0 > 0) || !std::isfinite(s0))) return fail(c, SEI_ERR_ARG, "nucleation needs t0 > 0 and a finite s0");
  c->dr_nucleate = on != 0;
  if (on) {
    c->dr_t0 = t0;
    c->dr_s0 = s0;
  }
  dropLtsGraph(c);
  return SEI_OK;
}

int sei_dr_get_time(sei_ctx* c, double* t) {
  if (!c || !t) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  SEI_CUDA(cudaMemcpyAsync(t, c->d_time, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_dr_set_time(sei_ctx* c, double t) {
  if (!c) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  if (!std::isfinite(t) || t < 0) return fail(c, SEI_ERR_ARG, "fault time must be finite and >= 0");
  SEI_CUDA(cudaMemcpyAsync(c->d_time, &t, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_dr_get_faces(sei_ctx* c, int32_t* cells, int8_t* sides, float* tinvt, float* flux_plus, float* flux_minus,
                     double* impedance) {
  if (!c) return SEI_ERR_ARG;
  if (!c->has_fault) return fail(c, SEI_ERR_STATE, "mesh has no fault");
  const sei::HostFault& F = c->fault;
  for (int64_t f = 0; f < F.nf; ++f) {
    if (cells) {
      cells[2 * f] = F.plus_cell[f];
      cells[2 * f + 1] = F.minus_cell[f];
    }
    if (sides) {
      sides[3 * f] = (int8_t)F.plus_side[f];
      sides[3 * f + 1] = (int8_t)F.minus_side[f];
      sides[3 * f + 2] = (int8_t)F.rel[f];
    }
  }
  if (tinvt) std::memcpy(tinvt, F.tinvt.data(), F.tinvt.size() * 4);
  if (flux_plus) std::memcpy(flux_plus, F.fsp.data(), F.fsp.size() * 4);
  if (flux_minus) std::memcpy(flux_minus, F.fsm.data(), F.fsm.size() * 4);
  if (impedance) std::memcpy(impedance, F.imp.data(), F.imp.size() * 8);
  return SEI_OK;
}

static int drField(sei_ctx* c, int field, double*& dev) {
  if (!c) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  if (field < 0 || field >= SEI_DR_NUM_FIELDS) return fail(c, SEI_ERR_ARG, "unknown friction-state field");
  dev = c->d_state + (size_t)field * c->fault.nf * c->npts;
  return SEI_OK;
}

int sei_dr_get_state(sei_ctx* c, int field, double* out) {
  double* dev = nullptr;
  int rc = drField(c, field, dev);
  if (rc) return rc;
  if (!out) return fail(c, SEI_ERR_ARG, "null output");
  SEI_CUDA(cudaMemcpyAsync(out, dev, (size_t)c->fault.nf * c->npts * 8, cudaMemcpyDeviceToHost, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_dr_set_state(sei_ctx* c, int field, const double* in) {
  double* dev = nullptr;
  int rc = drField(c, field, dev);
  if (rc) return rc;
  if (!in) return fail(c, SEI_ERR_ARG, "null input");
  SEI_CUDA(cudaMemcpyAsync(dev, in, (size_t)c->fault.nf * c->npts * 8, cudaMemcpyHostToDevice, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_dr_get_imposed(sei_ctx* c, float* plus, float* minus) {
  if (!c) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  const size_t bytes = (size_t)c->fault.nf * 9 * c->npts * 4;
  if (plus) SEI_CUDA(cudaMemcpyAsync(plus, c->d_isp, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (minus) SEI_CUDA(cudaMemcpyAsync(minus, c->d_ism, bytes, cudaMemcpyDeviceToHost, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  return SEI_OK;
}

int sei_dr_newton_iterations(sei_ctx* c, int64_t* total, int64_t* points, int64_t* first) {
  if (!c || !total || !points) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  const size_t np = (size_t)c->fault.nf * c->npts;
  std::vector<int32_t> it(2 * np);
  SEI_CUDA(cudaMemcpyAsync(it.data(), c->d_iters, it.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  int64_t s = 0, f = 0;
  for (size_t i = 0; i < np; ++i) s += it[i], f += it[np + i];
  *total = s;
  *points = (int64_t)np;
  if (first) *first = f;
  return SEI_OK;
}

int sei_dr_newton_iterations32(sei_ctx* c, int64_t* total32) {
  if (!c || !total32) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  const size_t np = (size_t)c->fault.nf * c->npts;
  std::vector<int32_t> it(np);
  SEI_CUDA(cudaMemcpyAsync(it.data(), c->d_iters + 2 * np, np * 4, cudaMemcpyDeviceToHost, c->stream));
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  int64_t s = 0;
  for (size_t i = 0; i < np; ++i) s += it[i];
  *total32 = s;
  return SEI_OK;
}

int sei_dr_reset_counters(sei_ctx* c) {
  if (!c) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  SEI_CUDA(cudaMemsetAsync(c->d_iters, 0, 3 * (size_t)c->fault.nf * c->npts * 4, c->stream));
  return SEI_OK;
}

int sei_dr_faces_step(sei_ctx* c, double dt) {
  int rc = checkReady(c);
  if (rc) return rc;
  return launchDr(c, dt);
}

int sei_dr_get_slots(sei_ctx* c, int32_t* slots) {
  if (!c || !slots) return SEI_ERR_ARG;
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up");
  SEI_CUDA(cudaMemcpy(slots, c->dslot, (size_t)c->n * 4, cudaMemcpyDeviceToHost));
  return SEI_OK;
}

int sei_mlp_num_params(void) { return sei::mlpNumParams(); }

int sei_dr_record_samples(sei_ctx* c, int64_t capacity) {
  if (!c || capacity < 0 || capacity > (int64_t)1 << 31) return SEI_ERR_ARG;
  dropLtsGraph(c);
  if (c->cfg.device < 0) return fail(c, SEI_ERR_STATE, "host-only context");
  cudaFree(c->d_rec);
  cudaFree(c->d_rec_count);
  c->d_rec = nullptr;
  c->d_rec_count = nullptr;
  c->rec_cap = 0;
  if (capacity == 0) return SEI_OK;
  if (cudaMalloc(&c->d_rec, (size_t)capacity * 6 * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&c->d_rec_count, sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, SEI_ERR_OOM, "sample buffer allocation failed");
  }
  SEI_CUDA(cudaMemset(c->d_rec_count, 0, sizeof(unsigned)));
  c->rec_cap = (unsigned)capacity;
  return SEI_OK;
}

int sei_dr_get_samples(sei_ctx* c, float* out, int64_t max, int64_t* count) {
  if (!c || !count) return SEI_ERR_ARG;
  if (!c->d_rec) return fail(c, SEI_ERR_STATE, "no sample recording active");
  unsigned n = 0;
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  SEI_CUDA(cudaMemcpy(&n, c->d_rec_count, sizeof(unsigned), cudaMemcpyDeviceToHost));
  const int64_t avail = n < c->rec_cap ? n : c->rec_cap;
  *count = avail;
  if (out && max > 0) {
    const int64_t k = avail < max ? avail : max;
    SEI_CUDA(cudaMemcpy(out, c->d_rec, (size_t)k * 6 * sizeof(float), cudaMemcpyDeviceToHost));
  }
  return SEI_OK;
}

namespace {
constexpr size_t kNormBytes = sizeof(float) * sei_mlp::kNorm;

// Normalisation of a sample set: mean and 1 / standard deviation of the five features, mean and
// standard deviation of the target (scale 1 for constant columns), ln(2 V0).
void sampleNorm(const float* smp, int64_t n, double v0, float* norm) {
  const double ln2v0 = std::log(2.0 * v0);
  double sum[6] = {0}, sq[6] = {0};
  for (int64_t i = 0; i < n; ++i) {
    const float* r = smp + i * 6;
    double f[6];
    sei_mlp::features(r[0], r[1], r[2], r[3], r[4], f);
    f[5] = sei_mlp::target(f, ln2v0, r[5]);
    for (int k = 0; k < 6; ++k) {
      sum[k] += f[k];
      sq[k] += f[k] * f[k];
    }
  }
  for (int k = 0; k < sei_mlp::kNorm; ++k) norm[k] = 0.f;
  for (int k = 0; k < 6; ++k) {
    const double m = sum[k] / (double)n;
    const double var = sq[k] / (double)n - m * m;
    const double sd = var > 1e-12 * (1.0 + m * m) ? std::sqrt(var) : 0.0;
    if (k < 5) {
      norm[k] = (float)m;
      norm[5 + k] = sd > 0 ? (float)(1.0 / sd) : 1.f;
    } else {
      norm[10] = (float)m;
      norm[11] = sd > 0 ? (float)sd : 1.f;
    }
  }
  norm[12] = (float)ln2v0;
}

// Keeps the samples the network applies to (sei_mlp::usable).
std::vector<float> usableSamples(const float* smp, int64_t n) {
  std::vector<float> out;
  out.reserve((size_t)n * 6);
  for (int64_t i = 0; i < n; ++i)
    if (sei_mlp::usable(smp[i * 6], smp[i * 6 + 1], smp[i * 6 + 3])) out.insert(out.end(), smp + i * 6, smp + i * 6 + 6);
  return out;
}

// Splits [n][6] samples into inputs [n][5] and targets [n].
void splitSamples(const float* smp, int64_t n, std::vector<float>& X, std::vector<float>& T) {
  X.resize((size_t)n * 5);
  T.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 5; ++k) X[i * 5 + k] = smp[i * 6 + k];
    T[i] = smp[i * 6 + 5];
  }
}
}  // namespace

int sei_mlp_train(sei_ctx* c, const float* samples, int64_t n, int steps, float lr, uint64_t seed, float* loss_first,
                  float* loss_last) {
  if (!c || steps <= 0 || !(lr > 0)) return SEI_ERR_ARG;
  if (c->cfg.device < 0) return fail(c, SEI_ERR_STATE, "host-only context");
  std::vector<float> host;
  if (!samples) {
    int64_t cnt = 0;
    int rc = sei_dr_get_samples(c, nullptr, 0, &cnt);
    if (rc) return rc;
    host.resize((size_t)cnt * 6);
    rc = sei_dr_get_samples(c, host.data(), cnt, &cnt);
    if (rc) return rc;
    n = cnt;
    samples = host.data();
  }
  const std::vector<float> kept = usableSamples(samples, n);
  n = (int64_t)kept.size() / 6;
  samples = kept.data();
  if (n < 16) return fail(c, SEI_ERR_ARG, "too few training samples");
  std::vector<float> X, T;
  splitSamples(samples, n, X, T);
  if (!c->dr_ready) return fail(c, SEI_ERR_STATE, "dynamic rupture not set up (the network needs V0)");
  if (c->dr_law != SEI_LAW_FVW) return fail(c, SEI_ERR_STATE, "the network serves the rate-and-state law");
  float norm[sei_mlp::kNorm];
  sampleNorm(samples, n, c->rs.v0, norm);
  const int np = sei::mlpNumParams();
  std::vector<float> P(np, 0.f);
  // Glorot-uniform initialisation (seeded), zero biases
  uint64_t z = seed;
  auto uni = [&](double lim) {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (float)(lim * (2.0 * ((x >> 11) * (1.0 / 9007199254740992.0)) - 1.0));
  };
  const int H = 64;
  for (int i = 0; i < H * 5; ++i) P[i] = uni(std::sqrt(6.0 / (5 + H)));
  for (int i = 0; i < H * H; ++i) P[H * 5 + H + i] = uni(std::sqrt(6.0 / (2 * H)));
  for (int i = 0; i < H; ++i) P[H * 5 + H + H * H + H + i] = uni(std::sqrt(6.0 / (H + 1)));
  float *dP = nullptr, *dG = nullptr, *dM = nullptr, *dV = nullptr, *dL = nullptr, *dX = nullptr, *dT = nullptr, *dN = nullptr;
  auto cleanup = [&]() {
    for (float* p : {dG, dM, dV, dL, dX, dT, dN}) cudaFree(p);
  };
  if (cudaMalloc(&dP, np * 4) || cudaMalloc(&dG, np * 4) || cudaMalloc(&dM, np * 4) || cudaMalloc(&dV, np * 4) ||
      cudaMalloc(&dL, 4) || cudaMalloc(&dX, X.size() * 4) || cudaMalloc(&dT, T.size() * 4) || cudaMalloc(&dN, kNormBytes)) {
    cudaGetLastError();
    cudaFree(dP);
    cleanup();
    return fail(c, SEI_ERR_OOM, "training buffers");
  }
  int rc = SEI_OK;
  if (cudaMemcpy(dP, P.data(), np * 4, cudaMemcpyHostToDevice) || cudaMemset(dM, 0, np * 4) || cudaMemset(dV, 0, np * 4) ||
      cudaMemcpy(dX, X.data(), X.size() * 4, cudaMemcpyHostToDevice) ||
      cudaMemcpy(dT, T.data(), T.size() * 4, cudaMemcpyHostToDevice) || cudaMemcpy(dN, norm, kNormBytes, cudaMemcpyHostToDevice))
    rc = fail(c, SEI_ERR_CUDA, "training upload failed");
  for (int st = 0; st < steps && rc == SEI_OK; ++st) {
    const float lrt = lr * (0.05f + 0.95f * 0.5f * (1.f + std::cos(3.14159265f * st / steps)));
    if (cudaMemsetAsync(dG, 0, np * 4, c->stream) || cudaMemsetAsync(dL, 0, 4, c->stream) ||
        sei::launchMlpGrad(dP, dN, dX, dT, (int)n, dG, dL, c->sms, c->stream) ||
        sei::launchMlpAdam(dP, dG, dM, dV, lrt, st + 1, c->stream)) {
      rc = fail(c, SEI_ERR_CUDA, "training step failed");
      break;
    }
    if (st == 0 || st == steps - 1) {
      float l = 0;
      if (cudaMemcpyAsync(&l, dL, 4, cudaMemcpyDeviceToHost, c->stream) || cudaStreamSynchronize(c->stream)) {
        rc = fail(c, SEI_ERR_CUDA, "loss read failed");
        break;
      }
      if (st == 0 && loss_first) *loss_first = l;
      if (st == steps - 1 && loss_last) *loss_last = l;
    }
  }
  cleanup();
  if (rc) {
    cudaFree(dP);
    return rc;
  }
  cudaFree(c->d_mlp);
  c->d_mlp = dP;
  std::memcpy(c->mlp_norm, norm, sizeof(norm));
  dropLtsGraph(c);
  return SEI_OK;
}

int sei_mlp_get(sei_ctx* c, float* params, float* norm) {
  if (!c || !params || !norm) return SEI_ERR_ARG;
  if (!c->d_mlp) return fail(c, SEI_ERR_STATE, "no network");
  SEI_CUDA(cudaMemcpy(params, c->d_mlp, sei::mlpNumParams() * 4, cudaMemcpyDeviceToHost));
  std::memcpy(norm, c->mlp_norm, kNormBytes);
  return SEI_OK;
}

int sei_mlp_set(sei_ctx* c, const float* params, const float* norm) {
  if (c) dropLtsGraph(c);
  if (!c || !params || !norm) return SEI_ERR_ARG;
  if (c->cfg.device < 0) return fail(c, SEI_ERR_STATE, "host-only context");
  if (!c->d_mlp && cudaMalloc(&c->d_mlp, sei::mlpNumParams() * 4) != cudaSuccess) return fail(c, SEI_ERR_OOM, "network");
  SEI_CUDA(cudaMemcpy(c->d_mlp, params, sei::mlpNumParams() * 4, cudaMemcpyHostToDevice));
  std::memcpy(c->mlp_norm, norm, kNormBytes);
  return SEI_OK;
}

int sei_dr_warm_start(sei_ctx* c, int on) {
  if (!c) return SEI_ERR_ARG;
  if (on && !c->d_mlp) return fail(c, SEI_ERR_STATE, "no trained network (sei_mlp_train or sei_mlp_set)");
  if (on && c->dr_ready && c->dr_law != SEI_LAW_FVW) return fail(c, SEI_ERR_STATE, "the warm start serves the rate-and-state law");
  c->warm_start = on != 0;
  dropLtsGraph(c);
  return SEI_OK;
}

int sei_mlp_gradient(const float* params, const float* norm, const float* samples, int64_t n, float* grads, float* loss) {
  if (!params || !norm || !samples || !grads || !loss || n <= 0 || n > (int64_t)1 << 28) return SEI_ERR_ARG;
  std::vector<float> X, T;
  splitSamples(samples, n, X, T);
  const int np = sei::mlpNumParams();
  float *dP = nullptr, *dN = nullptr, *dX = nullptr, *dT = nullptr, *dG = nullptr, *dL = nullptr;
  int sms = 0, dev = 0;
  int rc = SEI_OK;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaMalloc(&dP, np * 4) || cudaMalloc(&dN, kNormBytes) || cudaMalloc(&dX, X.size() * 4) || cudaMalloc(&dT, T.size() * 4) ||
      cudaMalloc(&dG, np * 4) || cudaMalloc(&dL, 4))
    rc = SEI_ERR_OOM;
  else if (cudaMemcpy(dP, params, np * 4, cudaMemcpyHostToDevice) || cudaMemcpy(dN, norm, kNormBytes, cudaMemcpyHostToDevice) ||
           cudaMemcpy(dX, X.data(), X.size() * 4, cudaMemcpyHostToDevice) ||
           cudaMemcpy(dT, T.data(), T.size() * 4, cudaMemcpyHostToDevice) || cudaMemset(dG, 0, np * 4) ||
           cudaMemset(dL, 0, 4) || sei::launchMlpGrad(dP, dN, dX, dT, (int)n, dG, dL, sms > 0 ? sms : 1, nullptr) ||
           cudaDeviceSynchronize() || cudaMemcpy(grads, dG, np * 4, cudaMemcpyDeviceToHost) ||
           cudaMemcpy(loss, dL, 4, cudaMemcpyDeviceToHost))
    rc = SEI_ERR_CUDA;
  cudaGetLastError();
  for (float* p : {dP, dN, dX, dT, dG, dL}) cudaFree(p);
  return rc;
}

int sei_mlp_predict(const float* params, const float* norm, const float* samples, int64_t n, float* out) {
  if (!params || !norm || !samples || !out || n <= 0 || n > (int64_t)1 << 28) return SEI_ERR_ARG;
  std::vector<float> X, T;
  splitSamples(samples, n, X, T);
  const int np = sei::mlpNumParams();
  float *dP = nullptr, *dN = nullptr, *dX = nullptr, *dO = nullptr;
  int rc = SEI_OK;
  if (cudaMalloc(&dP, np * 4) || cudaMalloc(&dN, kNormBytes) || cudaMalloc(&dX, X.size() * 4) || cudaMalloc(&dO, n * 4))
    rc = SEI_ERR_OOM;
  else if (cudaMemcpy(dP, params, np * 4, cudaMemcpyHostToDevice) || cudaMemcpy(dN, norm, kNormBytes, cudaMemcpyHostToDevice) ||
           cudaMemcpy(dX, X.data(), X.size() * 4, cudaMemcpyHostToDevice) ||
           sei::launchMlpPredict(dP, dN, dX, (int)n, dO, nullptr) || cudaDeviceSynchronize() ||
           cudaMemcpy(out, dO, n * 4, cudaMemcpyDeviceToHost))
    rc = SEI_ERR_CUDA;
  cudaGetLastError();
  for (float* p : {dP, dN, dX, dO}) cudaFree(p);
  return rc;
}

namespace {
// MonomialBasis::integrate(a, b): (b^{i+1} - a^{i+1}) / (i+1)!
void subCoeffs(int order, double a, double b, float* out) {
  double pa = a, pb = b, fact = 1.0;
  for (int i = 0; i < order; ++i) {
    fact *= (i + 1);
    out[i] = (float)((pb - pa) / fact);
    pa *= a;
    pb *= b;
  }
}

int upload(sei_ctx* c, int32_t** dst, const std::vector<int32_t>& src) {
  cudaFree(*dst);
  *dst = nullptr;
  if (src.empty()) return SEI_OK;
  if (cudaMalloc(dst, src.size() * sizeof(int32_t)) != cudaSuccess) return fail(c, SEI_ERR_OOM, "LTS table allocation");
  SEI_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  return SEI_OK;
}
}  // namespace

// Host operators of the viscoelastic equations for the context's mesh: elastic blocks with the
// unrelaxed moduli (h_star, h_aplus, h_aminus), gradients, theta, W+/- and omega.
static int buildViscoHost(sei_ctx* c) {
  const double qp = c->visco_params[0], qs = c->visco_params[1], fc = c->visco_params[2], fr = c->visco_params[3];
  const int64_t n = c->mesh.n;
  sei::HostMesh um = c->mesh;  // unrelaxed moduli
  std::vector<float> theta((size_t)n * 9);
  double om[3] = {0, 0, 0};
  for (int64_t i = 0; i < n; ++i) {
    double mu = um.material[i * 3 + 1], lam = um.material[i * 3 + 2], th[3][3];
    sei::fitAttenuation(qp, qs, fc, fr, mu, lam, om, th);
    um.material[i * 3 + 1] = mu;
    um.material[i * 3 + 2] = lam;
    for (int m = 0; m < 3; ++m)
      for (int k = 0; k < 3; ++k) theta[i * 9 + m * 3 + k] = (float)th[m][k];
  }
  std::vector<float> grad, wp, wm;
  try {
    sei::buildOperators(um, c->h_star, c->h_aplus, c->h_aminus);
    sei::buildViscoOperators(um, grad, wp, wm);
  } catch (const std::exception& e) {
    return fail(c, SEI_ERR_ARG, e.what());
  }
  c->h_grad = grad;
  c->h_theta = theta;
  c->h_wplus = wp;
  c->h_wminus = wm;
  for (int m = 0; m < 3; ++m) c->omega[m] = (float)om[m];
  return SEI_OK;
}

int sei_visco_setup(sei_ctx* c, double qp, double qs, double freq_central, double freq_ratio) {
  if (!c) return SEI_ERR_ARG;
  const bool host = c->cfg.device < 0;
  int rc = host ? SEI_OK : checkReady(c);
  if (rc) return rc;
  if (!c->has_mesh) return fail(c, SEI_ERR_STATE, "the viscoelastic set-up needs a mesh built by the context");
  if (c->has_fault || c->lts || c->visco || c->plast)
    return fail(c, SEI_ERR_UNSUPPORTED,
                "viscoelastic set-up: not built with a fault, local time stepping or plasticity, or twice");
  if (c->cfg.precision != SEI_PREC_FP32) return fail(c, SEI_ERR_UNSUPPORTED, "viscoelastic kernels are FP32 only");
  sei::ViscoKernels vk{};
  if (!sei::viscoKernelsForOrder(c->cfg.order, vk))
    return fail(c, SEI_ERR_UNSUPPORTED, "viscoelastic kernels are built for orders 4 and 5");
  if (!(qp > 0) || !(qs > 0) || !(freq_central > 0) || !(freq_ratio > 1)) return fail(c, SEI_ERR_ARG, "Qp, Qs, fc > 0, ratio > 1");
  const int64_t n = c->mesh.n;
  c->visco_params[0] = qp;
  c->visco_params[1] = qs;
  c->visco_params[2] = freq_central;
  c->visco_params[3] = freq_ratio;
  if ((rc = buildViscoHost(c))) return rc;
  const std::vector<float>&grad = c->h_grad, &theta = c->h_theta, &wp = c->h_wplus, &wm = c->h_wminus;
  if (host) {  // host-only context: the operators only
    c->nq = 27;
    c->visco = true;
    return SEI_OK;
  }
  rc = uploadCells(c, n, c->h_star.data(), c->h_aplus.data(), c->h_aminus.data(), c->mesh.nbr.data(),
                   c->mesh.side.data(), c->mesh.orient.data(), c->mesh.ftype.data());
  if (rc) return rc;
  auto up = [&](float** d, const std::vector<float>& h) -> int {
    if (cudaMalloc(d, h.size() * sizeof(float)) != cudaSuccess) return fail(c, SEI_ERR_OOM, "viscoelastic arrays");
    SEI_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    return SEI_OK;
  };
  if ((rc = up(&c->d_grad, grad)) || (rc = up(&c->d_theta, theta)) || (rc = up(&c->d_wplus, wp)) ||
      (rc = up(&c->d_wminus, wm)))
    return rc;
  // Q and I with 27 quantities: the elastic DOFs move over, the memory variables start at zero
  const size_t blk9 = (size_t)9 * c->Bp, blk27 = (size_t)27 * c->Bp;
  std::vector<float> q9((size_t)n * blk9), q27((size_t)n * blk27, 0.f);
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  SEI_CUDA(cudaMemcpy(q9.data(), c->Q, q9.size() * sizeof(float), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; ++i) std::memcpy(&q27[i * blk27], &q9[i * blk9], blk9 * sizeof(float));
  cudaFree(c->Q);
  cudaFree(c->I);
  c->Q = c->I = nullptr;
  if (cudaMalloc(&c->Q, q27.size() * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&c->I, q27.size() * sizeof(float)) != cudaSuccess)
    return fail(c, SEI_ERR_OOM, "viscoelastic DOF arrays");
  SEI_CUDA(cudaMemcpy(c->Q, q27.data(), q27.size() * sizeof(float), cudaMemcpyHostToDevice));
  SEI_CUDA(cudaMemset(c->I, 0, q27.size() * sizeof(float)));
  c->vk = vk;
  c->nq = 27;
  c->visco = true;
  return SEI_OK;
}

int sei_num_quantities(const sei_ctx* c) { return c ? c->nq : 0; }

int sei_visco_operators(sei_ctx* c, float* grad, float* theta, float* wplus, float* wminus, double* omega) {
  if (!c) return SEI_ERR_ARG;
  if (!c->visco) return fail(c, SEI_ERR_STATE, "viscoelastic set-up not done");
  auto cp = [](float* dst, const std::vector<float>& src) {
    if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(float));
  };
  cp(grad, c->h_grad);
  cp(theta, c->h_theta);
  cp(wplus, c->h_wplus);
  cp(wminus, c->h_wminus);
  if (omega)
    for (int m = 0; m < 3; ++m) omega[m] = c->omega[m];
  return SEI_OK;
}

int sei_fit_attenuation(double qp, double qs, double freq_central, double freq_ratio, double* mu, double* lam,
                        double* omega, double* theta) {
  if (!mu || !lam || !omega || !theta || !(qp > 0) || !(qs > 0) || !(freq_central > 0) || !(freq_ratio > 1))
    return SEI_ERR_ARG;
  double th[3][3];
  sei::fitAttenuation(qp, qs, freq_central, freq_ratio, *mu, *lam, omega, th);
  for (int m = 0; m < 3; ++m)
    for (int k = 0; k < 3; ++k) theta[m * 3 + k] = th[m][k];
  return SEI_OK;
}

int sei_lts_setup(sei_ctx* c, double cfl, int max_clusters, int* nclusters) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->has_mesh) return fail(c, SEI_ERR_STATE, "local time stepping needs a mesh built by the context");
  if (c->has_fault && !c->dr_ready)
    return fail(c, SEI_ERR_STATE, "set up dynamic rupture (sei_dr_setup) before local time stepping");
  if (c->lts) return fail(c, SEI_ERR_STATE, "local time stepping is already set up");
  if (!(cfl > 0) || max_clusters < 1 || max_clusters > 16) return fail(c, SEI_ERR_ARG, "cfl > 0, 1 <= max_clusters <= 16");
  const int64_t n = c->n;
  std::vector<double> dt;
  sei::cellTimesteps(c->mesh, c->cfg.order, cfl, dt);
  double dt0 = 1e300;
  for (double v : dt) dt0 = std::min(dt0, v);
  // rate-2 clusters: cluster k holds the time steps in [2^k dt0, 2^{k+1} dt0)
  std::vector<int> cl(n);
  for (int64_t i = 0; i < n; ++i) {
    int k = (int)std::floor(std::log2(dt[i] / dt0) + 1e-12);
    cl[i] = std::max(0, std::min(max_clusters - 1, k));
  }
  // maximum difference property: neighbouring clusters differ by at most one; both cells of a
  // dynamic-rupture face share one cluster, the lower (docs/local-timestepping.rst:91-96)
  const int64_t nf = c->dr_ready ? c->fault.nf : 0;
  for (bool changed = true; changed;) {
    changed = false;
    for (int64_t f = 0; f < nf; ++f) {
      const int32_t pa = c->fault.plus_cell[f], pb = c->fault.minus_cell[f];
      const int m = std::min(cl[pa], cl[pb]);
      if (cl[pa] != m || cl[pb] != m) {
        cl[pa] = cl[pb] = m;
        changed = true;
      }
    }
    for (int64_t i = 0; i < n; ++i)
      for (int f = 0; f < 4; ++f) {
        if (c->mesh.ftype[i * 4 + f] != 0) continue;
        const int32_t nb = c->mesh.nbr[i * 4 + f];
        if (cl[i] > cl[nb] + 1) {
          cl[i] = cl[nb] + 1;
          changed = true;
        }
      }
  }
  int ncl = 0;
  for (int v : cl) ncl = std::max(ncl, v + 1);
  // stable reorder by cluster
  std::vector<int64_t> order(n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cl[a] < cl[b]; });
  const int blk = c->nq * c->Bp;
  std::vector<float> qold((size_t)n * blk), qnew((size_t)n * blk);
  SEI_CUDA(cudaStreamSynchronize(c->stream));
  SEI_CUDA(cudaMemcpy(qold.data(), c->Q, qold.size() * sizeof(float), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; ++i)
    std::memcpy(&qnew[(size_t)i * blk], &qold[(size_t)order[i] * blk], blk * sizeof(float));
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; ++i) inv[order[i]] = i;
  try {
    sei::permuteCells(c->mesh, order);
    // the fault faces follow their cells; the recomputed face relations are regular, so the
    // dynamic-rupture faces are marked again before the operators are built
    for (int64_t f = 0; f < nf; ++f) {
      c->fault.plus_cell[f] = (int32_t)inv[c->fault.plus_cell[f]];
      c->fault.minus_cell[f] = (int32_t)inv[c->fault.minus_cell[f]];
      c->mesh.ftype[(int64_t)c->fault.plus_cell[f] * 4 + c->fault.plus_side[f]] = 1;
      c->mesh.ftype[(int64_t)c->fault.minus_cell[f] * 4 + c->fault.minus_side[f]] = 1;
    }
    if (!c->visco) sei::buildOperators(c->mesh, c->h_star, c->h_aplus, c->h_aminus);
  } catch (const std::exception& e) {
    return fail(c, SEI_ERR_ARG, e.what());
  }
  if (c->visco) {  // the viscoelastic operators of the reordered cells
    if ((rc = buildViscoHost(c))) return rc;
    for (auto [d, h] : {std::pair<float*, const std::vector<float>*>{c->d_grad, &c->h_grad}, {c->d_theta, &c->h_theta},
                        {c->d_wplus, &c->h_wplus}, {c->d_wminus, &c->h_wminus}})
      SEI_CUDA(cudaMemcpy(d, h->data(), h->size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  rc = uploadCells(c, n, c->h_star.data(), c->h_aplus.data(), c->h_aminus.data(), c->mesh.nbr.data(),
                   c->mesh.side.data(), c->mesh.orient.data(), c->mesh.ftype.data());
  if (rc) return rc;
  SEI_CUDA(cudaMemcpy(c->Q, qnew.data(), qnew.size() * sizeof(float), cudaMemcpyHostToDevice));
  std::vector<int> cn(n);
  for (int64_t i = 0; i < n; ++i) cn[i] = cl[order[i]];
  std::vector<int64_t> cs(ncl + 1, 0);
  for (int64_t i = 0; i < n; ++i) ++cs[cn[i] + 1];
  for (int k = 0; k < ncl; ++k) cs[k + 1] += cs[k];
  // buffers (cells with a coarser neighbour), derivative slots (cells with a finer neighbour)
  std::vector<int32_t> bslot(n, -1), dsl(n, -1);
  int64_t nB = 0, nD = 0;
  for (int64_t i = 0; i < n; ++i) {
    bool coarser = false, finer = false;
    for (int f = 0; f < 4; ++f) {
      if (c->mesh.ftype[i * 4 + f] != 0) continue;
      const int d = cn[c->mesh.nbr[i * 4 + f]] - cn[i];
      coarser |= d > 0;
      finer |= d < 0;
    }
    if (coarser) bslot[i] = (int32_t)nB++;
    if (finer) dsl[i] = (int32_t)nD++;
  }
  // fault cells store their derivatives too (the fault kernel interpolates them in time), and
  // the faces are listed by the cluster of their cells
  std::vector<int32_t> pslot(nf), mslot(nf), fidx;
  std::vector<int64_t> fst(ncl + 1, 0);
  for (int64_t f = 0; f < nf; ++f)
    for (int sd = 0; sd < 2; ++sd) {
      const int32_t cc = sd ? c->fault.minus_cell[f] : c->fault.plus_cell[f];
      if (dsl[cc] < 0) dsl[cc] = (int32_t)nD++;
      (sd ? mslot : pslot)[f] = dsl[cc];
    }
  for (int k = 0; k < ncl; ++k) {
    for (int64_t f = 0; f < nf; ++f)
      if (cn[c->fault.plus_cell[f]] == k) fidx.push_back((int32_t)f);
    fst[k + 1] = (int64_t)fidx.size();
  }
  // every cell with a finer neighbour gets two half-step blocks, the Taylor integrals of its step's
  // first and second half (computed once after its ADER); a finer cell's face reads the one of its
  // sub-step, through the source table of that parity
  std::vector<int32_t> hslot(n, -1);
  int64_t nH = 0;
  for (int64_t i = 0; i < n; ++i) {
    bool finer = false;
    for (int f = 0; f < 4; ++f)
      if (c->mesh.ftype[i * 4 + f] == 0) finer |= cn[c->mesh.nbr[i * 4 + f]] < cn[i];
    if (finer) hslot[i] = (int32_t)nH++;
  }
  // per-face sources (two parities); buffer entries grouped by the cluster of the reading cell,
  // half-step entries by the cluster of the coarse cell
  std::vector<int32_t> src((size_t)n * 4), src1((size_t)n * 4);
  std::vector<std::vector<int32_t>> bc(ncl), bd(ncl), gs(ncl), gd(ncl);
  for (int64_t i = 0; i < n; ++i) {
    if (bslot[i] >= 0) {
      bc[cn[i]].push_back((int32_t)i);
      bd[cn[i]].push_back((int32_t)(n + bslot[i]));
    }
    if (hslot[i] >= 0) {
      gs[cn[i]].push_back(dsl[i]);
      gd[cn[i]].push_back((int32_t)(n + nB + 2 * hslot[i]));
    }
    for (int f = 0; f < 4; ++f) {
      const int32_t nb = c->mesh.nbr[i * 4 + f];
      int32_t a = nb, b = nb;
      if (c->mesh.ftype[i * 4 + f] == 0) {
        const int d = cn[nb] - cn[i];
        if (d < 0) {
          a = b = (int32_t)(n + bslot[nb]);
        } else if (d > 0) {
          a = (int32_t)(n + nB + 2 * hslot[nb]);
          b = a + 1;
        }
      }
      src[i * 4 + f] = a;
      src1[i * 4 + f] = b;
    }
  }
  const int64_t nS = 2 * nH;
  if (n + nB + nS > INT32_MAX) return fail(c, SEI_ERR_ARG, "mesh too large for 32-bit pool indices");
  std::vector<int32_t> fbc, fbd, fgs, fgd, fgd1;
  std::vector<int64_t> bs(ncl + 1, 0), gst(ncl + 1, 0);
  for (int k = 0; k < ncl; ++k) {
    fbc.insert(fbc.end(), bc[k].begin(), bc[k].end());
    fbd.insert(fbd.end(), bd[k].begin(), bd[k].end());
    fgs.insert(fgs.end(), gs[k].begin(), gs[k].end());
    fgd.insert(fgd.end(), gd[k].begin(), gd[k].end());
    bs[k + 1] = (int64_t)fbc.size();
    gst[k + 1] = (int64_t)fgs.size();
  }
  for (int32_t v : fgd) fgd1.push_back(v + 1);
  // device: the I pool, derivative slots, tables
  cudaFree(c->I);
  c->I = nullptr;
  c->trace_valid = false;
  if (cudaMalloc(&c->I, (size_t)(n + nB + nS) * blk * sizeof(float)) != cudaSuccess)
    return fail(c, SEI_ERR_OOM, "LTS pool allocation");
  SEI_CUDA(cudaMemset(c->I, 0, (size_t)(n + nB + nS) * blk * sizeof(float)));
  cudaFree(c->derivs);
  c->derivs = nullptr;
  const int dsz = c->visco ? c->vk.derivSize : sei::derivativesSize(c->cfg.order);
  if (nD > 0 && cudaMalloc(&c->derivs, (size_t)nD * dsz * sizeof(float)) != cudaSuccess)
    return fail(c, SEI_ERR_OOM, "LTS derivative allocation");
  c->nslots = nD;
  c->npool = n + nB + nS;
  c->lts_trace = false;
  if (c->cfg.precision == SEI_PREC_F16X3 && !c->visco) {
    // the tensor-core neighbour path reads face traces through the pool indices of d_src
    cudaFree(c->d_trace);
    c->d_trace = nullptr;
    const size_t tb = (size_t)c->npool * sei::traceFloatsPerCell(c->cfg.order) * sizeof(float);
    if (cudaMalloc(&c->d_trace, tb) != cudaSuccess) return fail(c, SEI_ERR_OOM, "LTS trace allocation");
    SEI_CUDA(cudaMemset(c->d_trace, 0, tb));
    c->lts_trace = true;
  }
  if ((rc = upload(c, &c->dslot, dsl)) || (rc = upload(c, &c->d_src, src)) || (rc = upload(c, &c->d_src1, src1)) ||
      (rc = upload(c, &c->d_bcell, fbc)) || (rc = upload(c, &c->d_bdst, fbd)) || (rc = upload(c, &c->d_gsrc, fgs)) ||
      (rc = upload(c, &c->d_gdst, fgd)) || (rc = upload(c, &c->d_gdst1, fgd1)))
    return rc;
  if (nf > 0) {
    if ((rc = upload(c, &c->d_fidx, fidx)) || (rc = upload(c, &c->d_pslot, pslot)) || (rc = upload(c, &c->d_mslot, mslot)) ||
        (rc = upload(c, &c->d_pc, c->fault.plus_cell)) || (rc = upload(c, &c->d_mc, c->fault.minus_cell)))
      return rc;
  }
  c->f_start = fst;
  c->lts = true;
  c->ncl = ncl;
  c->lts_dt0 = dt0;
  c->cl_start = cs;
  c->b_start = bs;
  c->g_start = gst;
  c->lts_perm = order;
  if (nclusters) *nclusters = ncl;
  if (c->plast && (rc = plastPermute(c, order))) return rc;
  if (c->nrecv > 0) {
    // the cells moved: locate the receivers again on the reordered mesh (their clocks restart)
    const std::vector<double> pts = c->recv_xyz;
    const int derived = c->recv_derived;
    return sei_receivers_setup(c, (int64_t)pts.size() / 3, pts.data(), c->recv_interval, c->recv_qmask, derived, nullptr);
  }
  return SEI_OK;
}

namespace {
// Cells [s, e) of the context as a kernel view; the neighbour view reads the pool through d_src.
sei::DeviceArrays rangeView(sei_ctx* c, int64_t s, int64_t e, bool neighbour, int parity = 0) {
  const size_t blk = (size_t)9 * c->Bp;
  sei::DeviceArrays d{};
  d.n = (int)(e - s);
  d.Q = c->Q + s * blk;
  d.I = neighbour ? c->I : c->I + s * blk;
  d.derivs = c->derivs;
  d.dslot = c->dslot ? c->dslot + s : nullptr;
  d.star_nz = c->star_nz + s * 3 * sei::kStarNnz;
  d.aplus = c->aplus + s * 4 * 81;
  d.aminus = c->aminus + s * 4 * 81;
  d.nbr = (neighbour ? (parity ? c->d_src1 : c->d_src) : c->nbr) + s * 4;
  d.rel = c->rel + s * 4;
  d.ftype = c->ftype + s * 4;
  d.status = c->d_status;
  if (c->lts_trace) {  // traces addressed by pool block: plane stride npool, the range from cell s
    d.first = (int)s;
    d.ntotal = (int)c->npool;
  }
  return d;
}

sei::ViscoArrays viscoRangeView(sei_ctx* c, int64_t s, int64_t e, bool neighbour, int parity = 0) {
  const size_t blk = (size_t)c->nq * c->Bp;
  sei::ViscoArrays v = viscoArrays(c);
  v.n = (int)(e - s);
  v.Q = c->Q + s * blk;
  v.I = neighbour ? c->I : c->I + s * blk;
  v.star_nz = c->star_nz + s * 3 * sei::kStarNnz;
  v.grad = c->d_grad + s * 9;
  v.theta = c->d_theta + s * 9;
  v.aplus = c->aplus + s * 4 * 81;
  v.wplus = c->d_wplus + s * 4 * 54;
  v.aminus = c->aminus + s * 4 * 81;
  v.wminus = c->d_wminus + s * 4 * 54;
  v.nbr = (neighbour ? (parity ? c->d_src1 : c->d_src) : c->nbr) + s * 4;
  v.rel = c->rel + s * 4;
  v.ftype = c->ftype + s * 4;
  v.derivs = c->derivs;
  v.dslot = c->dslot ? c->dslot + s : nullptr;
  return v;
}

// One cycle: every cluster advances by dt0 2^(ncl-1).  Sub-step k of the finest cluster starts
// with the predictions (ADER, the half-step integrals of cells with a finer neighbour, integration
// buffer, local integral) of the clusters whose step begins at k, then the corrections (the fault
// faces of the cluster, neighbour flux) of the clusters whose step ends at k + 1 (TimeCluster
// predict / correct, TimeCommon::computeIntegrals).
int ltsCycle(sei_ctx* c) {
  NvtxRange range("sei LTS cycle");
  int rc0 = SEI_OK;
  const int blk = c->nq * c->Bp;
  const int64_t steps = (int64_t)1 << (c->ncl - 1);
  float co[8];
  for (int64_t k = 0; k < steps; ++k) {
    for (int cl = 0; cl < c->ncl; ++cl) {
      const int64_t len = (int64_t)1 << cl;
      if (k % len) continue;
      const int64_t s = c->cl_start[cl], e = c->cl_start[cl + 1];
      if (s == e) continue;
      const double dtc = c->lts_dt0 * (double)len;
      if (c->nrecv && (rc0 = recordReceivers(c, cl, c->sim_time + c->lts_dt0 * (double)k, dtc,
                                             c->nrecv + c->recv_gstart[cl],
                                             c->recv_gstart[cl + 1] - c->recv_gstart[cl])))
        return rc0;
      taylorCoeffs(c->cfg.order, dtc, co);
      sei::DeviceArrays d = rangeView(c, s, e, false);
      const sei::ViscoArrays v = c->visco ? viscoRangeView(c, s, e, false) : sei::ViscoArrays{};
      int rc;
      if (c->visco) {
        if ((rc = profMark(c, 0))) return rc;
        if (c->vk.ader(v, co, c->stream)) return fail(c, SEI_ERR_CUDA, "viscoelastic ADER launch failed");
      } else if ((rc = launchAderOnly(c, d, co))) {
        return rc;
      }
      // the two half-step integrals of the cells with a finer neighbour (TimeCommon.cpp:40-87,
      // evaluated once per coarse step instead of once per reading face)
      const int64_t gs = c->g_start[cl], ge = c->g_start[cl + 1];
      if (ge > gs) {
        if ((rc = profMark(c, 4))) return rc;
        const int m = (int)(ge - gs);
        for (int half = 0; half < 2; ++half) {
          subCoeffs(c->cfg.order, 0.5 * dtc * half, 0.5 * dtc * (half + 1), co);
          const int32_t* dst = (half ? c->d_gdst1 : c->d_gdst) + gs;
          if (c->visco ? sei::launchTaylorGatherFull(m, c->d_gsrc + gs, dst, c->derivs, c->cfg.order, c->nq,
                                                     sei::numBasis(c->cfg.order), c->Bp, co, c->I, c->stream)
                       : c->k.taylorGather(m, c->d_gsrc + gs, dst, c->derivs, co, c->I, c->stream))
            return fail(c, SEI_ERR_CUDA, "LTS half-step kernel launch failed");
          // the traces of the half-step blocks, which the finer neighbours' faces read
          if (c->lts_trace && c->k.traceBlocks(m, dst, c->I, c->d_trace, (int)c->npool, c->stream))
            return fail(c, SEI_ERR_CUDA, "LTS half-step trace kernel launch failed");
        }
      }
      const int64_t bs = c->b_start[cl], be = c->b_start[cl + 1];
      // the tensor-core path reads the buffer's traces (summed after the local integral below),
      // not its time-integrated DOFs
      if (be > bs && !c->lts_trace) {
        if ((rc = profMark(c, 4))) return rc;
        // a new step of the next coarser cluster begins when k / len is even
        if (sei::launchLtsBuffer((int)(be - bs), c->d_bcell + bs, c->d_bdst + bs, c->I, blk, ((k / len) % 2) == 0,
                                 c->stream))
          return fail(c, SEI_ERR_CUDA, "LTS buffer kernel launch failed");
      }
      if (c->visco) {
        if ((rc = profMark(c, 3))) return rc;
        if (c->vk.lint(v, c->stream)) return fail(c, SEI_ERR_CUDA, "viscoelastic local-integral launch failed");
      } else if ((rc = launchLintOnly(c, d, fusedFlux(c)))) {
        return rc;
      }
      if (be > bs && c->lts_trace) {
        if ((rc = profMark(c, 4))) return rc;
        const int row = 9 * ((sei::numFaceBasis(c->cfg.order) + 3) / 4 * 4);
        if (sei::launchLtsTraceBuffer((int)(be - bs), c->d_bcell + bs, c->d_bdst + bs, c->d_trace, c->npool, row,
                                      ((k / len) % 2) == 0, c->stream))
          return fail(c, SEI_ERR_CUDA, "LTS trace buffer kernel launch failed");
      }
    }
    for (int cl = 0; cl < c->ncl; ++cl) {
      const int64_t len = (int64_t)1 << cl;
      if ((k + 1) % len) continue;
      const int64_t s = c->cl_start[cl], e = c->cl_start[cl + 1];
      if (s == e) continue;
      // which half of the next coarser cluster's step this step is
      const int parity = (int)(((k + 1 - len) / len) % 2);
      // the fault faces of this cluster first (TimeCluster.cpp:804-823), over its own step
      if (!c->f_start.empty() && c->f_start[cl + 1] > c->f_start[cl]) {
        int rc = profMark(c, 2);
        if (rc) return rc;
        sei::DrArgs a = drArgs(c, c->lts_dt0 * (double)len);
        a.time_offset = c->lts_dt0 * (double)(k + 1 - len);  // this step's start within the cycle
        a.fidx = c->d_fidx;
        a.face_begin = (int)c->f_start[cl];
        a.face_count = (int)(c->f_start[cl + 1] - c->f_start[cl]);
        if (sei::launchDrFaces(c->cfg.order, a, c->stream) != 0) return fail(c, SEI_ERR_CUDA, "fault kernel launch failed");
      }
      if (c->visco) {
        int rc = profMark(c, 1);
        if (rc) return rc;
        if (c->vk.neighbor(viscoRangeView(c, s, e, true, parity), c->stream))
          return fail(c, SEI_ERR_CUDA, "viscoelastic neighbour launch failed");
        continue;
      }
      int rc = launchNeighbor(c, rangeView(c, s, e, true, parity), fusedFlux(c));
      if (!rc) rc = launchPlast(c, s, e, c->lts_dt0 * (double)len);
      if (rc) return rc;
    }
  }
  // the fault time moves on by one cycle (the fault kernels above read it as their base)
  if (!c->f_start.empty() && c->f_start.back() > 0 &&
      sei::launchDrAdvanceTime(c->d_time, c->lts_dt0 * (double)steps, c->stream) != 0)
    return fail(c, SEI_ERR_CUDA, "fault time launch failed");
  return SEI_OK;
}
}  // namespace

int sei_lts_run(sei_ctx* c, int ncycles) {
  int rc = checkReady(c);
  if (rc) return rc;
  if (!c->lts) return fail(c, SEI_ERR_STATE, "local time stepping not set up (sei_lts_setup)");
  if (ncycles < 0) return fail(c, SEI_ERR_ARG, "ncycles < 0");
  c->prof_used = 0;
  // receivers change their launches from cycle to cycle (sample counts, staging): no graph then
  const bool graph = c->lts_graph && c->nrecv == 0;
  if (graph && !c->lts_exec && ncycles > 0) {
    // record one cycle (relaxed mode: the launchers set kernel attributes while recording)
    SEI_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    c->capturing = true;
    rc = ltsCycle(c);
    c->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc == SEI_OK && e != cudaSuccess) rc = cudaFail(c, e, "cudaStreamEndCapture");
    if (rc == SEI_OK && cudaGraphInstantiate(&c->lts_exec, g, 0) != cudaSuccess)
      rc = fail(c, SEI_ERR_CUDA, "cudaGraphInstantiate of the LTS cycle failed");
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (rc) return rc;
  }
  SEI_CUDA(cudaEventRecord(c->ev0, c->stream));
  for (int i = 0; i < ncycles && rc == SEI_OK; ++i) {
    if (graph) {
      if (cudaGraphLaunch(c->lts_exec, c->stream) != cudaSuccess) rc = fail(c, SEI_ERR_CUDA, "cudaGraphLaunch failed");
    } else {
      rc = ltsCycle(c);
    }
    if (rc == SEI_OK) c->sim_time += c->lts_dt0 * (double)((int64_t)1 << (c->ncl - 1));
  }
  if (!rc) rc = profMark(c, -1);
  SEI_CUDA(cudaEventRecord(c->ev1, c->stream));
  return rc;
}

int sei_lts_clusters(sei_ctx* c, int* nclusters, int64_t* start, double* dt) {
  if (!c || !nclusters) return SEI_ERR_ARG;
  if (!c->lts) return fail(c, SEI_ERR_STATE, "local time stepping not set up (sei_lts_setup)");
  *nclusters = c->ncl;
  for (int k = 0; k <= c->ncl; ++k)
    if (start) start[k] = c->cl_start[k];
  for (int k = 0; k < c->ncl; ++k)
    if (dt) dt[k] = c->lts_dt0 * (double)((int64_t)1 << k);
  return SEI_OK;
}

int sei_lts_permutation(sei_ctx* c, int64_t* perm) {
  if (!c || !perm) return SEI_ERR_ARG;
  if (!c->lts) return fail(c, SEI_ERR_STATE, "local time stepping not set up (sei_lts_setup)");
  std::memcpy(perm, c->lts_perm.data(), c->lts_perm.size() * sizeof(int64_t));
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
    if (c->prof_kind[i] == 0 || c->prof_kind[i] == 3) *local_ms += ms;
    if (c->prof_kind[i] == 1) *neighbor_ms += ms;
    ++*launches;
  }
  return SEI_OK;
}

int sei_kernel_times_by_kind(sei_ctx* c, double* ms, int* counts) {
  if (!c || !ms || !counts) return SEI_ERR_ARG;
  for (int k = 0; k < 4; ++k) ms[k] = 0.0, counts[k] = 0;
  if (!c->profiling || c->prof_used < 2) return fail(c, SEI_ERR_STATE, "profiling off or nothing recorded");
  SEI_CUDA(cudaEventSynchronize(c->prof_events[c->prof_used - 1]));
  for (size_t i = 0; i + 1 < c->prof_used; ++i) {
    const int k = c->prof_kind[i];
    if (k < 0 || k > 3) continue;
    float t = 0;
    SEI_CUDA(cudaEventElapsedTime(&t, c->prof_events[i], c->prof_events[i + 1]));
    ms[k] += t;
    ++counts[k];
  }
  return SEI_OK;
}

int sei_autotune(sei_ctx* c, double dt, int steps, sei_tune_result* out) {
  NvtxRange range("sei_autotune");
  int rc = checkReady(c);
  if (rc) return rc;
  if (c->visco || c->lts) return fail(c, SEI_ERR_UNSUPPORTED, "the autotuner covers global stepping of the elastic kernels");
  if (!(dt > 0) || steps < 1 || steps > 1000) return fail(c, SEI_ERR_ARG, "dt > 0, 1 <= steps <= 1000");
  struct Cand {
    int fused, tcLocal, nbCtas, nbForm;
  };
  std::vector<Cand> cands;
  if (c->cfg.precision == SEI_PREC_FP32) {
    cands = {{0, 0, 3, 1}, {1, 0, 3, 1}};
  } else {
    // local integral on the CUDA cores, transposed or rows-form tensor cores; neighbour
    // transposed, or rows form with 1..3 CTAs per SM
    for (int t = 0; t < 3; ++t) {
      cands.push_back({0, t, 3, 1});
      for (int k = 1; k <= 3; ++k) cands.push_back({0, t, k, 0});
    }
    cands.push_back({0, 0, 3, 2});  // local flux inside the transposed neighbour kernel
    cands.push_back({1, 0, 3, 2});  // the same after one ADER + volume + trace launch
  }
  // the DOFs are restored after every candidate: tuning leaves the state unchanged
  const size_t bytes = (size_t)c->n * 9 * c->Bp * sizeof(float);
  float* save = nullptr;
  if (cudaMalloc(&save, bytes) != cudaSuccess) return fail(c, SEI_ERR_OOM, "autotuner DOF copy");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool prof = c->profiling;
  c->profiling = false;
  // the knobs the context had on entry: a failed tune gives them back instead of the failed variant
  const bool fused0 = c->fused_local;
  const int tc0 = c->tc_local;
  const int nbCtas0 = c->nb_ctas, nbForm0 = c->nb_form;
  bool saved = false;
  auto done = [&](int code) {
    if (code != SEI_OK) {
      c->fused_local = fused0;
      c->tc_local = tc0;
      c->nb_ctas = nbCtas0;
      c->nb_form = nbForm0;
      c->trace_valid = false;  // the DOFs are put back below; traces of a variant are stale
    }
    if (code != SEI_OK && saved) {  // a variant failed: put the DOFs back before giving up
      cudaMemcpyAsync(c->Q, save, bytes, cudaMemcpyDeviceToDevice, c->stream);
      cudaStreamSynchronize(c->stream);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(save);
    c->profiling = prof;
    return code;
  };
  if (cudaMemcpyAsync(save, c->Q, bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
    return done(fail(c, SEI_ERR_CUDA, "autotuner DOF copy"));
  saved = true;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return done(fail(c, SEI_ERR_CUDA, "autotuner set-up"));
  double best = 1e300, worst = 0.0;
  Cand pick = cands[0];
  for (size_t ci = 0; ci < cands.size(); ++ci) {
    const Cand& k = cands[ci];
    c->fused_local = k.fused != 0;
    c->tc_local = k.tcLocal;
    c->nb_ctas = k.nbCtas;
    c->nb_form = k.nbForm;
    c->trace_valid = false;
    if ((rc = runKernel(c, SEI_KERNEL_ALL, dt, 1))) return done(rc);  // warm-up
    if ((int)ci == c->tune_fail_at) return done(fail(c, SEI_ERR_CUDA, "autotuner: failure injected on the host"));
    if (cudaEventRecord(e0, c->stream) != cudaSuccess) return done(fail(c, SEI_ERR_CUDA, "event record"));
    if ((rc = runKernel(c, SEI_KERNEL_ALL, dt, steps))) return done(rc);
    float ms = 0.f;
    if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      return done(fail(c, SEI_ERR_CUDA, "autotuner timing"));
    const double per = (double)ms / steps;
    if (per < best) {
      best = per;
      pick = k;
    }
    worst = per > worst ? per : worst;
    if (cudaMemcpyAsync(c->Q, save, bytes, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
      return done(fail(c, SEI_ERR_CUDA, "autotuner DOF restore"));
  }
  c->fused_local = pick.fused != 0;
  c->tc_local = pick.tcLocal;
  c->nb_ctas = pick.nbCtas;
  c->nb_form = pick.nbForm;
  c->trace_valid = false;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return done(fail(c, SEI_ERR_CUDA, "autotuner sync"));
  if (out) {
    out->fused_local = pick.fused;
    out->tc_local = pick.tcLocal;
    out->nb_ctas = pick.nbCtas;
    out->nb_form = pick.nbForm;
    out->candidates = (int)cands.size();
    out->best_ms = best;
    out->worst_ms = worst;
  }
  return done(SEI_OK);
}

int sei_metrics(const sei_ctx* c, int kernel, sei_perf* out) {
  if (!c || !out) return SEI_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  if (c->visco) return SEI_ERR_UNSUPPORTED;
  // per cell: the generated kernels execute exactly their non-zero flops (hardware = non-zero);
  // bytes: compulsory float32 traffic, every array touched once (DOF blocks 9 x Bp)
  const double dof = 4.0 * 9 * c->Bp, star = 4.0 * 72, flux = 4.0 * 4 * 81, rel = 4.0 * 4 + 4 + 4;
  const double fa = c->k.flopAder, fl = c->k.flopLocal, fn = c->k.flopNeighbor;
  double flop = 0, bytes = 0;
  switch (kernel) {
    case SEI_KERNEL_ALL: flop = fa + fl + fn; bytes = 4 * dof + star + 2 * flux + 4.0 * 4 + 4; break;
    case SEI_KERNEL_LOCAL: flop = fa + fl; bytes = 3 * dof + star + flux + 4; break;
    case SEI_KERNEL_ADER: flop = fa; bytes = 2 * dof + star; break;
    case SEI_KERNEL_LOCAL_WO_ADER: flop = fl; bytes = 3 * dof + star + flux + 4; break;
    case SEI_KERNEL_NEIGHBOR: flop = fn; bytes = 3 * dof + flux + rel; break;
    default: return SEI_ERR_UNSUPPORTED;
  }
  out->nonzero_flop = flop;
  out->hardware_flop = flop;
  out->bytes = bytes;
  return SEI_OK;
}

}  // extern "C"
