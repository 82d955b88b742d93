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
  std::vector<int8_t> bc;  // [n][4] boundary condition of a boundary face (1 free surface, 5 absorbing), else 0; empty: none
  double fault_x = 0.0;  // x of the cube's fault plane (cube vertex plane fault_plane), when built
};

void buildPeriodicCube(const sei_cube_params& p, HostMesh& m);
void computeFaceRelations(HostMesh& m);
void buildOperators(const HostMesh& m, std::vector<float>& star, std::vector<float>& aplus, std::vector<float>& aminus);
double cflTimestep(const HostMesh& m, int order, double cfl);
// CFL time step of every cell (GlobalTimestep.cpp:27-47 per element).
void cellTimesteps(const HostMesh& m, int order, double cfl, std::vector<double>& dt);
// Reorders the cells: new cell i is old cell order[i]; face relations are recomputed.
void permuteCells(HostMesh& m, const std::vector<int64_t>& order);

// Viscoelastic attenuation (3 mechanisms): relaxed mu, lambda in, unrelaxed out (Attenuation.h).
constexpr int kMechanisms = 3;
void fitAttenuation(double qp, double qs, double freqCentral, double freqRatio, double& mu, double& lam,
                    double omega[kMechanisms], double theta[kMechanisms][3]);
// Per cell: grad [n][3][3] (d xi_e / d x), and the 9 x 6 memory-variable flux blocks W+, W-
// [n][4][9 + 9 j] (memory variable j of mechanism l receives omega_l W).
void buildViscoOperators(const HostMesh& m, std::vector<float>& grad, std::vector<float>& wplus,
                         std::vector<float>& wminus);
void seedDofs(int64_t n, int order, uint64_t seed, std::vector<float>& dofs);

// Kernel launchers (one translation unit per order).
struct DeviceArrays {
  int n;
  float* Q;
  float* I;
  float* derivs;        // nullable
  const int32_t* dslot;  // nullable: derivative slot per cell (-1 none); nullptr = slot is the cell
  const float* star_nz;
  const float* aplus;
  const float* aminus;
  const int32_t* nbr;
  const uint8_t* rel;    // side | orient << 2
  const uint8_t* ftype;  // 0 regular, 1 dynamic rupture, 2 none
  float* trace = nullptr;  // nullable: face traces fMrT_f I out of the local integral, [4][ntotal][9][FP]
  int ntotal = 0;          // cells of the whole mesh when this view covers a range of them (0: n)
  int first = 0;           // first cell of the range
  int* status = nullptr;   // nullable: device status word (set when a bounded wait gives up)
};

using LaunchLocalFn = int (*)(const DeviceArrays&, const float* coeffs, void* stream);
using LaunchNeighborFn = int (*)(const DeviceArrays&, void* stream);
using LaunchTaylorFn = int (*)(int n, const float* derivs, const float* coeffs, float* out, void* stream);

using LaunchLintFn = int (*)(const DeviceArrays&, void* stream);
// pool[dst[e]] = Taylor sum of derivative slot src[e], e < m (local time stepping)
using LaunchTaylorGatherFn = int (*)(int m, const int32_t* src, const int32_t* dst, const float* derivs,
                                     const float* coeffs, float* pool, void* stream);

struct OrderKernels {
  LaunchLocalFn local;        // ADER + local integral, one launch
  LaunchNeighborFn neighbor;  // neighbour flux
  LaunchTaylorFn taylor;      // Taylor evaluation of stored derivatives
  LaunchLocalFn ader;         // ADER alone (writes I, optional derivatives)
  LaunchLintFn lint;          // volume + local flux from I
  LaunchTaylorGatherFn taylorGather;
  double flopAder, flopLocal, flopNeighbor;  // non-zero flops per cell
  LaunchLintFn lintVol;       // volume + face traces, no local flux (the neighbour kernel applies it)
  LaunchLocalFn localVol;     // ADER + volume + face traces, one launch (I stays on chip)
  // trace[4][tplane][9][FP] of the pool blocks blk[e], e < m (local time stepping)
  int (*traceBlocks)(int m, const int32_t* blk, const float* pool, float* trace, int tplane, void* stream);
};

// pool[dst[e]] = (reset ? 0 : pool[dst[e]]) + pool[cell[e]] for e < m, blocks of blk floats
// (integration buffers of local time stepping).
int launchLtsBuffer(int m, const int32_t* cell, const int32_t* dst, float* pool, int blk, int reset, void* stream);
// The same for face traces [4][plane][row] (row = 9 FP floats): all four faces of each entry.
int launchLtsTraceBuffer(int m, const int32_t* cell, const int32_t* dst, float* trace, int64_t plane, int row,
                         int reset, void* stream);

bool kernelsForOrder(int order, OrderKernels& out);

// Viscoelastic (27 quantities) device arrays; Q, I [n][27][Bp].
struct ViscoArrays {
  int n;
  float* Q;
  float* I;
  const float* star_nz;  // [n][3][24] elastic star non-zeros with the unrelaxed moduli
  const float* grad;     // [n][3][3]
  const float* theta;    // [n][3][3]
  const float* aplus;    // [n][4][81] elastic block
  const float* wplus;    // [n][4][54] memory block per unit omega
  const float* aminus;
  const float* wminus;
  const int32_t* nbr;
  const uint8_t* rel;
  const uint8_t* ftype;
  float omega[3];
  float* derivs = nullptr;         // nullable: ADER derivative output [slots][derivSize]
  const int32_t* dslot = nullptr;  // nullable: slot per cell (-1 none); nullptr = slot is the cell
};
struct ViscoKernels {
  int (*ader)(const ViscoArrays&, const float* coeffs, void* stream);
  int (*lint)(const ViscoArrays&, void* stream);
  int (*neighbor)(const ViscoArrays&, void* stream);
  int derivSize;  // floats of one cell's stored derivatives: order x 27 x B
};
// pool[dst[e]][nq][Bp] = sum_i coeffs[i] dQ(i) of derivative slot src[e] stored as [order][nq][B]
// (all basis rows at every stage), e < m; local time stepping of the viscoelastic equations.
int launchTaylorGatherFull(int m, const int32_t* src, const int32_t* dst, const float* derivs, int order, int nq, int b,
                           int bp, const float* coeffs, float* pool, void* stream);
bool viscoKernelsForOrder(int order, ViscoKernels& out);

}  // namespace sei

namespace sei {
// Device arguments of the dynamic-rupture face kernel (passed by value).
struct DrArgs {
  int nfaces;             // all faces (plane stride of the [field][nf][npts] arrays)
  const int32_t* fidx;    // nullable: faces processed are fidx[face_begin + i], else face_begin + i
  int face_begin, face_count;  // i < face_count
  const int32_t* plus_cell;
  const int32_t* minus_cell;
  const uint8_t* plus_side;
  const uint8_t* minus_side;
  const uint8_t* rel;  // minus-side face relation 1..3 (plus side uses 0)
  const int32_t* plus_slot;
  const int32_t* minus_slot;
  const float* derivs;  // [slots][derivativesSize]
  const float* tinvt;   // [nf][81] column-major
  const float* fsp;     // flux solvers [nf][81]
  const float* fsm;
  const double* imp;   // [nf][8]: zp, zs, zpn, zsn, etap, etas, inv_etas, unused
  const double* a;     // [nf][npts]
  double* init;        // [3][nf][npts]: sn0, tau1_0, tau2_0 (nucleation adds to them)
  double *psi, *v1, *v2, *slip1, *slip2, *slip, *mu, *trac1, *trac2;  // [nf][npts]
  float* isp;  // imposed states [nf][9][npts]
  float* ism;
  int32_t* newton_iters;  // [3][nf][npts], accumulated: float64 iterations of all solves, of the first
                          // solve of each time point, float32 pre-iterations of all solves
  float* Q;               // DOFs [n][9][Bp] (nodal flux target)
  double f0, b, v0, l, muw, vw, newton_tol, state_tol;
  int max_newton, max_outer;
  int refine32;         // 1: every solve iterates in float32 (log slip rate) before the float64 Newton
  double deltat[8], tweights[8];
  float coll[8][8];     // collocation coefficients t_s^p / p! of the time points
  const float* mlp;     // warm-start network parameters (nullptr: plain Newton)
  float mlp_norm[16];   // normalisation of the network (layout in mlp.cuh)
  float* rec;           // training samples [rec_cap][6] (nullptr: not recorded)
  unsigned* rec_count;
  unsigned rec_cap;
  // friction law (SEI_LAW_*): 0 rate and state with fast velocity weakening, 1 linear slip
  // weakening, 2 its bimaterial (Prakash-Clifton) form, 3 the TP proxy, 4-6 the aging, slip and
  // severe rate-and-state laws, 7-9 imposed slip rates (Yoffe, Gaussian, delta)
  int law;
  const double* time;  // device scalar: fault time at the start of the current step or LTS cycle
  double time_offset;  // start of this launch's step relative to *time
  double t0, s0;       // nucleation duration and start; t0 also ramps the forced rupture
  int nucleate;        // 1: nucleation stresses nuc [3][nf][npts] are added over [s0, s0 + t0]
  const double* nuc;
  double *peak, *trup, *tdyn;  // [nf][npts] peak slip rate, rupture and dynamic-stress times
  const double *mu_s, *mu_d, *d_c, *cohesion, *t_forced;  // slip weakening, [nf][npts]
  double* reg;                                            // regularised strength (law 2)
  double healing, v_star, prakash_length, tp_exponent;
  const double *dir1, *dir2, *onset, *taus, *taur;  // imposed slip rates, [nf][npts]
  // thermal pressurisation of the rate-and-state laws (tp = 1): constants, per-point shear-zone
  // half width and hydraulic diffusivity, Fourier modes of temperature and pressure [60][nf][npts],
  // temperature and pressure [nf][npts]
  int tp;
  double tp_alpha, tp_rhoc, tp_lambda, tp_t0, tp_p0;
  const double *tp_hw, *tp_hyd;
  double *tp_theta, *tp_sigma, *tp_temp, *tp_pres;
};
constexpr int kTpModes = 60;
// Fills the device tables of the thermal-pressurisation modes (wave numbers, inverse-transform
// weights, heat source); once per device.
int launchTpTables(void* stream);
// Adds dt to the device fault time t.
int launchDrAdvanceTime(double* t, double dt, void* stream);
int launchDrFaces(int order, const DrArgs& a, void* stream);
int drNumPoints(int order);
}  // namespace sei

namespace sei {
// Planar fault of a periodic cube: faces on the plane x = plane * h.  The plus side is the
// cell on the -x side (the reference point lies there), so the fault normal is +x
// (src/Geometry/MeshReader.cpp:160-200).
struct HostFault {
  int64_t nf = 0;
  std::vector<int32_t> plus_cell, minus_cell;
  std::vector<uint8_t> plus_side, minus_side, rel;  // rel = orientation of the plus side + 1
  std::vector<float> tinvt, fsp, fsm;               // [nf][81] column-major
  std::vector<double> imp;                          // [nf][8]
};
// Fault faces on the plane x = xf (one cube-vertex plane of the mesh; h is the length scale of
// the coordinate comparison).
void buildPlanarFault(HostMesh& m, double xf, double h, HostFault& f);
// Mesh from PUML arrays: cells, face relations, boundary conditions and the fault faces (plus
// side by the fault reference point).  Throws std::invalid_argument on bad input and
// std::domain_error on boundary conditions this build does not support.
void ingestMesh(const sei_mesh& p, HostMesh& m, HostFault& f);
void faultFaceData(const HostMesh& m, HostFault& f);
// Steady-state state variable of the fast-velocity-weakening law at slip rate v.
double fvwSteadyState(double v, double a, double b, double f0, double v0, double muw, double vw);
void gaussLegendre01(int n, double* x, double* w);
}  // namespace sei

namespace sei {
// Arguments of the tensor-core local-integral kernel.
struct TcLintArgs {
  int n;
  float* Q;
  const float* I;
  const float* star_nz;
  const float* aplus;
  const uint8_t* ftype;
  const uint16_t* opVol;  // pre-split FP16 operand tables (hi then lo), core-matrix layout
  const float* scVol;     // per-row power-of-two scales of the operand tables
  const uint16_t* opRd;
  const float* scRd;
  float* trace;   // nullable: face traces fMrT_f I out, [4][tplane][9][FP] (FP = F rounded up to 4)
  int tplane;     // cells per face plane of the traces (trace points at this launch's first cell)
  int traceOnly;  // 1: write the traces only (Q unchanged)
  int* status;    // set to 1 when a wait gave up
};
int launchLintTensorCore(int order, const DeviceArrays& d, float* trace, int traceOnly, int* status, int sms,
                         void* stream);

// Arguments of the tensor-core neighbour kernel (face traces in, Q updated in place).
struct TcNbArgs {
  int n;       // cells of this launch (Q, aminus, nbr, rel, ftype point at its first cell)
  int ntotal;  // cells of the mesh: face-plane stride of the traces, range of neighbour indices
  int first = 0;                  // mesh index of this launch's first cell (its own traces)
  const float* aplus = nullptr;   // non-null: also the local flux from the cell's own traces
  float* Q;
  const float* trace;  // [4][n][9][FP] traces fMrT_f I of every cell and face
  const float* aminus;
  const int32_t* nbr;
  const uint8_t* rel;
  const uint8_t* ftype;
  const uint16_t* opRd;  // pre-split rDivM stack (B operand), core-matrix layout
  const float* scRd;
  int* status;
};
// ctasPerSm: persistent CTAs per SM (1..3; 3 fit the shared memory at order 6)
int launchNeighborTensorCore(int order, const DeviceArrays& d, const float* trace, int* status, int sms, int ctasPerSm,
                             void* stream);
// Transposed tensor-core neighbour kernel (tc_nbt.cu): the same inputs and result as
// launchNeighborTensorCore, with the basis index on the TMEM lanes and the per-cell mixing in
// registers; two persistent CTAs per SM.
// withLocalFlux: also the local flux rDivM_i T_i A+_i from the cell's own stored traces (one lift
// for both fluxes; the local integral then ran as volume + traces, OrderKernels::lintVol).
int launchNeighborTransposed(int order, const DeviceArrays& d, const float* trace, int* status, int sms, void* stream,
                             bool withLocalFlux = false);
// Transposed tensor-core local integral (tc_lintt.cu): volume + local flux of launchLintTensorCore
// with the basis index on the TMEM lanes; writes the face traces (traceOnly: only them).
int launchLintTransposed(int order, const DeviceArrays& d, float* trace, int traceOnly, int* status, int sms,
                         void* stream);
// Diagnostic: one warp's bounded mbarrier wait that gives up (arrive = 0) or completes (arrive = 1).
int launchWaitProbe(uint32_t polls, int arrive, int* status, void* stream);
// Floats per cell of the face-trace array of the tensor-core path: 4 faces x 9 quantities x FP.
inline int traceFloatsPerCell(int order) { return 4 * 9 * ((numFaceBasis(order) + 3) / 4 * 4); }
}  // namespace sei

namespace sei {
// Warm-start network kernels (mlp_kernels.cu).
int mlpNumParams();
int launchMlpGrad(const float* P, const float* norm, const float* X, const float* T, int n, float* grads, float* loss,
                  int sms, void* stream);
int launchMlpAdam(float* P, const float* grads, float* m, float* v, float lr, int step, void* stream);
int launchMlpPredict(const float* P, const float* norm, const float* X, int n, float* out, void* stream);
}  // namespace sei

namespace sei {
// Off-fault plasticity (plasticity.cu): the nodal Drucker-Prager check and viscoplastic return map
// of Plasticity.cpp:47-214 on cells [begin, end) after their neighbour integral.
struct PlasticityArgs {
  float* Q;                   // DOFs [cells][9][Bp] (stresses: quantities 0..5)
  const float* mats;          // V [B][Bp] (basis values at the nodes) then Vinv [B][Bp]
  // per-node arrays tiled by 32 cells: [cells / 32][K][B][32] (cell c: tile c / 32, lane c % 32)
  const float* s0;            // initial loading, K = 6
  const float* ccos;          // cohesion cos(phi), K = 1
  const float* ssin;          // sin(phi), K = 1
  const float* mufac;         // 1 / (2 mu) [cells]
  float* pstrain;             // plastic strain, K = 7 (six components, then eta)
  unsigned long long* yield;  // cells with yielding, accumulated
  int64_t begin, end;
  float relax;     // r = 1 - exp(-dt / T_v)
  float inv_tvr;   // 1 / (T_v r)
  float dt;
};
int launchPlasticity(int order, const PlasticityArgs& a, void* stream);
// V [B][B] (phi_k at node n) and its inverse, float64, from reference-element nodes [B][3];
// false when the nodes are not unisolvent.
bool plasticityMatrices(int order, const double* nodes, std::vector<double>& v, std::vector<double>& vinv);
// The equispaced lattice of degree order - 1 on the reference tetrahedron: B nodes [B][3].
void latticeNodes(int order, double* nodes);
}  // namespace sei
