/*
 * sei_gb300 — C ABI of the GB300 ADER-DG element update.
 *
 * One context owns one CUDA device's data for one mesh: DOFs, time-integrated DOFs,
 * per-cell operators and neighbour relations, all resident in HBM.  Host arrays passed
 * in are copied and never retained; arrays passed out are owned by the caller.
 * Every function returns SEI_OK (0) or a negative SEI_ERR_* code and never aborts;
 * sei_last_error() describes the last failure.  A context is not thread-safe: use one
 * per host thread.  All device work runs on the context's own CUDA stream.
 *
 * Layouts (the reference's yateto column-major convention):
 *   DOF tensors   [ncells][9][B]   basis index fastest, B = order(order+1)(order+2)/6
 *   9x9 operators column-major, element (q, p) at q + 9 p
 *   star          [ncells][3][81]  (src/Initializer/Typedefs.h:187-196 starMatrices)
 *   aplus/aminus  [ncells][4][81]  (nApNm1 / nAmNm1, src/Initializer/Typedefs.h:187-205)
 *   neighbor      [ncells][4] int32 cell id or -1, side/orient [ncells][4] int8
 *                 (CellLocalInformation::faceRelations, src/Initializer/Typedefs.h:221-233)
 *   face_type     [ncells][4] int8: 0 regular, 1 dynamic rupture, 2 none (boundary)
 */
#ifndef SEI_GB300_H_
#define SEI_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEI_OK 0
#define SEI_ERR_ARG (-1)
#define SEI_ERR_OOM (-2)
#define SEI_ERR_CUDA (-3)
#define SEI_ERR_TIMEOUT (-4)
#define SEI_ERR_NAN (-5)
#define SEI_ERR_STATE (-6)
#define SEI_ERR_UNSUPPORTED (-7)
#define SEI_ERR_CAPACITY (-8) /* request larger than a fixed-size buffer of the library */

/* Proxy kernels (src/Proxy/Common.h:18, names in src/Proxy/Common.cpp:22-40). */
#define SEI_KERNEL_ALL 0
#define SEI_KERNEL_LOCAL 1
#define SEI_KERNEL_NEIGHBOR 2
#define SEI_KERNEL_ADER 3
#define SEI_KERNEL_LOCAL_WO_ADER 4
#define SEI_KERNEL_NEIGHBOR_DR 5
#define SEI_KERNEL_GODUNOV_DR 6
#define SEI_KERNEL_ALL_DR 7

/* Arithmetic of the global-matrix contractions. */
#define SEI_PREC_FP32 0 /* CUDA-core FP32, sparse (non-zero flops only) */
/* Mixed precision: global-matrix contractions on the tensor cores (tcgen05 kind::f16), each
 * product split into three FP16 products (hi*hi + hi*lo + lo*hi) of power-of-two row-scaled
 * operands with FP32 accumulation; everything else FP32.  The neighbour flux always runs on the
 * tensor cores, from the face traces of I that the local integral stores; by default
 * (SEI_OPT_NB_FORM 2) the local flux of a step of kernel 'all' runs there too, from the cell's
 * own traces, and the local integral keeps the volume term (FP32 CUDA cores; the tensor cores
 * with SEI_OPT_TC_LOCAL 1 or 2, then with the local flux). */
#define SEI_PREC_F16X3 1

typedef struct sei_ctx sei_ctx;

typedef struct sei_config {
  int order;     /* convergence order: 4, 5 or 6 */
  int device;    /* CUDA device ordinal */
  int precision; /* SEI_PREC_* */
  int store_derivatives; /* keep the CK derivatives of every cell (needed by dynamic rupture) */
} sei_config;

/* Synthetic periodic cube: nx*ny*nz cubes of edge h, 5 tetrahedra each (even counts >= 4).
 * Material rho, vp, vs, each multiplied per cell by U[1-perturb, 1+perturb] (seeded).
 * fault_plane in 1..nx-1 turns the faces on cube-vertex plane fault_plane along x (x =
 * fault_plane * h on a uniform cube) into a planar vertical dynamic-rupture fault (plus side at
 * smaller x); -1 builds no fault. */
typedef struct sei_cube_params {
  int nx, ny, nz;
  double h;
  double rho, vp, vs;
  double perturb;
  uint64_t seed;
  int fault_plane;
  /* > 1: graded tensor-product cube; along each direction the cube edges are drawn
   * log-uniformly in [h, grading h] (seeded); <= 1: uniform edge h.  The fault lies on the
   * cube-vertex plane fault_plane along x (x = fault_plane h when uniform). */
  double grading;
  /* 1 (with grading >= 8): the local-time-stepping profile of the graded mesh instead: only the
   * edges along the direction with the most intervals (x on ties) vary, in four bands of edge
   * 1, 2.736, 5.98 and 14.7 h on 60 / 25 / 10 / 5 % of its intervals, rising and falling once so
   * that neighbouring cells lie in the same or adjacent bands; the other edges are 32 h.  The
   * band edges put every tet's CFL step (inradius about (w / 2) / (1 + w / 32 h) for edge w, wave
   * speeds +-10 %) into octave b of the smallest, so rate-2 clustering gives four clusters of
   * about those shares.  0: as described for grading. */
  int lts_profile;
} sei_cube_params;

/* Fast-velocity-weakening rate-and-state friction (src/Initializer/Parameters/DRParameters.h:36-73,
 * names of the reference: rs_f0, rs_b, rs_sr0, rs_sl0, rs_muw, rs_srW) with the seeded initial
 * state of the synthetic fault: a ~ U[a_min, a_max] per point, normal stress ~ U[sn_min, sn_max]
 * (negative = compression), shear traction (along tangent 1) ~ U[tau_min, tau_max], slip rate
 * v_init, state variable at steady state for v_init.  Newton: max_newton updates, tolerance
 * newton_tol on |g|; fixed point: max_outer passes, tolerance state_tol on the slip-rate change
 * (reference defaults 60, 1e-8, 10, 1e-8). */
typedef struct sei_rs_params {
  double f0, b, v0, l, muw, vw;
  double a_min, a_max, sn_min, sn_max, tau_min, tau_max, v_init;
  double newton_tol, state_tol;
  int max_newton, max_outer;
  uint64_t seed;
} sei_rs_params;

/* Friction-state fields for sei_dr_get_state. */
#define SEI_DR_PSI 0
#define SEI_DR_SLIP_RATE1 1
#define SEI_DR_SLIP_RATE2 2
#define SEI_DR_SLIP1 3
#define SEI_DR_SLIP2 4
#define SEI_DR_SLIP 5
#define SEI_DR_MU 6
#define SEI_DR_TRACTION1 7
#define SEI_DR_TRACTION2 8
#define SEI_DR_A 9
#define SEI_DR_SN0 10
#define SEI_DR_TAU1_0 11
#define SEI_DR_TAU2_0 12
/* Linear slip weakening (sei_dr_setup_lsw): static and dynamic friction coefficients, critical slip
 * distance, cohesion, forced rupture time (LTSLinearSlipWeakening, MuS .. ForcedRuptureTime). */
#define SEI_DR_MU_S 13
#define SEI_DR_MU_D 14
#define SEI_DR_D_C 15
#define SEI_DR_COHESION 16
#define SEI_DR_FORCED_RUPTURE_TIME 17
/* Outputs of both laws (BaseFrictionLaw.h:127-134): peak slip rate, rupture time (slip rate above
 * 1e-3 m/s for the first time) and, slip weakening only, dynamic stress time (accumulated slip
 * reaches d_c); a time is the start of the time point and is negative while pending. */
#define SEI_DR_PEAK_SLIP_RATE 18
#define SEI_DR_RUPTURE_TIME 19
#define SEI_DR_DYN_STRESS_TIME 20
/* Nucleation stresses added to sn0, tau1_0, tau2_0 over [s0, s0 + t0] (sei_dr_set_nucleation). */
#define SEI_DR_NUC_SN 21
#define SEI_DR_NUC_TAU1 22
#define SEI_DR_NUC_TAU2 23
/* Regularised strength of the bimaterial law (LTSLinearSlipWeakeningBimaterial::RegularizedStrength). */
#define SEI_DR_REG_STRENGTH 24
/* Imposed slip rates (sei_dr_setup_imposed): slip direction (along tangent 1 and 2), onset time,
 * and the source time function's tau_S and tau_R (Yoffe) or rise time (SEI_DR_TAU_S, Gaussian). */
#define SEI_DR_SLIP_DIR1 25
#define SEI_DR_SLIP_DIR2 26
#define SEI_DR_ONSET_TIME 27
#define SEI_DR_TAU_S 28
#define SEI_DR_TAU_R 29
/* Thermal pressurisation (sei_dr_set_thermal_pressurization): shear-zone half width, hydraulic
 * diffusivity (tp_halfwidthshearzone, tp_hydraulicdiffusivity), temperature and pore pressure. */
#define SEI_DR_TP_HALF_WIDTH 30
#define SEI_DR_TP_HYDRAULIC_DIFFUSIVITY 31
#define SEI_DR_TP_TEMPERATURE 32
#define SEI_DR_TP_PRESSURE 33
#define SEI_DR_NUM_FIELDS 34

/* Thermal pressurisation of the rate-and-state laws (CpuImpl/ThermalPressurization/
 * ThermalPressurization.cpp, TPCommon.h): per point, 60 Fourier modes of temperature and pore
 * pressure across the shear zone diffuse and gain the frictional heat tau V of a Gaussian source;
 * the pore pressure lowers the effective normal stress in every pass of the slip-rate solve and
 * the modes advance after it (RateAndState.h:40-76, 185-215, 420-432).  Parameter names of the
 * reference: tp_thermaldiffusivity, tp_heatcapacity, tp_undrainedtpresponse, tp_initemp,
 * tp_inipressure; the per-point fields start at half_width_shear_zone and hydraulic_diffusivity. */
typedef struct sei_tp_params {
  double thermal_diffusivity, heat_capacity, undrained_tp_response;
  double initial_temperature, initial_pressure;
  double half_width_shear_zone, hydraulic_diffusivity;
} sei_tp_params;

/* Friction laws (src/Initializer/Parameters/DRParameters.h FrictionLawType): rate and state with
 * fast velocity weakening (FL 103, sei_dr_setup); linear slip weakening (FL 16 and FL 2), its
 * bimaterial form with the Prakash-Clifton regularised strength (FL 6) and the thermal-pressurisation
 * proxy (FL 1058), all three with sei_dr_setup_lsw. */
#define SEI_LAW_FVW 0
#define SEI_LAW_LSW 1
#define SEI_LAW_LSW_BIMATERIAL 2
#define SEI_LAW_LSW_TP_PROXY 3
#define SEI_LAW_RS_AGING 4  /* FL 3: rate and state, aging law (CpuImpl/AgingLaw.h) */
#define SEI_LAW_RS_SLIP 5   /* FL 4: rate and state, slip law (CpuImpl/SlipLaw.h) */
#define SEI_LAW_RS_SEVERE 6 /* FL 7: severe velocity weakening (CpuImpl/SevereVelocityWeakeningLaw.h) */
#define SEI_LAW_ISR_YOFFE 7    /* FL 33: imposed slip rate, regularised Yoffe function */
#define SEI_LAW_ISR_GAUSSIAN 8 /* FL 34: imposed slip rate, Gaussian (smooth step) */
#define SEI_LAW_ISR_DELTA 9    /* FL 35: imposed slip rate, delta pulse */

/* Imposed slip rates (CpuImpl/ImposedSlipRates.h, SourceTimeFunction.cpp): the slip rate is the
 * slip direction times the source time function at the end of each time point; the traction is
 * the fault stress minus eta_s times the slip rate.  Per-point fields start uniform (direction,
 * onset time, tau_s, tau_r; the Gaussian's rise time is tau_s) with initial stresses sn0, tau1_0. */
typedef struct sei_isr_params {
  int law;
  double slip_dir1, slip_dir2;
  double onset_time, tau_s, tau_r;
  double sn0, tau1_0;
} sei_isr_params;

/* Linear-slip-weakening parameters: per-point fields start uniform (mu_s, mu_d, d_c, cohesion,
 * forced_rupture_time) or seeded uniform random (sn0 in [sn_min, sn_max] <= 0, tau1_0 in
 * [tau_min, tau_max], tau2_0 = 0), all settable per point with sei_dr_set_state.  t0 is t_0 of the
 * parameter file: the ramp of the forced rupture (0: a step at the forced rupture time) and the
 * nucleation duration; healing_threshold is lsw_healingthreshold (-1: no healing); v_star and
 * prakash_length the Prakash-Clifton constants (pc_vstar, pc_prakashlength; law 2);
 * tp_proxy_exponent tpproxyexponent (law 3; reference default 1/3). */
typedef struct sei_lsw_params {
  int law;
  double mu_s, mu_d, d_c, cohesion;
  double sn_min, sn_max, tau_min, tau_max;
  double forced_rupture_time;
  double t0;
  double healing_threshold;
  double v_star, prakash_length;
  double tp_proxy_exponent;
  uint64_t seed;
} sei_lsw_params;

/* PerformanceEstimate of the reference (src/Monitoring/Metric.h:8-60), per cell and step. */
typedef struct sei_perf {
  double nonzero_flop;  /* executed non-zero flops */
  double hardware_flop; /* flops issued by the kernels */
  double bytes;         /* algorithmic HBM bytes (compulsory traffic) */
} sei_perf;

int sei_version(void);

/* Replaces setGlobalData + storage allocation (src/Kernels/Kernel.h:18, src/Proxy/Allocator.cpp:137-144).
 * cfg->device < 0 makes a host-only context: mesh/operator set-up and the sei_get_* copies of it,
 * no CUDA calls (used to check the set-up on machines without a GPU). */
int sei_create(const sei_config* cfg, sei_ctx** out);
void sei_destroy(sei_ctx* ctx);
const char* sei_last_error(const sei_ctx* ctx);

/* Builds the synthetic periodic cube on the host (geometry, face relations, materials,
 * star matrices and flux solvers as src/Initializer/Model/CellLocalMatrices.cpp:66-296),
 * uploads it and seeds the DOFs U[-1, 1].  Returns the cell count. */
int sei_build_periodic_cube(sei_ctx* ctx, const sei_cube_params* p, int64_t* ncells);

/* ---- mesh ingestion: the arrays of a PUML mesh (docs/puml-mesh-format.rst, read by
 * src/Geometry/PUMLReader.cpp; the HDF5 file itself is read by the caller) ----
 * Boundary formats: i32 (one uint32 per cell, 8 bits per face), i64 (one uint64 per cell, 16 bits
 * per face), i32x4 (one int32 per face).  Boundary conditions (default face map,
 * src/Initializer/FaceMap.cpp:100-110): 0 and 6 regular; 3 and above 64 dynamic rupture;
 * 1 free surface and 5 outflow (absorbing), both without a neighbour flux, the free surface with
 * the free-surface Godunov state in its local flux (src/Model/Common.h:319-364); 2 (gravity free
 * surface), 4 (Dirichlet) and 7 (analytical) return SEI_ERR_UNSUPPORTED.
 * Fault plus side (src/Geometry/MeshReader.cpp:150-170): SEI_FAULT_REF_POINT, the cell on the
 * reference point's side of the face; SEI_FAULT_REF_NORMAL, the cell whose outward face normal
 * has a positive dot product with the reference vector. */
#define SEI_BOUNDARY_I32 0
#define SEI_BOUNDARY_I64 1
#define SEI_BOUNDARY_I32X4 2
#define SEI_FAULT_REF_POINT 0
#define SEI_FAULT_REF_NORMAL 1
typedef struct sei_mesh {
  int64_t nvertices;
  const double* geometry;  /* [nvertices][3] */
  int64_t ncells;
  const int64_t* connect;  /* [ncells][4] vertex ids, every tetrahedron positively oriented */
  const void* boundary;    /* per boundary_format; NULL: every face regular */
  int boundary_format;
  const int64_t* identify; /* topology format identify-vertex: [nvertices] topological vertex of each
                              vertex (periodic or stitched meshes); NULL: geometric topology */
  const double* material;  /* [ncells][3] rho, mu, lambda (the caller's material model per cell) */
  double fault_ref[3];
  int fault_ref_method;
} sei_mesh;
/* Builds cells, face relations, operators and the fault faces of a PUML mesh, uploads them and
 * zeroes the DOFs; *ncells and *nfaults (either may be NULL) receive the cell and fault-face counts.
 * A rejected mesh changes nothing.  Cells may have several fault faces.  A fault is set up with
 * sei_dr_setup or sei_dr_setup_lsw as on the synthetic cube. */
int sei_set_mesh(sei_ctx* ctx, const sei_mesh* mesh, int64_t* ncells, int64_t* nfaults);

/* Generic mesh upload (drop-in for the LTS storage of one layer). */
int sei_set_cells(sei_ctx* ctx, int64_t ncells, const float* star, const float* aplus, const float* aminus,
                  const int32_t* neighbor, const int8_t* side, const int8_t* orient, const int8_t* face_type);
int64_t sei_num_cells(const sei_ctx* ctx);

/* Host copies of what sei_build_periodic_cube or sei_set_mesh made (for checking against independent set-ups). */
int sei_get_cells(sei_ctx* ctx, float* star, float* aplus, float* aminus, int32_t* neighbor, int8_t* side,
                  int8_t* orient, int8_t* face_type);
int sei_get_geometry(sei_ctx* ctx, double* vertices /*[n][4][3]*/, double* material /*[n][3] rho, mu, lambda*/,
                     int64_t* topology /*[n][4] vertex ids*/);
/* Smallest CFL time step of the mesh (src/Initializer/TimeStepping/GlobalTimestep.cpp:27-47). */
int sei_cfl_timestep(sei_ctx* ctx, double cfl, double* dt);

int sei_set_dofs(sei_ctx* ctx, const float* dofs);
int sei_get_dofs(sei_ctx* ctx, float* dofs);
int sei_get_time_integrated(sei_ctx* ctx, float* tint);
/* Stored CK derivatives: [n][size] with store_derivatives, or [slots][size] by fault slot after sei_dr_setup (one
 * slot per fault cell, sei_dr_get_slots; 2 nfaces when no cell has two fault faces). */
int sei_get_derivatives(sei_ctx* ctx, float* derivs);
int sei_derivatives_size(int order);

/* Spacetime::computeAder / computeBatchedAder (src/Kernels/Spacetime.h:52-67,
 * src/Kernels/LinearCK/Time.cpp:142-217) for all cells: I = sum_i coeffs[i] dQ_i, with coeffs[order]
 * the time-basis coefficients of the integration interval, as the reference's caller passes them
 * (a TimeCluster passes MonomialBasis::integrate(0, dt), or the sub-interval of a local time step);
 * coeffs = NULL takes MonomialBasis::integrate(0, dt) (src/Numerical/TimeBasis.h:82-93).  The
 * global matrices (the reference's setGlobalData, src/Kernels/Kernel.h:18) are compiled into the
 * kernels, so no global-data call exists. */
int sei_compute_ader(sei_ctx* ctx, const double* coeffs, double dt);
/* Local::computeBatchedIntegral (src/Kernels/LinearCK/Local.cpp:255-395): volume + local flux from the
 * time-integrated DOFs of the last sei_compute_ader. */
int sei_compute_local_integral(sei_ctx* ctx);
/* ADER followed by the local integral in one launch (src/Proxy/KernelHost.cpp:108-131). */
int sei_compute_ader_local(sei_ctx* ctx, double dt);
/* Neighbor::computeBatchedNeighborsIntegral (src/Kernels/LinearCK/Neighbor.cpp:111-188). */
int sei_compute_neighbors_integral(sei_ctx* ctx);
/* Time::evaluateBatched (src/Kernels/LinearCK/Time.cpp:256-292) of the stored derivatives. */
int sei_evaluate_taylor(sei_ctx* ctx, const double* coeffs, float* out_device);

/* Options. SEI_OPT_FUSED_LOCAL: 1 runs ADER and the local integral as one launch, 0 (default)
 * as two launches (smaller kernels; I is written and re-read once). */
#define SEI_OPT_FUSED_LOCAL 1
/* SEI_OPT_LTS_GRAPH: 1 records one local-time-stepping cycle as a CUDA graph on the first
 * sei_lts_run and replays it for every cycle (one graph launch per cycle); 0 (default) launches
 * the kernels of every cycle directly.  Per-launch profiling is not recorded inside the graph. */
#define SEI_OPT_LTS_GRAPH 2
/* SEI_OPT_TC_LOCAL (SEI_PREC_F16X3 only): where the local integral (volume + local flux, which also
 * stores the face traces) runs: 0 (default) FP32 CUDA cores; 1 tensor cores, transposed (the basis
 * index on the TMEM lanes, a tile's (cell, quantity) pairs on the MMA columns, the per-cell 9 x 9
 * mixing in registers); 2 tensor cores, rows form (a tile's rows (cell, quantity) on the lanes). */
#define SEI_OPT_TC_LOCAL 3
/* SEI_OPT_NB_CTAS (SEI_PREC_F16X3 only): persistent CTAs per SM of the rows-form tensor-core
 * neighbour kernel, 1..3 (default 3). */
#define SEI_OPT_NB_CTAS 4
/* SEI_OPT_NB_FORM (SEI_PREC_F16X3 only): layout of the tensor-core neighbour flux.  1,
 * transposed: the basis index on the TMEM lanes and a tile's (quantity, cell) pairs on the MMA
 * columns, so the per-cell 9 x 9 mixing stays in registers; 0, rows: a tile's (cell, quantity)
 * rows on the lanes, the mixing through shared memory; 2 (default): transposed, and in a step of
 * kernel 'all' (or 'all_dr', or a local-time-stepping cycle) the local flux of every face joins
 * the neighbour flux before their common lift rDivM_i (the local integral then computes the
 * volume term and the face traces only; SEI_OPT_TC_LOCAL 0).  The separate local-integral and
 * neighbour calls keep their full meaning.  Under local time stepping the transposed form is
 * used for 0 too. */
#define SEI_OPT_NB_FORM 5
/* SEI_OPT_DR_REFINE32: 1 makes every slip-rate solve of the fault kernel first iterate in float32
 * on ln V from its start (the previous slip rate, or the network's guess on a first solve with
 * the warm start on) until the step falls below 2e-6, then run the float64 Newton of the
 * reference from there with the reference's tolerance (it falls back to the plain start if its
 * residual stops falling), so the converged slip rates are those of the plain solve to within the
 * Newton tolerance.  No counterpart in the reference; float64 is the scarce pipe of GB300.
 * 0 (default): the float64 Newton alone. */
#define SEI_OPT_DR_REFINE32 6
/* SEI_OPT_TUNE_FAIL_AT (tests only): sei_autotune fails on the host at candidate `value` (after its
 * warm-up step, before its timing), as a variant whose launch failed would; -1 (default): never. */
#define SEI_OPT_TUNE_FAIL_AT 7
int sei_set_option(sei_ctx* ctx, int option, int value);
/* The current value of an option (SEI_ERR_ARG for an unknown one). */
int sei_get_option(sei_ctx* ctx, int option, int* value);

/* Autotuner (no counterpart in the reference, whose kernel shapes are fixed when its code is
 * generated): times `steps` steps of kernel 'all' on the context's own mesh for every variant of
 * the step this library has: SEI_OPT_FUSED_LOCAL 0/1 at SEI_PREC_FP32; SEI_OPT_TC_LOCAL 0/1/2 x
 * (SEI_OPT_NB_FORM 1, or SEI_OPT_NB_FORM 0 with SEI_OPT_NB_CTAS 1..3) at SEI_PREC_F16X3.  It keeps the fastest variant as the context's options.
 * The DOFs are restored after every variant, so the call leaves the state unchanged.  Global
 * stepping of the elastic kernels only (SEI_ERR_UNSUPPORTED after sei_visco_setup or
 * sei_lts_setup).  Synchronous. */
typedef struct sei_tune_result {
  int fused_local, tc_local, nb_ctas, nb_form; /* chosen options */
  int candidates;                     /* variants timed */
  double best_ms, worst_ms;           /* per step, fastest and slowest variant */
} sei_tune_result;
int sei_autotune(sei_ctx* ctx, double dt, int steps, sei_tune_result* out);

/* Runs a proxy kernel for nsteps steps (src/Proxy/Runner.cpp:99-111); asynchronous. */
int sei_run(sei_ctx* ctx, int kernel, double dt, int nsteps);
/* Same with host buffers: copies dofs_in to the device, runs, copies the result to dofs_out;
 * synchronous.  Kernel 'all' on global steps is pipelined in chunks of cells: the copies in
 * overlap ADER and the local integral, the copies out overlap the last neighbour flux. */
int sei_run_host(sei_ctx* ctx, int kernel, double dt, int nsteps, const float* dofs_in, float* dofs_out);
int sei_sync(sei_ctx* ctx);
/* Device-side duration of the last sei_run, milliseconds (CUDA events on the context stream). */
int sei_last_run_ms(sei_ctx* ctx, double* ms);

/* Viscoelastic equations with 3 attenuation mechanisms (the reference's `viscoelastic`
 * equations, codegen/kernels/equations/viscoelastic.py: 9 elastic quantities + 6 memory
 * variables per mechanism = 27; set-up of src/Equations/viscoelastic/Model/ViscoelasticSetup.h
 * and src/Physics/Attenuation.h).  Turns the context's mesh viscoelastic: the cells' moduli
 * (relaxed, from the mesh) are fitted to quality factors qp, qs over the band around
 * freq_central with freq_ratio (unrelaxed moduli, relaxation frequencies, theta); Q and I
 * become [n][27][Bp] (elastic DOFs kept, memory variables zero); sei_run then runs the
 * viscoelastic ADER (with the source term), local and neighbour kernels for SEI_KERNEL_ALL,
 * LOCAL, ADER, LOCAL_WO_ADER and NEIGHBOR, on global time steps or, after sei_lts_setup, with
 * rate-2 local time stepping.  Orders 4 and 5, FP32, no fault. */
int sei_visco_setup(sei_ctx* ctx, double qp, double qs, double freq_central, double freq_ratio);
/* Quantities per cell of the DOF arrays (9, or 27 after sei_visco_setup). */
int sei_num_quantities(const sei_ctx* ctx);
/* Operators of the viscoelastic set-up (also on a host-only context): grad [n][3][3] (d xi_e / d x),
 * theta [n][3][3], the memory-variable flux blocks wplus / wminus [n][4][9 x 6 column-major] per
 * unit omega (the flux solvers' memory columns of mechanism l are omega_l w), omega [3]. */
int sei_visco_operators(sei_ctx* ctx, float* grad, float* theta, float* wplus, float* wminus, double* omega);
/* The attenuation fit of one material (src/Physics/Attenuation.h:24-104): mu, lam relaxed in,
 * unrelaxed out; omega [3], theta [3][3] (mechanism-major). */
int sei_fit_attenuation(double qp, double qs, double freq_central, double freq_ratio, double* mu, double* lam,
                        double* omega, double* theta);

/* Local time stepping, rate 2 (replaces the clustering of src/Initializer/TimeStepping with the
 * maximum-difference property of docs/local-timestepping.rst, the predict / correct order of
 * src/Solver/TimeStepping/TimeCluster.cpp:358-440, 695-717 and TimeCommon::computeIntegrals,
 * src/Kernels/TimeCommon.cpp:40-87).  sei_lts_setup clusters the cells of the context's mesh by
 * their CFL time steps (cluster k: steps in [2^k dt0, 2^{k+1} dt0), at most max_clusters,
 * neighbours at most one cluster apart) and reorders the cells by cluster (stable; the DOFs move
 * with their cells; sei_lts_permutation gives new -> old).  A face reads its neighbour's
 * time-integrated DOFs (same cluster), integration buffer (finer neighbour) or the Taylor integral
 * of its derivatives over the sub-interval (coarser neighbour).  With a fault (sei_dr_setup
 * first; a fault cannot be set up after this call) both cells of every fault face share one
 * cluster, the lower, and each cluster's correction runs the fault step of its faces over its own
 * time step before its neighbour flux (TimeCluster.cpp:804-823). */
int sei_lts_setup(sei_ctx* ctx, double cfl, int max_clusters, int* nclusters);
/* Advances every cluster by dt0 2^(nclusters-1) per cycle (asynchronous; sei_last_run_ms times it). */
int sei_lts_run(sei_ctx* ctx, int ncycles);
/* Cluster k holds cells [start[k], start[k+1]) with time step dt[k] (start: nclusters + 1 entries). */
int sei_lts_clusters(sei_ctx* ctx, int* nclusters, int64_t* start, double* dt);
int sei_lts_permutation(sei_ctx* ctx, int64_t* perm /*[n]*/);

/* ---- output: receivers and fault snapshots, staged to the host asynchronously ----
 * Receivers (src/Kernels/Receiver.cpp:118-214, src/ResultWriter/ReceiverWriter.cpp): at the start
 * of every full step (kernels all and all_dr of sei_run) the CK derivatives of the receiver cells
 * give the solution at each sampling time inside the step, projected onto the basis functions at
 * the receiver point; rotation and strain come from the basis gradients (Receiver.cpp:271-302).
 * sei_receivers_setup locates the points (the lowest cell id among the cells that contain a point;
 * a point outside the mesh is an error), keeps the quantities of quantity_mask (bit q: quantity q of
 * xx, yy, zz, xy, yz, xz, u, v, w) and the derived ones of `derived`, and samples at sim_time,
 * sim_time + interval, ... (sei_get_time).  n = 0 removes the receivers.  Rows are staged on the
 * device and copied to pinned host memory on their own stream while the next steps run;
 * sei_receivers_read waits for the copies and returns up to max_samples samples, oldest first,
 * as [samples][receivers][columns]: time, the kept quantities, rot1-3, then eps_xx, eps_xy,
 * eps_xz, eps_yy, eps_yz, eps_zz.  Under local time stepping each cluster samples its receivers at
 * the start of each of its own steps (the times are the same sequence for all); a sample is
 * returned once every receiver has it, and cycles run without graph replay while receivers are
 * set.  sei_lts_setup locates existing receivers again on the reordered cells and restarts their
 * clocks.  With the viscoelastic equations the receivers give the nine elastic quantities (the
 * quantity mask covers those); set them up after sei_visco_setup.  A new mesh removes the
 * receivers. */
#define SEI_RECV_ROTATION 1
#define SEI_RECV_STRAIN 2
int sei_receivers_setup(sei_ctx* ctx, int64_t n, const double* xyz /*[n][3]*/, double interval, unsigned quantity_mask,
                        int derived, int64_t* cells /*[n] containing cell, may be NULL*/);
int sei_receivers_columns(const sei_ctx* ctx);
/* Basis functions phi [B] (B = order (order + 1) (order + 2) / 6, the reference ordering) and their
 * derivatives dphi [3][B] along xi, eta, zeta at reference point xez, as a receiver samples them
 * (src/Numerical/BasisFunction.h SampledBasisFunctions, SampledBasisFunctionDerivatives);
 * context-free, host only; dphi may be NULL.  Orders 1 to 8. */
int sei_basis_functions(int order, const double* xez /*[3]*/, double* phi, double* dphi);
int sei_receivers_read(sei_ctx* ctx, double* out, int64_t max_samples, int64_t* nsamples);

/* Off-fault plasticity (Drucker-Prager, viscoplastic relaxation), applied to every cell after its
 * neighbour integral in each full step (kernels all and all_dr, sei_run_host, every LTS cluster
 * step with the cluster's dt), as TimeCluster::computeNeighboringIntegration does
 * (src/Solver/TimeStepping/TimeCluster.cpp:966-975).  Replaces Plasticity::computePlasticity /
 * computePlasticityBatched (src/Kernels/Plasticity.cpp:47-238) and the PlasticityData set-up
 * (src/Model/Plasticity.h:28-59).
 * nodes: the B nodes [B][3] of the nodal basis on the reference tetrahedron (the vNodes of the
 * reference's plasticity-nb-matrices-<order>.json); V and its inverse are formed from the basis
 * functions at them.  NULL: the equispaced lattice of sei_plasticity_nodes (not the reference's
 * node set: results then differ from the reference's).  tv: relaxation time T_v > 0.
 * per_node 0: bulk_friction [n], plast_co [n] (cohesion), s0 [n][6] (initial stress xx, yy, zz, xy,
 * yz, xz) per cell; per_node 1: [n][B], [n][B], [n][B][6] per node.  The material's mu gives
 * 1 / (2 mu).  Elastic equations, orders 4-6; a new set-up resets the plastic strain.
 * sei_plasticity_get_strain: [n][7][B] nodal plastic strain (xx, yy, zz, xy, yz, xz) and eta.
 * sei_plasticity_yield_count: cell updates with yielding since the set-up (the reference's
 * numberOfTetsWithPlasticYielding summed over steps). */
int sei_plasticity_setup(sei_ctx* ctx, const double* nodes, double tv, const double* bulk_friction,
                         const double* plast_co, const double* s0, int per_node);
int sei_plasticity_disable(sei_ctx* ctx);
int sei_plasticity_get_strain(sei_ctx* ctx, float* out);
int sei_plasticity_yield_count(sei_ctx* ctx, int64_t* count);
/* 1 - exp(-dt / tv), or 1 for tv <= 0 (Plasticity::computeRelaxTime, src/Kernels/Plasticity.h:27-29). */
double sei_plasticity_relax_factor(double tv, double dt);
/* The equispaced lattice of degree order - 1: B nodes [B][3] (i, j, k) / (order - 1), i fastest. */
int sei_plasticity_nodes(int order, double* nodes);
/* Simulation time: the start of the next full step; advanced by dt per full step (by the cycle
 * length per LTS cycle).  sei_set_time restarts the receivers' sampling at t (unread samples are
 * dropped). */
int sei_get_time(const sei_ctx* ctx, double* t);
int sei_set_time(sei_ctx* ctx, double t);
/* Fault snapshots (the raw per-point counterpart of src/DynamicRupture/Output): after every
 * `every`-th full step, the fault time and the given fields (SEI_DR_*, each [nf][npts]) are copied on
 * the device into a staging ring and from there to pinned host memory on their own stream.
 * sei_fault_output_read returns up to max_snapshots snapshots, oldest first, each
 * 1 + nfields nf npts doubles.  every = 0 turns it off; a new fault set-up turns it off. */
int sei_fault_output_setup(sei_ctx* ctx, int every, const int* fields, int nfields);
int sei_fault_output_read(sei_ctx* ctx, double* out, int64_t max_snapshots, int64_t* nsnapshots);

/* ---- dynamic rupture (built with fault_plane >= 0; orders 4-6: (order + 1)^2 = 25, 36, 49 face points) ----
 * Replaces DynamicRupture::spaceTimeInterpolation + FrictionSolver::evaluate + the DR branch of
 * Neighbor::computeNeighborsIntegral (src/Kernels/DynamicRupture.cpp:57-168,
 * src/DynamicRupture/FrictionLaws/FrictionSolver.h:38-44, src/Kernels/LinearCK/Neighbor.cpp:91-101).
 * The step of SEI_KERNEL_ALL_DR is: ADER + local (storing the CK derivatives of fault cells),
 * the fault kernel (interpolation at the Gauss-Legendre time points, friction, imposed state,
 * nodal flux into both cells), the neighbour flux of the regular faces. */
int sei_dr_setup(sei_ctx* ctx, const sei_rs_params* p, int64_t* nfaces);
/* A rate-and-state fault with the law SEI_LAW_FVW (= sei_dr_setup), SEI_LAW_RS_AGING, SEI_LAW_RS_SLIP or
 * SEI_LAW_RS_SEVERE.  The slow laws take mu = a asinh(V / (2 V0) exp((f0 + b ln(V0 theta / L)) / a))
 * (SlowVelocityWeakeningLaw.h:38-52), severe velocity weakening mu = f0 + a V / (V + V0) -
 * b theta / (theta + L); their state variable theta (SEI_DR_PSI) starts at steady sliding at v_init
 * (L / V, or V L / V0) and is kept as it is after each step, not resampled.  muw and vw are unused
 * by them; the learned warm start and the float32 pre-solve serve the fast law only. */
int sei_dr_setup_rate_state(sei_ctx* ctx, const sei_rs_params* p, int law, int64_t* nfaces);
/* The fault with linear slip weakening (src/DynamicRupture/FrictionLaws/CpuImpl/LinearSlipWeakening.h:27-170):
 * per time point the strength -cohesion - mu min(sn, 0), the slip rate max(0, (|tau| - strength) / eta_s),
 * the accumulated slip (grown by the slip rate resampled over the face for SEI_LAW_LSW, by the slip
 * rate itself for the other two), the state from it and the forced rupture, mu = mu_s - (mu_s - mu_d)
 * state, healing.  Replaces an earlier fault set-up of the context; SEI_DR_SLIP holds the
 * accumulated slip magnitude, SEI_DR_PSI and SEI_DR_A are unused. */
int sei_dr_setup_lsw(sei_ctx* ctx, const sei_lsw_params* p, int64_t* nfaces);
/* The fault with an imposed slip rate (SEI_LAW_ISR_*); replaces an earlier fault set-up. */
int sei_dr_setup_imposed(sei_ctx* ctx, const sei_isr_params* p, int64_t* nfaces);
/* Turns thermal pressurisation on (modes zeroed, fields set from p) or off, for a rate-and-state
 * fault (SEI_LAW_FVW or SEI_LAW_RS_*); the learned warm start and the float32 pre-solve are
 * skipped while it is on. */
int sei_dr_set_thermal_pressurization(sei_ctx* ctx, int on, const sei_tp_params* p);
/* Friction law of the fault (SEI_LAW_*), -1 without one. */
int sei_dr_law(const sei_ctx* ctx);
/* Gaussian nucleation (FrictionSolverCommon.h:503-531 with src/Numerical/GaussianNucleationFunction.h):
 * at every time point ending at t in [s0, s0 + t0] the initial stresses grow by the nucleation
 * fields SEI_DR_NUC_* times smoothStep(t - s0) - smoothStep(t - s0 - dt), one nucleation as the
 * parameter file's default nucleationcount.  t0 is shared with the slip-weakening forced-rupture
 * ramp, as t_0 in the reference.  on = 0 turns it off (t0, s0 ignored). */
int sei_dr_set_nucleation(sei_ctx* ctx, int on, double t0, double s0);
/* Fault time: 0 after a fault set-up, advanced by dt per step (by the cycle length per LTS cycle);
 * the forced rupture, the nucleation and the output times read it. */
int sei_dr_get_time(sei_ctx* ctx, double* t);
int sei_dr_set_time(sei_ctx* ctx, double t);
int sei_dr_num_points(int order);
int64_t sei_dr_num_faces(const sei_ctx* ctx);
/* Per face: cells [nf][2] (plus, minus), sides [nf][3] (plus side, minus side, face relation 1..3),
 * TinvT / flux solvers [nf][81] column-major, impedances [nf][8] (zp, zs, zp', zs', eta_p, eta_s, 1/eta_s, 0). */
int sei_dr_get_faces(sei_ctx* ctx, int32_t* cells, int8_t* sides, float* tinvt, float* flux_plus, float* flux_minus,
                     double* impedance);
int sei_dr_get_state(sei_ctx* ctx, int field, double* out /*[nf][npts]*/);
int sei_dr_set_state(sei_ctx* ctx, int field, const double* in /*[nf][npts]*/);
/* Imposed states of the last step, [nf][9][npts] each (points fastest). */
int sei_dr_get_imposed(sei_ctx* ctx, float* plus, float* minus);
/* Accumulated Newton iterations over all points and steps since the last reset: *total over all
 * solves, *first (may be NULL) over the first solve of each time point (the solve a warm start
 * replaces); *solves_points = faces x points. */
int sei_dr_newton_iterations(sei_ctx* ctx, int64_t* total, int64_t* solves_points, int64_t* first);
/* Accumulated float32 pre-iterations (SEI_OPT_DR_REFINE32) over all points, solves and steps since
 * the last reset (the float64 iterations are those of sei_dr_newton_iterations). */
int sei_dr_newton_iterations32(sei_ctx* ctx, int64_t* total32);
int sei_dr_reset_counters(sei_ctx* ctx);
/* Runs only the fault kernel (after a step that stored the derivatives). */
int sei_dr_faces_step(sei_ctx* ctx, double dt);
/* Slot of each fault cell in the derivative buffer ([n], -1 for cells without a fault face). */
int sei_dr_get_slots(sei_ctx* ctx, int32_t* slots);

/* Learned warm start of the slip-rate Newton solve (no counterpart in the reference, whose solve
 * starts from the previous slip rate, src/DynamicRupture/FrictionLaws/CpuImpl/RateAndState.h:339-417, first guess :354-356).
 * Network 5 -> 64 -> 64 -> 1 with tanh, FP32, on the raw inputs (normal stress sn, absolute shear
 * traction tau, state variable psi, a, b) through fixed dimensionless features
 * (tau / (|sn| a), psi / a, ln(|sn| a), a, b), each normalised as (f - norm[i]) * norm[5 + i]; its
 * output y gives t = y * norm[11] + norm[10] and the guess ln V = norm[12] + tau / (|sn| a) - psi / a - t,
 * with norm[12] = ln(2 V0) and norm[13..15] = 0.  Parameters, in this order: W1 [64][5], b1 [64],
 * W2 [64][64], b2 [64], W3 [64], b3 (sei_mlp_num_params() floats).  The fault kernel evaluates it
 * only for the first Newton solve of each time point and only starts from the guess when the
 * residual there is smaller than at the previous slip rate; a solve whose residual stops falling
 * falls back to the plain start, so the converged slip rates are those of the plain solve to
 * within the Newton tolerance. */
int sei_mlp_num_params(void);
/* Records up to `capacity` training samples [6] = (inputs [5], log10 converged slip rate) from the
 * first, plainly started Newton solve of each point in later fault steps (0 stops recording). */
int sei_dr_record_samples(sei_ctx* ctx, int64_t capacity);
/* Copies min(max, recorded) samples to out [.][6]; *count = the recorded number (<= capacity). */
int sei_dr_get_samples(sei_ctx* ctx, float* out, int64_t max, int64_t* count);
/* Trains the context's network on the GPU (Adam, full batch, cosine-decayed rate from lr, seeded
 * Glorot initialisation), `samples` [n][6] from the host or NULL for the recorded samples; the
 * normalisation is the samples' mean and standard deviation.  Mean-squared losses of the first
 * and last step are returned in normalised units. */
int sei_mlp_train(sei_ctx* ctx, const float* samples, int64_t n, int steps, float lr, uint64_t seed, float* loss_first,
                  float* loss_last);
int sei_mlp_get(sei_ctx* ctx, float* params, float* norm /*[16]*/);
int sei_mlp_set(sei_ctx* ctx, const float* params, const float* norm /*[16]*/);
/* Turns the warm start of the fault kernel on or off (needs a network). */
int sei_dr_warm_start(sei_ctx* ctx, int on);
/* Context-free checks on the current device: gradient of the mean-squared loss (normalised target)
 * over samples [n][6] and the network's log10 slip rate for each sample (target column ignored). */
int sei_mlp_gradient(const float* params, const float* norm, const float* samples, int64_t n, float* grads, float* loss);
int sei_mlp_predict(const float* params, const float* norm, const float* samples, int64_t n, float* out);
/* sei_mlp_gradient without device allocation (no counterpart in the reference), for callers that
 * own all device memory through their own pool and keep streams in flight: a cudaMalloc could fail
 * or take memory outside that pool, and cudaFree synchronises the whole device.  Its scratch is a
 * fixed static device array of 421 KiB that limits n to SEI_MLP_NOALLOC_MAX_SAMPLES (larger n
 * returns SEI_ERR_CAPACITY).  The first call on a device (the current one) looks up the array's
 * address: make it before any stream capture.  Under lazy module loading (the CUDA default) that
 * first call also loads the module, which allocates the array and may synchronise the device, so
 * make it at start-up (or set CUDA_MODULE_LOADING=EAGER).  The work runs on the calling thread's
 * per-thread default stream (cudaStreamPerThread) and the call waits for that stream only, so it
 * does not wait for the caller's other streams (it does order with the legacy stream 0).  All
 * calls on a device share the array; the accumulators are cleared by every call, and calls that
 * overlap on the GPU race. */
#define SEI_MLP_NOALLOC_MAX_SAMPLES 16384
int sei_mlp_gradient_noalloc(const float* params, const float* norm, const float* samples, int64_t n, float* grads,
                             float* loss);

/* Per-launch device timing: when on, every kernel launch of sei_run is bracketed by CUDA events on the
 * context stream; sei_kernel_times_ms sums the durations of the last sei_run per kernel kind. */
int sei_set_profiling(sei_ctx* ctx, int on);
int sei_kernel_times_ms(sei_ctx* ctx, double* local_ms, double* neighbor_ms, int* launches);
/* The same per launch kind: ms[4] and counts[4] for 0 ADER (or fused ADER + local integral),
 * 1 neighbour flux, 2 fault kernel, 3 local integral. */
int sei_kernel_times_by_kind(sei_ctx* ctx, double* ms, int* counts);

/* Diagnostic of the kernels' failure path (no counterpart in the reference): enqueues on the
 * context stream one warp that waits on an mbarrier with a limit of `polls` polls.  arrive = 0:
 * nothing arrives and nothing asynchronous is in flight, so the wait gives up, sets the context's
 * status word and returns, and the next sei_sync reports SEI_ERR_TIMEOUT (and clears the word);
 * arrive = 1: the wait completes and sei_sync reports SEI_OK.  The context stays usable either way.
 * 1 <= polls <= 2^20. */
int sei_check_wait_timeout(sei_ctx* ctx, int polls, int arrive);
/* Maximum SM clock of a device in kHz; the proxy derives its cycle count from it (the reference
 * proxy counts host cycles, src/Proxy/Runner.cpp:87-129). */
int sei_device_clock_khz(int device, int* khz);

/* Diagnostic: one 128 x N x K tile D = A B^T on the tensor cores (tcgen05 kind::tf32, TMEM
 * accumulator), A [128][K] and B [N][K] row-major host arrays, D [128][N]; terms 1 = plain TF32,
 * 3 = split TF32.  N multiple of 16 in 16..256, K multiple of 8 in 8..64.  Checks the tensor-core
 * conventions of the library on the current device. */
int sei_tc_gemm_check(const float* A, const float* B, float* D, int N, int K, int terms);

/* Diagnostic: one M x N x K tile D = A B^T on tcgen05 kind::f16 (operands rounded to FP16, FP32
 * accumulator) with A K-major and B K-major (bMN = 0) or MN-major (bMN = 1; lboIsK: the
 * descriptor's leading offset carries the K stride), A K-major (aMN = 0) or MN-major (aMN = 1,
 * the leading offset carrying the K stride).  A [M][K], B [N][K] row-major host arrays;
 * D [128][ceil16(N)] receives all 128 TMEM lanes (zeroed before the MMA), so the lane placement of
 * M = 64 results can be checked.  M 64 or 128; N multiple of 8 (M = 64) or 16 (M = 128) in 8..128;
 * K multiple of 16 in 16..96. */
int sei_tc_layout_check(const float* A, const float* B, float* D, int M, int N, int K, int bMN, int lboIsK, int aMN);
/* Diagnostic: the values each thread of one warp receives from a tcgen05.ld of shape 16x64b.x32
 * (shape 0: lanes 0..15 of the warp's quarter) after every lane wrote 1000 * lane + column into
 * columns 0..63; out [32 threads][32 registers]. */
int sei_tc_ld_probe(int shape, float* out);

/* Per-cell, per-step estimate of a proxy kernel (Local.cpp:462-522, Neighbor.cpp:190-228), elastic:
 * SEI_KERNEL_ALL, LOCAL, ADER, LOCAL_WO_ADER, NEIGHBOR (others SEI_ERR_UNSUPPORTED).  Works on a
 * host-only context. */
int sei_metrics(const sei_ctx* ctx, int kernel, sei_perf* out);

#ifdef __cplusplus
}
#endif
#endif /* SEI_GB300_H_ */
