/*
 * CPU oracle, dynamic-rupture half (TEST INFRASTRUCTURE ONLY; compiled into liboracle_*.so
 * together with oracle.c).  Float64 restatement of
 *   projectToDR          codegen/kernels/dynamic_rupture.py:126-172 (QDR(s) = V3mTo2n(side, rel) .
 *                        (sum_p coeffDR(s, p) dQ(p)) . TinvT), time points collocated as
 *                        src/Solver/TimeStepping/TimeCluster.cpp:236-241
 *   precompute stress    src/DynamicRupture/FrictionLaws/FrictionSolverCommon.h:146-200
 *   FVW rate and state   src/DynamicRupture/FrictionLaws/GpuImpl/RateAndState.h:51-270,
 *                        GpuImpl/FastVelocityWeakeningLaw.h:35-108, RateAndStateCommon.h:22-139
 *                        (per-point Newton; the outer fixed point stops when every point of a
 *                        group of 32 consecutive face points has converged, as the reference's
 *                        GPU warp vote deviceWarpAll, GpuImpl/RateAndState.h:138-142: one group
 *                        per face up to 32 points, two at orders 5 and 6)
 *   state resampling     GpuImpl/FastVelocityWeakeningLaw.h:98-106 with the resample matrix
 *   imposed state        FrictionSolverCommon.h:333-420
 *   nodal flux           dynamic_rupture.py:174-190 (Q += V3mTo2nTWDivM(side, rel) . imposed . fluxSolver)
 *   time sub-steps       src/DynamicRupture/FrictionLaws/FrictionSolver.cpp:20-37
 *   evaluate loop        CpuImpl/BaseFrictionLaw.h:49-160 (per time point: nucleation, friction,
 *                        rupture-front, dynamic-stress and peak-slip-rate outputs)
 *   nucleation           FrictionSolverCommon.h:503-531 (adjustInitialStress) with the smooth step
 *                        of src/Numerical/GaussianNucleationFunction.h
 *   linear slip weakening CpuImpl/LinearSlipWeakening.h (strength, slip rate and traction,
 *                        state from the accumulated slip with forced rupture, friction with
 *                        healing) and its specialisations NoSpecialization (resampled slip rate,
 *                        LinearSlipWeakening.cpp), BiMaterialFault (Prakash-Clifton regularised
 *                        strength) and TPApprox; initial values LinearSlipWeakeningInitializer.cpp:24-50
 *
 * Layouts: per fault face, QInterpolated[ts][9][npts] (points fastest, as the reference's
 * QInterpolated view), imposed state [9][npts]; 9x9 matrices column-major (q + 9 p);
 * V3mTo2n[16][npts][B] (index side * 4 + rel, column-major npts x B), V3mTo2nTWDivM[16][B][npts].
 * Friction state is float64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL double
#endif
typedef REAL real;

static int dr_nb3(int n) { return n * (n + 1) * (n + 2) / 6; }

/* QInterpolated of one side for all time points from packed derivatives (layout of oracle.c). */
void oracle_dr_interpolate(int order, int npts, int nts, int64_t nfaces, const real* derivs, const int32_t* cell,
                           const int8_t* side, const int8_t* rel, const double* tinvt, const double* v3m,
                           const double* coeff /*[nts][order]*/, real* qi /*[nfaces][nts][9][npts]*/) {
  const int B = dr_nb3(order);
  int dsz = 0;
  for (int i = 0; i < order; ++i) dsz += dr_nb3(order - i) * 9;
#pragma omp parallel
  {
    double* ts = (double*)malloc(sizeof(double) * (size_t)B * 9);
    double* tr = (double*)malloc(sizeof(double) * (size_t)B * 9);
#pragma omp for schedule(static)
    for (int64_t f = 0; f < nfaces; ++f) {
      const real* d = derivs + (size_t)cell[f] * dsz;
      const double* V = v3m + (size_t)(side[f] * 4 + rel[f]) * npts * B;
      const double* R = tinvt + (size_t)f * 81;
      for (int s = 0; s < nts; ++s) {
        memset(ts, 0, sizeof(double) * (size_t)B * 9);
        size_t off = 0;
        for (int i = 0; i < order; ++i) {
          const int bi = dr_nb3(order - i);
          for (int q = 0; q < 9; ++q)
            for (int l = 0; l < bi; ++l) ts[l + (size_t)B * q] += coeff[s * order + i] * (double)d[off + l + (size_t)bi * q];
          off += (size_t)bi * 9;
        }
        /* tr = ts . TinvT */
        for (int p = 0; p < 9; ++p)
          for (int l = 0; l < B; ++l) {
            double v = 0;
            for (int q = 0; q < 9; ++q) v += ts[l + (size_t)B * q] * R[q + 9 * p];
            tr[l + (size_t)B * p] = v;
          }
        real* out = qi + ((size_t)f * nts + s) * 9 * npts;
        for (int p = 0; p < 9; ++p)
          for (int k = 0; k < npts; ++k) {
            double v = 0;
            for (int l = 0; l < B; ++l) v += V[k + (size_t)npts * l] * tr[l + (size_t)B * p];
            out[k + (size_t)npts * p] = (real)v;
          }
      }
    }
    free(ts);
    free(tr);
  }
}

/* Friction parameters that are uniform over the fault (DRParameters); a is per point. */
typedef struct {
  double f0, b, v0, l, muw, vw;
  double newton_tol, state_tol;
  int max_newton, max_outer;
} oracle_rs_params;

/* Per-face impedances (DynamicRuptureMatrices.cpp:339-357). */
typedef struct {
  double zp, zs, zpn, zsn, etap, etas, inv_etas;
} oracle_imp;

/* Fault time, nucleation, outputs and linear-slip-weakening fields of one fault step (all
 * per-point arrays [nfaces][npts], nucleation stresses [nfaces][3][npts] as init). */
typedef struct {
  double time;     /* fault time at the start of the step */
  double t0, s0;   /* nucleation duration and start; t0 also ramps the forced rupture */
  int nucleate;    /* nonzero: add nuc x the smooth-step increment to the initial stresses */
  const double* nuc;
  double* peak;    /* peak slip rate */
  double* trup;    /* rupture time, negative while pending */
  double* tdyn;    /* dynamic stress time (slip weakening), negative while pending */
  int law;         /* oracle_dr_friction_lsw: 1 linear slip weakening, 2 bimaterial (Prakash-Clifton),
                    * 3 TP proxy; oracle_dr_friction: 0 fast velocity weakening, 4 aging, 5 slip,
                    * 6 severe velocity weakening */
  double healing, v_star, prakash_length, tp_exponent;
  const double *mu_s, *mu_d, *d_c, *cohesion, *t_forced;
  double* reg;     /* regularised strength (law 2) */
  /* thermal pressurisation of the rate-and-state laws (tp != 0): thermal diffusivity, heat
   * capacity, undrained response Lambda, initial temperature and pressure; per point the shear
   * zone half width and hydraulic diffusivity; state: 60 Fourier modes of temperature (theta)
   * and pressure (sigma), [nfaces][60][npts]; outputs temperature and pressure [nfaces][npts] */
  int tp;
  double tp_alpha, tp_rhoc, tp_lambda, tp_t0, tp_p0;
  const double *tp_hw, *tp_hyd;
  double *tp_theta, *tp_sigma, *tp_temp, *tp_pres;
} oracle_dr_aux;

#define TP_MODES 60
/* Thermal pressurisation (CpuImpl/ThermalPressurization/ThermalPressurization.cpp:27-107,
 * TPCommon.h): the modes' wave numbers, inverse-transform weights and Gaussian heat source. */
static double tp_grid(int i) { return 10.0 * exp(-0.3 * (TP_MODES - i - 1)); }
static double tp_inv(int i) {
  const double c = sqrt(2.0 / 3.14159265358979323846) * tp_grid(i);
  return i == 0 ? c * (1.0 + 0.3) : (i == TP_MODES - 1 ? c * 0.5 * 0.3 : c * 0.3);
}
static double tp_heat(int i) { return 1.0 / sqrt(2.0 * 3.14159265358979323846) * exp(-0.5 * tp_grid(i) * tp_grid(i)); }

/* Fluid pressure of point (face f, index k) after dt with slip rate v, friction mu and normal
 * stress sn; the modes advance only with save.  Sets the point's temperature and pressure. */
static double tp_pressure(const oracle_dr_aux* x, int64_t f, int npts, int k, double sn, double mu, double v, double dt,
                          int save) {
  const size_t i = (size_t)f * npts + k;
  const double hw = x->tp_hw[i], hyd = x->tp_hyd[i];
  const double tauv = -mu * sn * v;
  const double lp = x->tp_lambda * x->tp_alpha / (hyd - x->tp_alpha);
  double tu = 0.0, pu = 0.0;
  for (int m = 0; m < TP_MODES; ++m) {
    const size_t mi = ((size_t)f * TP_MODES + m) * npts + k;
    const double g2 = (tp_grid(m) / hw) * (tp_grid(m) / hw);
    const double th = x->tp_alpha * g2, sg = hyd * g2;
    const double om = tauv * tp_heat(m);
    const double tn = x->tp_theta[mi] * exp(-th * dt) + om / (x->tp_rhoc * th) * -expm1(-th * dt);
    const double sn_ = x->tp_sigma[mi] * exp(-sg * dt) + om * (x->tp_lambda + lp) / (x->tp_rhoc * sg) * -expm1(-sg * dt);
    const double w = tp_inv(m) / hw;
    tu += w * tn;
    pu += w * sn_;
    if (save) {
      x->tp_theta[mi] = tn;
      x->tp_sigma[mi] = sn_;
    }
  }
  pu -= lp * tu;
  x->tp_temp[i] = tu + x->tp_t0;
  x->tp_pres[i] = -pu + x->tp_p0;
  return x->tp_pres[i];
}

/* smoothStep and the nucleation of one time point ending at t_end over dt. */
static double smooth_step(double t, double t0) {
  if (t <= 0) return 0.0;
  if (t < t0) {
    const double tau = t - t0;
    return exp(tau * tau / (t * (t - 2 * t0)));
  }
  return 1.0;
}

static void nucleate(const oracle_dr_aux* x, int64_t f, int npts, double* init, double t_end, double dt) {
  if (!x || !x->nucleate || !(t_end <= x->t0 + x->s0 && t_end >= x->s0)) return;
  const double g = smooth_step(t_end - x->s0, x->t0) - smooth_step(t_end - x->s0 - dt, x->t0);
  for (int i = 0; i < 3 * npts; ++i) init[(size_t)f * 3 * npts + i] += x->nuc[(size_t)f * 3 * npts + i] * g;
}

/* Rupture-front and peak-slip-rate outputs of one point (FrictionSolverCommon.h:546-592). */
static void outputs(const oracle_dr_aux* x, size_t i, double v, double t_start) {
  if (!x) return;
  if (x->trup && x->trup[i] < 0 && v > 0.001) x->trup[i] = t_start;
  if (x->peak && v > x->peak[i]) x->peak[i] = v;
}

static double sq(double x) { return x * x; }

static double logsinh(double x, double c) {
  const double sign = c >= 0 ? 1.0 : -1.0;
  const double ac = fabs(c);
  return ac + log(x / 2 * -sign * expm1(-2 * ac));
}

static double compute_cexp(double cexplog) { return cexplog > 0 ? exp(-cexplog) : exp(cexplog); }

static double arsinhexp(double x, double explog, double e) {
  int xexp = 0;
  (void)frexp(x, &xexp);
  const double log2 = 0.69314718055994530943;
  if (explog + (xexp > 0 ? xexp : 0) * log2 > 10.0 || explog >= 50.0) {
    if (explog <= 0) e = 1 / e;
    const double xa = fabs(x);
    const double xs = x >= 0 ? 1.0 : -1.0;
    return xs * (explog + log(xa + sqrt(xa * xa + e * e)));
  }
  if (explog > 0) e = 1 / e;
  return asinh(e * x);
}

static double arsinhexp_deriv(double x, double explog, double e) {
  int xexp = 0;
  (void)frexp(x, &xexp);
  const double log2 = 0.69314718055994530943;
  if (explog + (xexp > 0 ? xexp : 0) * log2 > 10.0 || explog >= 50.0) {
    if (explog <= 0) e = 1 / e;
    return 1 / sqrt(x * x + e * e);
  }
  if (explog > 0) e = 1 / e;
  const double v = e * x;
  return e / sqrt(1 + v * v);
}

static double state_update(const oracle_rs_params* P, double a, double psi_ref, double dt, double v) {
  double lowv = P->f0 - (P->b - a) * log(v / P->v0);
  if (lowv < 0) lowv = 0;
  const double vv = v / P->vw;
  const double v8 = sq(sq(sq(vv)));
  const double fss = P->muw + (lowv - P->muw) / pow(1.0 + v8, 1.0 / 8.0);
  const double psiss = a * logsinh(P->v0 / v * 2, fss / a);
  const double pre = -v * (dt / P->l);
  return psiss * -expm1(pre) + exp(pre) * psi_ref;
}

#define ALMOST_ZERO 1e-45

/* Rate-and-state laws of the slow family and severe velocity weakening (law 4 aging, 5 slip,
 * 6 severe velocity weakening): state updates (CpuImpl/AgingLaw.h, SlipLaw.h,
 * SevereVelocityWeakeningLaw.h:14-29) on the state variable theta; law 0 is the fast law above. */
static double law_state_update(const oracle_rs_params* P, int law, double a, double ref, double dt, double v) {
  if (law == 4) {
    const double pre = -v * (dt / P->l);
    return ref * exp(pre) + P->l / v * -expm1(pre);
  }
  if (law == 5) return P->l / v * pow(v * ref / P->l, exp(-v * (dt / P->l)));
  if (law == 6) {
    const double steady = v * P->l / P->v0;
    const double pre = -P->v0 * (dt / P->l);
    return steady * -expm1(pre) + exp(pre) * ref;
  }
  return state_update(P, a, ref, dt, v);
}

/* The exponent argument psi of mu = a asinh(V / (2 V0) exp(psi / a)): the state itself for the fast
 * law, f0 + b ln(V0 theta / L) for the slow laws (SlowVelocityWeakeningLaw.h:38-52). */
static double psi_eff(const oracle_rs_params* P, int law, double state) {
  return law == 0 ? state : P->f0 + P->b * log(P->v0 * state / P->l);
}

/* Severe velocity weakening: mu = f0 + a V / (V + V0) - b theta / (theta + L) and the generic
 * Newton of RateAndState.h:327-385 (the residual tested before each update). */
static double svw_mu(const oracle_rs_params* P, double a, double theta, double v) {
  return P->f0 + a * v / (v + P->v0) - P->b * theta / (theta + P->l);
}

static int newton_svw(const oracle_rs_params* P, double a, double theta, double sn, double tau, double inv_etas,
                      double guess, double* vout, double* muout, int* conv) {
  double v = guess;
  for (int i = 0; i < P->max_newton; ++i) {
    const double mu = svw_mu(P, a, theta, v);
    const double g = -inv_etas * (fabs(sn) * mu - tau) - v;
    if (fabs(g) < P->newton_tol) {
      *vout = v;
      *muout = mu;
      *conv = 1;
      return i;
    }
    const double d = v + P->v0;
    const double dg = -inv_etas * (fabs(sn) * a * P->v0 / (d * d)) - 1.0;
    v = v - g / dg;
    if (v < ALMOST_ZERO) v = ALMOST_ZERO;
  }
  *vout = v;
  *muout = 0.0;
  *conv = 0;
  return P->max_newton;
}

/* Newton solve of g(V) = -(|sn| mu(V, psi) - tau) / eta_s - V = 0 from guess v0; returns the
 * iteration count (number of updates made) and sets *conv.  With bail, the solve gives up as
 * soon as |g| does not fall (used for the network's starting value). */
static int newton(const oracle_rs_params* P, double a, double psi, double sn, double tau, double inv_etas,
                  double guess, double* vout, double* muout, int* conv, int bail) {
  const double clin = 0.5 / P->v0;
  const double cexplog = psi / a;
  const double cexp = compute_cexp(cexplog);
  double v = guess;
  double prev = 1e300;
  for (int i = 0; i < P->max_newton; ++i) {
    const double mu = a * arsinhexp(clin * v, cexplog, cexp);
    const double g = -inv_etas * (fabs(sn) * mu - tau) - v;
    if (fabs(g) < P->newton_tol) {
      *vout = v;
      *muout = mu;
      *conv = 1;
      return i;
    }
    if (bail && !(fabs(g) < prev)) {
      *vout = v;
      *muout = 0.0;
      *conv = 0;
      return i;
    }
    prev = fabs(g);
    const double dmu = a * clin * arsinhexp_deriv(clin * v, cexplog, cexp);
    const double dg = -inv_etas * (fabs(sn) * dmu) - 1.0;
    v = v - g / dg;
    if (v < ALMOST_ZERO) v = ALMOST_ZERO;
  }
  *vout = v;
  *muout = 0.0;
  *conv = 0;
  return P->max_newton;
}

/* Warm-start network 5 -> 64 -> 64 -> 1 (tanh), float32: returns the natural log of the guessed
 * slip rate.  Parameters W1[64][5], b1[64], W2[64][64], b2[64], W3[64], b3.  The inputs are the
 * fixed features (tau / (|sn| a), psi / a, ln(|sn| a), a, b) with |sn| a floored at 1 Pa,
 * normalised by norm[0..4] (shift) and norm[5..9] (scale); the output y gives
 * r = y norm[11] + norm[10] and ln V = norm[12] + tau / (|sn| a) - psi / a - softplus(z) - r with
 * z = tau / (|sn| a) - psi / a - ln(|sn| a). */
#define MLP_H 64
/* Points the network applies to: |sn| a > 1 Pa and tau < 500 |sn| a. */
static int mlp_usable(double sn, double tau, double a) {
  const double an = fabs(sn) * a;
  return an > 1.0 && tau < 500.0 * an;
}
void oracle_mlp_features(double sn, double tau, double psi, double a, double b, double* f) {
  double an = fabs(sn) * a;
  if (!(an > 1.0)) an = 1.0;
  f[0] = tau / an;
  f[1] = psi / a;
  f[2] = log(an);
  f[3] = a;
  f[4] = b;
}

double oracle_mlp_forward(const float* w, const float* norm, double sn, double tau, double psi, double a, double b) {
  double f[5];
  oracle_mlp_features(sn, tau, psi, a, b, f);
  float x[5];
  for (int i = 0; i < 5; ++i) x[i] = (float)((f[i] - norm[i]) * norm[5 + i]);
  const float* W1 = w;
  const float* b1 = W1 + MLP_H * 5;
  const float* W2 = b1 + MLP_H;
  const float* b2 = W2 + MLP_H * MLP_H;
  const float* W3 = b2 + MLP_H;
  const float b3 = W3[MLP_H];
  float h1[MLP_H];
  for (int j = 0; j < MLP_H; ++j) {
    float s = b1[j];
    for (int i = 0; i < 5; ++i) s = fmaf(W1[j * 5 + i], x[i], s);
    h1[j] = tanhf(s);
  }
  float out = b3;
  for (int j = 0; j < MLP_H; ++j) {
    float s = b2[j];
    for (int i = 0; i < MLP_H; ++i) s = fmaf(W2[j * MLP_H + i], h1[i], s);
    out = fmaf(W3[j], tanhf(s), out);
  }
  const double z = f[0] - f[1] - f[2];
  const double softplus = z > 30.0 ? z : log1p(exp(z));
  return norm[12] + f[0] - f[1] - softplus - ((double)out * norm[11] + norm[10]);
}

/* Friction solve of all faces for one time step.  State arrays are [nfaces][npts] float64:
 * psi, v1, v2, slip1, slip2, slip (accumulated magnitude), mu, traction1, traction2;
 * init[nfaces][3][npts] holds sn0, tau1_0, tau2_0.  With mlp non-null the first Newton solve
 * of every time point starts from the network's guess when its residual is below that of the
 * plain start (previous slip rate), and falls back to the plain start when the residual from
 * the guess stops falling.  newton_iters[nfaces][npts] accumulates the Newton iteration counts
 * and first_iters (optional) those of the first solve of each time point.  With rec non-null the
 * inputs and log10 of the converged slip rate of every plainly started, converged first solve are
 * appended as [6] floats at rec[(*rec_count)++] (up to rec_cap). */

void oracle_dr_friction(int npts, int nts, int64_t nfaces, const oracle_rs_params* P, const oracle_imp* imp,
                        const real* qip, const real* qim, const double* a, double* init, double* psi,
                        double* v1, double* v2, double* slip1, double* slip2, double* slip, double* mu,
                        double* trac1, double* trac2, const double* deltat, const double* tweights,
                        const double* resample, real* isp, real* ism, int64_t* newton_iters,
                        const float* mlp, const float* mlp_norm, int64_t* first_iters, float* rec,
                        int64_t rec_cap, int64_t* rec_count, const oracle_dr_aux* aux) {
  const int law = aux ? aux->law : 0; /* 0 fast velocity weakening, 4 aging, 5 slip, 6 severe */
  const int tp = aux && aux->tp;
  if (law != 0 || tp) mlp = NULL, rec = NULL;
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * (size_t)npts * 12);
    double* psib = buf;
    double* vmag = buf + npts;
    double* lsr = buf + 2 * npts;
    double* sref = buf + 3 * npts;
    double* taus = buf + 4 * npts;
    double* sns = buf + 5 * npts;
    double* vt = buf + 6 * npts;
    double* dpsi = buf + 7 * npts;
    double* isacc = (double*)malloc(sizeof(double) * 18 * (size_t)npts);
    double* fs = (double*)malloc(sizeof(double) * 3 * (size_t)nts * npts);
    double* tr = (double*)malloc(sizeof(double) * 2 * (size_t)nts * npts);
    int* convo = (int*)malloc(sizeof(int) * (size_t)npts);
#pragma omp for schedule(static)
    for (int64_t f = 0; f < nfaces; ++f) {
      const oracle_imp* im = imp + f;
      const size_t fo = (size_t)f * npts;
      /* precompute stress (etaPDamp = 1) */
      for (int s = 0; s < nts; ++s) {
        const real* P_ = qip + ((size_t)f * nts + s) * 9 * npts;
        const real* M_ = qim + ((size_t)f * nts + s) * 9 * npts;
        for (int k = 0; k < npts; ++k) {
#define QP(q) ((double)P_[k + (size_t)npts * (q)])
#define QM(q) ((double)M_[k + (size_t)npts * (q)])
          fs[(0 * nts + s) * npts + k] = im->etap * (QM(6) - QP(6) + QP(0) / im->zp + QM(0) / im->zpn);
          fs[(1 * nts + s) * npts + k] = im->etas * (QM(7) - QP(7) + QP(3) / im->zs + QM(3) / im->zsn);
          fs[(2 * nts + s) * npts + k] = im->etas * (QM(8) - QP(8) + QP(5) / im->zs + QM(5) / im->zsn);
        }
      }
      for (int k = 0; k < npts; ++k) psib[k] = psi[fo + k];
      double t_start = aux ? aux->time : 0.0;
      for (int s = 0; s < nts; ++s) {
        const double dt = deltat[s];
        nucleate(aux, f, npts, init, t_start + dt, dt);
        for (int k = 0; k < npts; ++k) {
          const double sn0 = init[(size_t)f * 3 * npts + k];
          const double t10 = init[(size_t)f * 3 * npts + npts + k];
          const double t20 = init[(size_t)f * 3 * npts + 2 * npts + k];
          double sn = fs[(0 * nts + s) * npts + k] + sn0 - (tp ? aux->tp_pres[fo + k] : 0.0);
          sns[k] = sn < 0 ? sn : 0.0;
          sref[k] = psib[k];
          const double tt1 = t10 + fs[(1 * nts + s) * npts + k];
          const double tt2 = t20 + fs[(2 * nts + s) * npts + k];
          taus[k] = sqrt(tt1 * tt1 + tt2 * tt2);
          double vm = sqrt(v1[fo + k] * v1[fo + k] + v2[fo + k] * v2[fo + k]);
          if (vm < ALMOST_ZERO) vm = ALMOST_ZERO;
          vmag[k] = vm;
          lsr[k] = vm;
        }
        for (int g0 = 0; g0 < npts; g0 += 32) {  /* one vote per group of 32 points */
        const int g1 = g0 + 32 < npts ? g0 + 32 : npts;
        for (int j = 0; j < P->max_outer; ++j) {
          int all = 1;
          for (int k = g0; k < g1; ++k) {
            const double ak = a[fo + k];
            psib[k] = law_state_update(P, law, ak, sref[k], dt, lsr[k]);
            if (tp) { /* pressure of this pass from the previous pass's stress and friction */
              const double pr = tp_pressure(aux, f, npts, k, sns[k], mu[fo + k], lsr[k], dt, 0);
              const double sn = fs[(0 * nts + s) * npts + k] + init[(size_t)f * 3 * npts + k] - pr;
              sns[k] = sn < 0 ? sn : 0.0;
            }
            double vnew = 0, munew = 0;
            int conv = 0, its = 0;
            if (law == 6) {
              its = newton_svw(P, ak, psib[k], sns[k], taus[k], im->inv_etas, vmag[k], &vnew, &munew, &conv);
              newton_iters[fo + k] += its;
              if (first_iters && j == 0) first_iters[fo + k] += its;
              lsr[k] = 0.5 * (vmag[k] + vnew);
              convo[k] = fabs(vmag[k] - vnew) < P->state_tol;
              vmag[k] = vnew;
              mu[fo + k] = munew;
              all &= convo[k];
              continue;
            }
            const double pe = psi_eff(P, law, psib[k]);
            if (mlp && j == 0 && mlp_usable(sns[k], taus[k], ak)) {
              double lg = oracle_mlp_forward(mlp, mlp_norm, sns[k], taus[k], psib[k], ak, P->b);
              lg = lg < -103.616329 ? -103.616329 : (lg > 6.907755 ? 6.907755 : lg); /* 1e-45 .. 1e3 m/s */
              const double g0 = exp(lg);
              const double cl = psib[k] / ak, ce = compute_cexp(cl), clin = 0.5 / P->v0;
              const double rg = -im->inv_etas * (fabs(sns[k]) * ak * arsinhexp(clin * g0, cl, ce) - taus[k]) - g0;
              const double rp = -im->inv_etas * (fabs(sns[k]) * ak * arsinhexp(clin * vmag[k], cl, ce) - taus[k]) - vmag[k];
              if (fabs(rg) < fabs(rp)) its += newton(P, ak, psib[k], sns[k], taus[k], im->inv_etas, g0, &vnew, &munew, &conv, 1);
            }
            if (!conv) {
              its += newton(P, ak, pe, sns[k], taus[k], im->inv_etas, vmag[k], &vnew, &munew, &conv, 0);
              if (rec && j == 0 && conv && mlp_usable(sns[k], taus[k], ak)) {
                int64_t idx;
#pragma omp atomic capture
                idx = (*rec_count)++;
                if (idx < rec_cap) {
                  float* o = rec + idx * 6;
                  o[0] = (float)sns[k];
                  o[1] = (float)taus[k];
                  o[2] = (float)psib[k];
                  o[3] = (float)ak;
                  o[4] = (float)P->b;
                  o[5] = (float)log10(vnew);
                }
              }
            }
            newton_iters[fo + k] += its;
            if (first_iters && j == 0) first_iters[fo + k] += its;
            lsr[k] = 0.5 * (vmag[k] + vnew);
            convo[k] = fabs(vmag[k] - vnew) < P->state_tol;
            vmag[k] = vnew;
            mu[fo + k] = munew;
            all &= convo[k];
          }
          if (all) break;
        }
        }
        for (int k = 0; k < npts; ++k) {
          const double ak = a[fo + k];
          if (tp) { /* the modes advance with the pass's final slip rate */
            const double pr = tp_pressure(aux, f, npts, k, sns[k], mu[fo + k], lsr[k], dt, 1);
            const double sn = fs[(0 * nts + s) * npts + k] + init[(size_t)f * 3 * npts + k] - pr;
            sns[k] = sn < 0 ? sn : 0.0;
          }
          psib[k] = law_state_update(P, law, ak, sref[k], dt, lsr[k]);
          const double clin = 0.5 / P->v0;
          const double cexplog = psi_eff(P, law, psib[k]) / ak;
          const double m =
              law == 6 ? svw_mu(P, ak, psib[k], vmag[k]) : ak * arsinhexp(clin * vmag[k], cexplog, compute_cexp(cexplog));
          mu[fo + k] = m;
          const double strength = -m * sns[k];
          const double t10 = init[(size_t)f * 3 * npts + npts + k];
          const double t20 = init[(size_t)f * 3 * npts + 2 * npts + k];
          const double st1 = fs[(1 * nts + s) * npts + k], st2 = fs[(2 * nts + s) * npts + k];
          const double tt1 = t10 + st1, tt2 = t20 + st2;
          slip[fo + k] += vmag[k] * dt;
          const double div = strength + im->etas * vmag[k];
          const double sr1 = vmag[k] * tt1 / div, sr2 = vmag[k] * tt2 / div;
          const double tr1 = st1 - im->etas * sr1, tr2 = st2 - im->etas * sr2;
          trac1[fo + k] = tr1;
          trac2[fo + k] = tr2;
          slip1[fo + k] += sr1 * dt;
          slip2[fo + k] += sr2 * dt;
          tr[(0 * nts + s) * npts + k] = tr1;
          tr[(1 * nts + s) * npts + k] = tr2;
          v1[fo + k] = sr1;
          v2[fo + k] = sr2;
          outputs(aux, fo + k, vmag[k], t_start);
        }
        t_start += dt;
      }
      /* resample the state variable increment (FastVelocityWeakeningLaw.h:98-106); the other
       * laws copy the state (SlowVelocityWeakeningLaw.h:66-72) */
      for (int k = 0; k < npts; ++k) dpsi[k] = psib[k] - psi[fo + k];
      for (int k = 0; k < npts; ++k) {
        double v = 0;
        for (int j = 0; j < npts; ++j) v += resample[k + (size_t)npts * j] * dpsi[j];
        vt[k] = law == 0 ? psi[fo + k] + v : psib[k];
      }
      for (int k = 0; k < npts; ++k) psi[fo + k] = vt[k];
      /* imposed state */
      memset(isacc, 0, sizeof(double) * 18 * (size_t)npts);
      for (int s = 0; s < nts; ++s) {
        const double w = tweights[s];
        const real* P_ = qip + ((size_t)f * nts + s) * 9 * npts;
        const real* M_ = qim + ((size_t)f * nts + s) * 9 * npts;
        for (int k = 0; k < npts; ++k) {
          const double sn = fs[(0 * nts + s) * npts + k];
          const double t1 = tr[(0 * nts + s) * npts + k], t2 = tr[(1 * nts + s) * npts + k];
          double* m_ = isacc;
          double* p_ = isacc + 9 * npts;
          m_[0 * npts + k] += w * sn;
          m_[3 * npts + k] += w * t1;
          m_[5 * npts + k] += w * t2;
          m_[6 * npts + k] += w * (QM(6) - (sn - QM(0)) / im->zpn);
          m_[7 * npts + k] += w * (QM(7) - (t1 - QM(3)) / im->zsn);
          m_[8 * npts + k] += w * (QM(8) - (t2 - QM(5)) / im->zsn);
          p_[0 * npts + k] += w * sn;
          p_[3 * npts + k] += w * t1;
          p_[5 * npts + k] += w * t2;
          p_[6 * npts + k] += w * (QP(6) + (sn - QP(0)) / im->zp);
          p_[7 * npts + k] += w * (QP(7) + (t1 - QP(3)) / im->zs);
          p_[8 * npts + k] += w * (QP(8) + (t2 - QP(5)) / im->zs);
#undef QP
#undef QM
        }
      }
      for (int i = 0; i < 9 * npts; ++i) {
        ism[(size_t)f * 9 * npts + i] = (real)isacc[i];
        isp[(size_t)f * 9 * npts + i] = (real)isacc[9 * npts + i];
      }
    }
    free(buf);
    free(isacc);
    free(fs);
    free(tr);
    free(convo);
  }
}

#define QP(q) ((double)P_[k + (size_t)npts * (q)])
#define QM(q) ((double)M_[k + (size_t)npts * (q)])
/* Linear slip weakening, one time step of all faces (CpuImpl/LinearSlipWeakening.h:27-170 inside
 * the evaluate loop of CpuImpl/BaseFrictionLaw.h:49-160).  Per time point: nucleation of the
 * initial stresses; strength -cohesion - mu min(sn_total, 0) (law 2: regularised towards it with
 * exp(-(max(V_prev, 0) + v_star) dt / L), BiMaterialFault::strengthHook); slip rate
 * max(0, (|tau_total| - strength) / eta_s) split along the total traction; tractions and slips;
 * the accumulated slip grows by the slip rate resampled over the face (law 1, resample matrix) or
 * by the slip rate itself (laws 2, 3); state min(|slip| / d_c, 1) (law 3: 1 - (1 + |slip| /
 * d_c)^-p), at least the forced-rupture ramp of the time point's end; mu = mu_s - (mu_s - mu_d)
 * state, back to mu_s where the peak slip rate passed the healing threshold and the slip rate is
 * below it; outputs.  State fields as oracle_dr_friction, slip = accumulated slip magnitude. */
void oracle_dr_friction_lsw(int npts, int nts, int64_t nfaces, const oracle_imp* imp, const real* qip, const real* qim,
                            double* init, double* v1, double* v2, double* slip1, double* slip2, double* slip,
                            double* mu, double* trac1, double* trac2, const double* deltat, const double* tweights,
                            const double* resample, real* isp, real* ism, const oracle_dr_aux* x) {
  double* fs = (double*)malloc(sizeof(double) * 3 * (size_t)nts * npts);
  double* tr = (double*)malloc(sizeof(double) * 2 * (size_t)nts * npts);
  double* vm = (double*)malloc(sizeof(double) * (size_t)npts);
  double* rv = (double*)malloc(sizeof(double) * (size_t)npts);
  double* isacc = (double*)malloc(sizeof(double) * 18 * (size_t)npts);
  for (int64_t f = 0; f < nfaces; ++f) {
    const oracle_imp* im = imp + f;
    const size_t fo = (size_t)f * npts;
    for (int s = 0; s < nts; ++s) {
      const real* P_ = qip + ((size_t)f * nts + s) * 9 * npts;
      const real* M_ = qim + ((size_t)f * nts + s) * 9 * npts;
      for (int k = 0; k < npts; ++k) {
        fs[(0 * nts + s) * npts + k] = im->etap * (QM(6) - QP(6) + QP(0) / im->zp + QM(0) / im->zpn);
        fs[(1 * nts + s) * npts + k] = im->etas * (QM(7) - QP(7) + QP(3) / im->zs + QM(3) / im->zsn);
        fs[(2 * nts + s) * npts + k] = im->etas * (QM(8) - QP(8) + QP(5) / im->zs + QM(5) / im->zsn);
      }
    }
    /* slip-rate magnitude of the previous time point (the bimaterial strength reads it) */
    for (int k = 0; k < npts; ++k) vm[k] = sqrt(v1[fo + k] * v1[fo + k] + v2[fo + k] * v2[fo + k]);
    double t_start = x->time;
    for (int s = 0; s < nts; ++s) {
      const double dt = deltat[s], t_end = t_start + dt;
      nucleate(x, f, npts, init, t_end, dt);
      for (int k = 0; k < npts; ++k) {
        const double* in = init + (size_t)f * 3 * npts;
        const double sn = in[k] + fs[(0 * nts + s) * npts + k];
        double strength = -x->cohesion[fo + k] - mu[fo + k] * (sn < 0 ? sn : 0.0);
        if (x->law == 2) {
          const double e = -((vm[k] > 0 ? vm[k] : 0.0) + x->v_star) * dt / x->prakash_length;
          strength = x->reg[fo + k] * exp(e) + strength * -expm1(e);
          x->reg[fo + k] = strength;
        }
        const double st1 = fs[(1 * nts + s) * npts + k], st2 = fs[(2 * nts + s) * npts + k];
        const double tt1 = in[npts + k] + st1, tt2 = in[2 * npts + k] + st2;
        const double tau = sqrt(tt1 * tt1 + tt2 * tt2);
        double v = (tau - strength) * im->inv_etas;
        v = v > 0 ? v : 0.0;
        const double div = strength + im->etas * v;
        const double sr1 = v * tt1 / div, sr2 = v * tt2 / div;
        v1[fo + k] = sr1;
        v2[fo + k] = sr2;
        const double t1 = st1 - im->etas * sr1, t2 = st2 - im->etas * sr2;
        trac1[fo + k] = t1;
        trac2[fo + k] = t2;
        tr[(0 * nts + s) * npts + k] = t1;
        tr[(1 * nts + s) * npts + k] = t2;
        slip1[fo + k] += sr1 * dt;
        slip2[fo + k] += sr2 * dt;
        vm[k] = v;
      }
      for (int k = 0; k < npts; ++k) {
        double r = vm[k];
        if (x->law == 1) {
          r = 0;
          for (int j = 0; j < npts; ++j) r += resample[k + (size_t)npts * j] * vm[j];
        }
        rv[k] = r;
      }
      for (int k = 0; k < npts; ++k) {
        const size_t i = fo + k;
        slip[i] += rv[k] * dt;
        const double ratio = fabs(slip[i]) / x->d_c[i];
        double state = x->law == 3 ? 1.0 - pow(1.0 + ratio, -x->tp_exponent) : (ratio < 1.0 ? ratio : 1.0);
        double f2;
        if (x->t0 == 0) {
          f2 = t_end >= x->t_forced[i] ? 1.0 : 0.0;
        } else {
          f2 = (t_end - x->t_forced[i]) / x->t0;
          f2 = f2 < 0 ? 0.0 : (f2 > 1 ? 1.0 : f2);
        }
        state = state > f2 ? state : f2;
        mu[i] = x->mu_s[i] - (x->mu_s[i] - x->mu_d[i]) * state;
        if (x->peak[i] > x->healing && vm[k] < x->healing) mu[i] = x->mu_s[i];
        outputs(x, i, vm[k], t_start);
        if (x->tdyn && x->tdyn[i] < 0 && fabs(slip[i]) >= x->d_c[i]) x->tdyn[i] = t_start;
      }
      t_start = t_end;
    }
    /* imposed state (FrictionSolverCommon.h:333-420) */
    memset(isacc, 0, sizeof(double) * 18 * (size_t)npts);
    for (int s = 0; s < nts; ++s) {
      const double w = tweights[s];
      const real* P_ = qip + ((size_t)f * nts + s) * 9 * npts;
      const real* M_ = qim + ((size_t)f * nts + s) * 9 * npts;
      for (int k = 0; k < npts; ++k) {
        const double sn = fs[(0 * nts + s) * npts + k];
        const double t1 = tr[(0 * nts + s) * npts + k], t2 = tr[(1 * nts + s) * npts + k];
        double* m_ = isacc;
        double* p_ = isacc + 9 * npts;
        m_[0 * npts + k] += w * sn;
        m_[3 * npts + k] += w * t1;
        m_[5 * npts + k] += w * t2;
        m_[6 * npts + k] += w * (QM(6) - (sn - QM(0)) / im->zpn);
        m_[7 * npts + k] += w * (QM(7) - (t1 - QM(3)) / im->zsn);
        m_[8 * npts + k] += w * (QM(8) - (t2 - QM(5)) / im->zsn);
        p_[0 * npts + k] += w * sn;
        p_[3 * npts + k] += w * t1;
        p_[5 * npts + k] += w * t2;
        p_[6 * npts + k] += w * (QP(6) + (sn - QP(0)) / im->zp);
        p_[7 * npts + k] += w * (QP(7) + (t1 - QP(3)) / im->zs);
        p_[8 * npts + k] += w * (QP(8) + (t2 - QP(5)) / im->zs);
      }
    }
    for (int i = 0; i < 9 * npts; ++i) {
      ism[(size_t)f * 9 * npts + i] = (real)isacc[i];
      isp[(size_t)f * 9 * npts + i] = (real)isacc[9 * npts + i];
    }
  }
  free(fs);
  free(tr);
  free(vm);
  free(rv);
  free(isacc);
}

/* Regularised Yoffe function (Tinti et al. 2005, closed form of the Yoffe function of rise time
 * tR convolved with a triangle of half width tS; Numerical/RegularizedYoffe.h). */
double oracle_regularized_yoffe(double t, double tS, double tR) {
  const double pi = 3.14159265358979323846;
  const double k = 2.0 / (pi * tR * tS * tS);
  if (t <= 0.0 || t >= tR + 2.0 * tS) return 0.0;
#define C1 ((0.5 * t + 0.25 * tR) * sqrt(t * (tR - t)) + (t * tR - tR * tR) * asin(sqrt(t / tR)) - \
            0.75 * tR * tR * atan(sqrt((tR - t) / t)))
#define C2 (0.375 * pi * tR * tR)
#define C3 ((tS - t - 0.5 * tR) * sqrt((t - tS) * (tR - t + tS)) + tR * (2.0 * tR - 2.0 * t + 2.0 * tS) * asin(sqrt((t - tS) / tR)) + \
            1.5 * tR * tR * atan(sqrt((tR - t + tS) / (t - tS))))
#define C4 ((-tS + 0.5 * t + 0.25 * tR) * sqrt((t - 2.0 * tS) * (tR - t + 2.0 * tS)) - \
            tR * (tR - t + 2.0 * tS) * asin(sqrt((t - 2.0 * tS) / tR)) - 0.75 * tR * tR * atan(sqrt((tR - t + 2.0 * tS) / (t - 2.0 * tS))))
#define C5 (0.5 * pi * tR * (t - tR))
#define C6 (0.5 * pi * tR * (2.0 * tS - t + tR))
  double r;
  if (t <= tS) r = C1 + C2;
  else if (tR > 2.0 * tS) r = t <= 2.0 * tS ? C1 - C2 + C3 : (t < tR ? C1 + C3 + C4 : (t < tR + tS ? C3 + C4 + C5 : C4 + C6));
  else r = t < tR ? C1 - C2 + C3 : (t <= 2.0 * tS ? C5 + C3 - C2 : (t < tR + tS ? C3 + C4 + C5 : C4 + C6));
#undef C1
#undef C2
#undef C3
#undef C4
#undef C5
#undef C6
  return k * r;
}

/* Imposed slip rates, one time step of all faces (CpuImpl/ImposedSlipRates.h:21-60 in the evaluate
 * loop of BaseFrictionLaw.h:103-137): per time point the source time function at the point's end
 * (law 7 regularised Yoffe of (t - onset, tau_S, tau_R), 8 Gaussian smooth-step increment over
 * the sub-step with rise time tau_S divided by it, 9 delta pulse 1/dt on (0, dt]), slip rate =
 * direction x STF, traction = fault stress - eta_s x slip rate, slips, outputs.  dir1, dir2, onset,
 * taus, taur are [nfaces][npts]; state fields as oracle_dr_friction (slip = accumulated magnitude). */
void oracle_dr_friction_isr(int npts, int nts, int64_t nfaces, const oracle_imp* imp, const real* qip, const real* qim,
                            double* init, double* v1, double* v2, double* slip1, double* slip2, double* slip,
                            double* trac1, double* trac2, const double* deltat, const double* tweights,
                            const double* dir1, const double* dir2, const double* onset, const double* taus,
                            const double* taur, real* isp, real* ism, const oracle_dr_aux* x) {
  double* fs = (double*)malloc(sizeof(double) * 3 * (size_t)nts * npts);
  double* tr = (double*)malloc(sizeof(double) * 2 * (size_t)nts * npts);
  double* isacc = (double*)malloc(sizeof(double) * 18 * (size_t)npts);
  for (int64_t f = 0; f < nfaces; ++f) {
    const oracle_imp* im = imp + f;
    const size_t fo = (size_t)f * npts;
    for (int s = 0; s < nts; ++s) {
      const real* P_ = qip + ((size_t)f * nts + s) * 9 * npts;
      const real* M_ = qim + ((size_t)f * nts + s) * 9 * npts;
      for (int k = 0; k < npts; ++k) {
        fs[(0 * nts + s) * npts + k] = im->etap * (QM(6) - QP(6) + QP(0) / im->zp + QM(0) / im->zpn);
        fs[(1 * nts + s) * npts + k] = im->etas * (QM(7) - QP(7) + QP(3) / im->zs + QM(3) / im->zsn);
        fs[(2 * nts + s) * npts + k] = im->etas * (QM(8) - QP(8) + QP(5) / im->zs + QM(5) / im->zsn);
      }
    }
    double t_start = x->time;
    for (int s = 0; s < nts; ++s) {
      const double dt = deltat[s], t_end = t_start + dt;
      nucleate(x, f, npts, init, t_end, dt);
      for (int k = 0; k < npts; ++k) {
        const size_t i = fo + k;
        const double t = t_end - onset[i];
        double stf;
        if (x->law == 7)
          stf = oracle_regularized_yoffe(t, taus[i], taur[i]);
        else if (x->law == 8)
          stf = (smooth_step(t, taus[i]) - smooth_step(t - dt, taus[i])) / dt;
        else
          stf = t > 0 && t <= dt ? 1.0 / dt : 0.0;
        const double st1 = fs[(1 * nts + s) * npts + k], st2 = fs[(2 * nts + s) * npts + k];
        v1[i] = dir1[i] * stf;
        v2[i] = dir2[i] * stf;
        const double t1 = st1 - im->etas * v1[i], t2 = st2 - im->etas * v2[i];
        trac1[i] = t1;
        trac2[i] = t2;
        tr[(0 * nts + s) * npts + k] = t1;
        tr[(1 * nts + s) * npts + k] = t2;
        const double vm = sqrt(v1[i] * v1[i] + v2[i] * v2[i]);
        slip1[i] += v1[i] * dt;
        slip2[i] += v2[i] * dt;
        slip[i] += vm * dt;
        outputs(x, i, vm, t_start);
      }
      t_start = t_end;
    }
    memset(isacc, 0, sizeof(double) * 18 * (size_t)npts);
    for (int s = 0; s < nts; ++s) {
      const double w = tweights[s];
      const real* P_ = qip + ((size_t)f * nts + s) * 9 * npts;
      const real* M_ = qim + ((size_t)f * nts + s) * 9 * npts;
      for (int k = 0; k < npts; ++k) {
        const double sn = fs[(0 * nts + s) * npts + k];
        const double t1 = tr[(0 * nts + s) * npts + k], t2 = tr[(1 * nts + s) * npts + k];
        double* m_ = isacc;
        double* p_ = isacc + 9 * npts;
        m_[0 * npts + k] += w * sn;
        m_[3 * npts + k] += w * t1;
        m_[5 * npts + k] += w * t2;
        m_[6 * npts + k] += w * (QM(6) - (sn - QM(0)) / im->zpn);
        m_[7 * npts + k] += w * (QM(7) - (t1 - QM(3)) / im->zsn);
        m_[8 * npts + k] += w * (QM(8) - (t2 - QM(5)) / im->zsn);
        p_[0 * npts + k] += w * sn;
        p_[3 * npts + k] += w * t1;
        p_[5 * npts + k] += w * t2;
        p_[6 * npts + k] += w * (QP(6) + (sn - QP(0)) / im->zp);
        p_[7 * npts + k] += w * (QP(7) + (t1 - QP(3)) / im->zs);
        p_[8 * npts + k] += w * (QP(8) + (t2 - QP(5)) / im->zs);
      }
    }
    for (int i = 0; i < 9 * npts; ++i) {
      ism[(size_t)f * 9 * npts + i] = (real)isacc[i];
      isp[(size_t)f * 9 * npts + i] = (real)isacc[9 * npts + i];
    }
  }
  free(fs);
  free(tr);
  free(isacc);
}

#undef QP
#undef QM

/* One thermal-pressurisation update of point k of face f (test hook of tp_pressure). */
double oracle_dr_tp_point(const oracle_dr_aux* x, int64_t f, int npts, int k, double sn, double mu, double v, double dt,
                          int save) {
  return tp_pressure(x, f, npts, k, sn, mu, v, dt, save);
}

/* Q(cell) += V3mTo2nTWDivM(side, rel) . imposed . fluxSolver for one side of every face. */
void oracle_dr_nodal_flux(int order, int npts, int64_t nfaces, const int32_t* cell, const int8_t* side,
                          const int8_t* rel, const double* twdivm, const real* imposed, const double* fluxsolver,
                          real* Q) {
  const int B = dr_nb3(order);
  for (int64_t f = 0; f < nfaces; ++f) {
    const double* W = twdivm + (size_t)(side[f] * 4 + rel[f]) * B * npts;
    const real* is = imposed + (size_t)f * 9 * npts;
    const double* fsv = fluxsolver + (size_t)f * 81;
    real* q = Q + (size_t)cell[f] * B * 9;
    for (int p = 0; p < 9; ++p)
      for (int l = 0; l < B; ++l) {
        double v = 0;
        for (int k = 0; k < npts; ++k) {
          double g = 0;
          for (int qq = 0; qq < 9; ++qq) g += (double)is[k + (size_t)npts * qq] * fsv[qq + 9 * p];
          v += W[l + (size_t)B * k] * g;
        }
        q[l + (size_t)B * p] += (real)v;
      }
  }
}

/* Precompute / postcompute known-answer helpers (FrictionSolverCommon.h), exposed for the
 * restated unit test of tests/DynamicRupture/FrictionLaws/FrictionSolverCommon.t.h. */
void oracle_dr_precompute(int npts, int nts, const oracle_imp* im, const real* qip, const real* qim, double* out) {
  for (int s = 0; s < nts; ++s)
    for (int k = 0; k < npts; ++k) {
      const real* P_ = qip + (size_t)s * 9 * npts;
      const real* M_ = qim + (size_t)s * 9 * npts;
      out[(0 * nts + s) * npts + k] = im->etap * (M_[6 * npts + k] - P_[6 * npts + k] + P_[k] / im->zp + M_[k] / im->zpn);
      out[(1 * nts + s) * npts + k] =
          im->etas * (M_[7 * npts + k] - P_[7 * npts + k] + P_[3 * npts + k] / im->zs + M_[3 * npts + k] / im->zsn);
      out[(2 * nts + s) * npts + k] =
          im->etas * (M_[8 * npts + k] - P_[8 * npts + k] + P_[5 * npts + k] / im->zs + M_[5 * npts + k] / im->zsn);
    }
}

/* Imposed states from the stresses of every time point (FrictionSolverCommon.h:333-420);
 * normal[nts][npts], t1/t2 are the new tractions [nts][npts]. */
void oracle_dr_postcompute(int npts, int nts, const oracle_imp* im, const real* qip, const real* qim,
                           const double* normal, const double* t1, const double* t2, const double* tweights, double* isp,
                           double* ism) {
  memset(isp, 0, sizeof(double) * 9 * (size_t)npts);
  memset(ism, 0, sizeof(double) * 9 * (size_t)npts);
  for (int s = 0; s < nts; ++s) {
    const double w = tweights[s];
    const real* P_ = qip + (size_t)s * 9 * npts;
    const real* M_ = qim + (size_t)s * 9 * npts;
    for (int k = 0; k < npts; ++k) {
      const double sn = normal[s * npts + k], a1 = t1[s * npts + k], a2 = t2[s * npts + k];
      ism[0 * npts + k] += w * sn;
      ism[3 * npts + k] += w * a1;
      ism[5 * npts + k] += w * a2;
      ism[6 * npts + k] += w * (M_[6 * npts + k] - (sn - M_[0 * npts + k]) / im->zpn);
      ism[7 * npts + k] += w * (M_[7 * npts + k] - (a1 - M_[3 * npts + k]) / im->zsn);
      ism[8 * npts + k] += w * (M_[8 * npts + k] - (a2 - M_[5 * npts + k]) / im->zsn);
      isp[0 * npts + k] += w * sn;
      isp[3 * npts + k] += w * a1;
      isp[5 * npts + k] += w * a2;
      isp[6 * npts + k] += w * (P_[6 * npts + k] + (sn - P_[0 * npts + k]) / im->zp);
      isp[7 * npts + k] += w * (P_[7 * npts + k] + (a1 - P_[3 * npts + k]) / im->zs);
      isp[8 * npts + k] += w * (P_[8 * npts + k] + (a2 - P_[5 * npts + k]) / im->zs);
    }
  }
}

/* Newton root of one point for the unit tests (returns iterations; conv set). */
int oracle_dr_newton_point(double a, double psi, double sn, double tau, double inv_etas, double v_start,
                           const oracle_rs_params* P, double* v, int* conv) {
  double mu = 0;
  return newton(P, a, psi, sn, tau, inv_etas, v_start, v, &mu, conv, 0);
}

double oracle_dr_state_update(const oracle_rs_params* P, double a, double psi_ref, double dt, double v) {
  return state_update(P, a, psi_ref, dt, v);
}

double oracle_dr_mu(const oracle_rs_params* P, double a, double psi, double v) {
  const double cl = psi / a;
  return a * arsinhexp(0.5 / P->v0 * v, cl, compute_cexp(cl));
}
