// Dynamic-rupture face kernel: one warp per fault face up to 32 face points (order 4), two warps
// per face up to 64 points (orders 5 and 6: 36 and 49 points); one thread per point; the outer
// fixed point stops per warp, as the reference's GPU solver.
//
// Per face and time step (reference: src/Kernels/DynamicRupture.cpp:57-168 projectToDR,
// src/DynamicRupture/FrictionLaws/GpuImpl/BaseFrictionSolver.h:133-236 evaluatePoint,
// GpuImpl/RateAndState.h:51-270, GpuImpl/FastVelocityWeakeningLaw.h:35-108,
// FrictionSolverCommon.h:146-200 and 333-420, codegen/kernels/dynamic_rupture.py:107-190):
//   1. QInterpolated of both sides at every Gauss-Legendre time point: Taylor evaluation of
//      the stored CK derivatives, rotation by TinvT, evaluation at the face quadrature points;
//   2. fast-velocity-weakening rate-and-state friction per point (lane): Newton on the slip
//      rate inside a fixed point on the state variable; residual, slip rate, state variable
//      and slip accumulation in float64; the fixed point stops when all points of the warp
//      converged (warp vote);
//   3. resampling of the state-variable increment (25x25 face projection);
//   4. time-weighted imposed states of both sides;
//   5. nodal flux Q += V3mTo2nTWDivM(side, rel) . imposed . fluxSolver into both cells.
// An optional small network (5 -> 64 -> 64 -> 1, tanh) proposes the starting slip rate of the
// first Newton solve of every time point: it is used when its residual is below that of the
// plain start (previous slip rate), and the plain solve runs whenever the residual from the
// network's start stops falling.  Optionally (refine32) every solve first iterates in float32 on
// the log slip rate from its start (a few cheap iterations that reach ~1e-6 relative accuracy)
// and the float64 Newton of the reference then only polishes; float64 is the scarce pipe of this
// part.  Optionally the converged first solves of the plain method are recorded as training
// samples (normal stress, shear, state, a, b, log10 V).
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"
#include "mlp.cuh"
#include "_gen/dr_tables_o4.cuh"
#include "_gen/dr_tables_o5.cuh"
#include "_gen/dr_tables_o6.cuh"

namespace {

constexpr int kHidden = sei_mlp::kHidden;
constexpr int kMlpParams = kHidden * 5 + kHidden + kHidden * kHidden + kHidden + kHidden + 1;
constexpr double kAlmostZero = 1e-45;


__device__ __forceinline__ bool largeBranch(double x, double explog) {
  int xexp = 0;
  (void)frexp(x, &xexp);
  return explog + (xexp > 0 ? xexp : 0) * 0.69314718055994530943 > 10.0 || explog >= 50.0;
}

// Natural log of a positive normal double, in float precision, without an FP64 transcendental:
// the binary exponent plus the float log of the mantissa in [1, 2).
__device__ __forceinline__ float lnPos(double v) {
  const long long bits = __double_as_longlong(v);
  const int e = (int)((bits >> 52) & 0x7FF) - 1023;
  const double m = __longlong_as_double((bits & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  return (float)e * 0.6931471806f + logf((float)m);
}

// asinh(x * exp(explog)) with the large-argument form of RateAndStateCommon.h:46-74 (the
// reference passes e = exp(-|explog|), inverted where its branch needs; it is formed here only
// where it is used).  When e < 2^-28 |x| (the usual case: e = exp(-psi / a) is tiny), the rounded
// e^2 is below a quarter ulp of the rounded x^2, so their sum rounds to x^2, whose correctly
// rounded square root is |x| exactly: the float64 square root is skipped with a bit-identical
// result.  A float test in log space with half an e-fold of margin finds that case without the
// float64 exponential; only the cases it cannot decide form e.
__device__ __forceinline__ double arsinhexp(double x, double explog) {
  if (largeBranch(x, explog)) {
    const double xa = fabs(x);
    double s;
    if (explog > 0 && xa > 0 && (float)(-explog) < lnPos(xa) - 19.9084f) {  // 28 ln 2 + 0.5
      s = xa + xa;
    } else {
      double e = exp(-fabs(explog));
      if (explog <= 0) e = 1 / e;
      s = e < 3.7252902984619140625e-9 * xa ? xa + xa : xa + sqrt(xa * xa + e * e);
    }
    return (x >= 0 ? 1.0 : -1.0) * (explog + log(s));
  }
  double e = exp(-fabs(explog));
  if (explog > 0) e = 1 / e;
  return asinh(e * x);
}

// State variable after a sub-step of length dt at slip rate v (RateAndState FVW law).  The
// steady state f_ss, psi_ss and the relaxation weight 1 - exp(-v dt / L) are evaluated in
// float; the state itself is advanced in float64: psi = psiRef + w (psi_ss - psiRef).
// psi_ss = a logsinh(2 V0 / v, f_ss / a) = f_ss - a ln(v / V0) + a ln(1 - exp(-2 f_ss / a)).
// Reciprocals of the law's constants, taken once per thread (float64 divisions are costly).
struct LawInv {
  double v0, vw, l;
};

__device__ double stateUpdate(const sei::DrArgs& A, const LawInv& inv, double a, double psiRef, double dt, double v) {
  const float af = (float)a;
  const float lnvv0 = lnPos(v * inv.v0);
  float lowv = (float)A.f0 - (float)(A.b - a) * lnvv0;
  lowv = lowv > 0.f ? lowv : 0.f;
  const float lnr = lnPos(v * inv.vw);
  const float r8 = expf(fminf(8.f * lnr, 80.f));
  const float fss = (float)A.muw + (lowv - (float)A.muw) * powf(1.f + r8, -0.125f);
  const float c = fss / af;
  const float psiss = fss - af * lnvv0 + af * log1pf(-expf(-2.f * c));
  const float w = -expm1f((float)(-v * dt * inv.l));
  return psiRef + (double)w * ((double)psiss - psiRef);
}

// Newton update delta = -g / g'(V) of the slip rate.  With y = V exp(psi / a) / (2 V0),
// -g'(V) = |sn| a / eta_s * exp(psi / a) / (2 V0) / sqrt(1 + y^2) + 1 = 1 + exp(z), so
// delta = g / (1 + exp(z)), z = ln(|sn| a / eta_s) + ln(exp(psi / a) / (2 V0)) - ln(1 + y^2) / 2.
// z is evaluated in float log space (its terms span hundreds of e-folds, beyond the float
// range as plain numbers); only the residual g needs float64.
__device__ __forceinline__ double newtonDelta(double g, double v, float lnScale, float lnSna) {
  const float ly = lnPos(v) + lnScale;
  float half;  // ln(1 + y^2) / 2
  if (ly > 15.f) {
    half = ly;
  } else if (ly < -15.f) {
    half = 0.f;
  } else {
    const float y = expf(ly);
    half = 0.5f * log1pf(y * y);
  }
  const float z = lnSna + lnScale - half;
  if (z < 20.f) return g * (double)(1.f / (1.f + expf(z)));
  // 1 / (1 + e^z) = e^-z to 2e-9 relative; e^-z = 2^k m with integer k and m in [1, 2)
  const float w = -z * 1.4426950409f;
  const float kf = floorf(w);
  if (kf < -1000.f) return 0.0;
  const double m = (double)exp2f(w - kf);
  const double p2 = __longlong_as_double((long long)((int)kf + 1023) << 52);
  return g * m * p2;
}

struct NewtonOut {
  double v, mu;
  int iters;
  bool conv;
};

// Newton on g(V) = -(|sn| mu(V) - tau) / eta_s - V from v; stops early when |g| grows if bail.
__device__ NewtonOut newton(const sei::DrArgs& A, const LawInv& inv, double a, double inva, double psi, double sn,
                            double tau, double invEtaS, double v, bool bail) {
  const double clin = 0.5 * inv.v0;
  const double cl = psi * inva;
  const float lnScale = (float)cl - lnPos(2.0 * A.v0);
  const float lnSna = logf((float)(invEtaS * fabs(sn) * a));
  double prev = 1e300;
  for (int i = 0; i < A.max_newton; ++i) {
    const double mu = a * arsinhexp(clin * v, cl);
    const double g = -invEtaS * (fabs(sn) * mu - tau) - v;
    if (fabs(g) < A.newton_tol) return {v, mu, i, true};
    if (bail && !(fabs(g) < prev)) return {v, 0.0, i, false};
    prev = fabs(g);
    v = v + newtonDelta(g, v, lnScale, lnSna);
    v = v < kAlmostZero ? kAlmostZero : v;
  }
  return {v, 0.0, A.max_newton, false};
}

// ---- the other rate-and-state laws (law 4 aging, 5 slip, 6 severe velocity weakening) on the
// state variable theta: state updates of CpuImpl/AgingLaw.h, SlipLaw.h and
// SevereVelocityWeakeningLaw.h:14-29; the slow laws' friction is the fast law's asinh form with
// psi = f0 + b ln(V0 theta / L) (SlowVelocityWeakeningLaw.h:38-52).
__device__ double slowStateUpdate(const sei::DrArgs& A, const LawInv& inv, double ref, double dt, double v) {
  if (A.law == 4) {
    const double pre = -v * (dt * inv.l);
    return ref * exp(pre) + A.l / v * -expm1(pre);
  }
  if (A.law == 5) return A.l / v * pow(v * ref * inv.l, exp(-v * (dt * inv.l)));
  const double pre = -A.v0 * (dt * inv.l);
  return v * A.l * inv.v0 * -expm1(pre) + exp(pre) * ref;
}

__device__ __forceinline__ double psiEff(const sei::DrArgs& A, const LawInv& inv, double state) {
  return A.law == 0 ? state : A.f0 + A.b * log(A.v0 * state * inv.l);
}

// Severe velocity weakening: mu = f0 + a V / (V + V0) - b theta / (theta + L), generic Newton
// (RateAndState.h:327-385).
__device__ NewtonOut newtonSvw(const sei::DrArgs& A, double a, double theta, double sn, double tau, double invEtaS,
                               double v) {
  const double c = A.b * theta / (theta + A.l);
  for (int i = 0; i < A.max_newton; ++i) {
    const double mu = A.f0 + a * v / (v + A.v0) - c;
    const double g = -invEtaS * (fabs(sn) * mu - tau) - v;
    if (fabs(g) < A.newton_tol) return {v, mu, i, true};
    const double d = v + A.v0;
    const double dg = -invEtaS * (fabs(sn) * a * A.v0 / (d * d)) - 1.0;
    v = v - g / dg;
    v = v < kAlmostZero ? kAlmostZero : v;
  }
  return {v, 0.0, A.max_newton, false};
}

// ---- float32 solve on u = ln V.  h(u) = |sn| a asinh(e^(u + lnScale)) + eta_s e^u - tau is -eta_s
// times the residual g and increasing and convex in u, so Newton converges from either side once
// it is right of the root.  asinh(y) = ln(2 y) beyond y = e^9 (error below 4e-9) and y below
// y = e^-9 (relative error below 3e-9).
struct Solve32 {
  float an, etas, tau, lnScale;  // |sn| a, eta_s, tau, psi / a - ln(2 V0)
};
__device__ __forceinline__ float h32(const Solve32& S, float u, float* dh) {
  const float ly = u + S.lnScale;
  float ash, dash;  // asinh(y), y / sqrt(1 + y^2)
  if (ly > 9.f) {
    ash = ly + 0.6931471806f;
    dash = 1.f;
  } else if (ly < -9.f) {
    ash = dash = expf(ly);
  } else {
    const float y = expf(ly);
    const float r = sqrtf(fmaf(y, y, 1.f));
    ash = asinhf(y);
    dash = y / r;
  }
  const float ev = expf(u);
  if (dh) *dh = fmaf(S.an, dash, S.etas * ev);
  return fmaf(S.an, ash, fmaf(S.etas, ev, -S.tau));
}
// range of a start of the float64 solve, natural log of m/s (1e-45 .. 1e3)
constexpr float kLnGuessMinF = -103.616329f, kLnGuessMaxF = 6.907755f;
__device__ __forceinline__ float newton32(const Solve32& S, float u, int& its) {
  its = 0;
#pragma unroll 1
  for (int i = 0; i < 16; ++i) {
    float dh;
    const float h = h32(S, u, &dh);
    const float du = h / dh;
    u = fminf(fmaxf(u - du, kLnGuessMinF), kLnGuessMaxF);
    its = i + 1;
    // a step at the float resolution of u (h carries a few ulp of tau): converged; also leaves on NaN
    if (!(fabsf(du) > 1e-6f + 3e-7f * fabsf(u))) break;
  }
  return u;
}
// e^u as a double from float arithmetic: 2^k m with integer k and m = 2^(w - k) in [1, 2).
__device__ __forceinline__ double expToDouble(float u) {
  const float w = u * 1.4426950409f;
  const float kf = floorf(w);
  const double m = (double)exp2f(w - kf);
  return m * __longlong_as_double((long long)((int)kf + 1023) << 52);
}

__device__ __forceinline__ float tanhApprox(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Network guess of ln V in float arithmetic: the features and output map of mlp.cuh evaluated in
// float (the training side uses float64; the guess only seeds a solve), tanh.approx activations.
__device__ float mlpGuess32(const float* __restrict__ w, const float* nrm, float sn, float tau, float psi, float a,
                            float b) {
  float an = fabsf(sn) * a;
  an = an > 1.f ? an : 1.f;
  const float f[5] = {tau / an, psi / a, logf(an), a, b};
  float x[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) x[i] = (f[i] - nrm[i]) * nrm[5 + i];
  const float* W1 = w;
  const float* b1 = W1 + kHidden * 5;
  const float* W2 = b1 + kHidden;
  const float* b2 = W2 + kHidden * kHidden;
  const float* W3 = b2 + kHidden;
  float h1[kHidden];
#pragma unroll 8
  for (int j = 0; j < kHidden; ++j) {
    float s = b1[j];
#pragma unroll
    for (int i = 0; i < 5; ++i) s = fmaf(W1[j * 5 + i], x[i], s);
    h1[j] = tanhApprox(s);
  }
  float out = W3[kHidden];
#pragma unroll 4
  for (int j = 0; j < kHidden; ++j) {
    float s = b2[j];
#pragma unroll
    for (int i = 0; i < kHidden; ++i) s = fmaf(W2[j * kHidden + i], h1[i], s);
    out = fmaf(W3[j], tanhApprox(s), out);
  }
  const float z = f[0] - f[1] - f[2];
  const float base = z > 30.f ? z : log1pf(expf(z));
  return nrm[12] + f[0] - f[1] - base - (out * nrm[11] + nrm[10]);
}

// Threads of one face (a multiple of the warp size covering the face points), faces per block.
template <int NP>
struct FaceGroup {
  static constexpr int kThreads = NP <= 32 ? 32 : 64;
  static constexpr int kFaces = 128 / kThreads;
  static_assert(NP <= 64, "at most 64 points per face");
};

// Barrier of the threads of face slot fs: the warp itself, or named barrier 1 + fs of two warps.
template <int TPF>
__device__ __forceinline__ void faceSync(int fs) {
  if constexpr (TPF == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;\n" ::"r"(1 + fs), "n"(TPF) : "memory");
  }
}

// Convergence vote of the outer fixed point: over the warp, i.e. a group of 32 consecutive face
// points, as the reference's GPU friction solver (deviceWarpAll, GpuImpl/RateAndState.h:138-142);
// the two warps of a face at orders 5 and 6 leave the loop independently.
__device__ __forceinline__ bool warpAll(bool c) { return __all_sync(0xffffffffu, c); }

// smoothStep of the Gaussian nucleation (src/Numerical/GaussianNucleationFunction.h).
__device__ double smoothStep(double t, double t0) {
  if (t <= 0.0) return 0.0;
  if (t < t0) {
    const double tau = t - t0;
    return exp(tau * tau / (t * (t - 2.0 * t0)));
  }
  return 1.0;
}

// ---- thermal pressurisation (CpuImpl/ThermalPressurization/ThermalPressurization.cpp:27-107,
// TPCommon.h): wave numbers 10 e^(-0.3 (59 - i)), inverse-transform weights, Gaussian heat source
__device__ double gTp[3][sei::kTpModes];

__global__ void sei_tp_tables() {
  const int i = threadIdx.x;
  if (i >= sei::kTpModes) return;
  const double k = 10.0 * exp(-0.3 * (sei::kTpModes - i - 1));
  const double c = sqrt(2.0 / M_PI) * k;
  gTp[0][i] = k;
  gTp[1][i] = i == 0 ? c * (1.0 + 0.3) : (i == sei::kTpModes - 1 ? c * 0.5 * 0.3 : c * 0.3);
  gTp[2][i] = 1.0 / sqrt(2.0 * M_PI) * exp(-0.5 * k * k);
}

// Fluid pressure of point po after dt at slip rate v, friction mu and normal stress sn; the modes
// advance only with save.  temp receives the temperature.
__device__ double tpPressure(const sei::DrArgs& A, size_t po, size_t plane, double hw, double hyd, double sn,
                             double mu, double v, double dt, bool save, double& temp) {
  const double tauv = -mu * sn * v;
  const double lp = A.tp_lambda * A.tp_alpha / (hyd - A.tp_alpha);
  double tu = 0.0, pu = 0.0;
#pragma unroll 1
  for (int m = 0; m < sei::kTpModes; ++m) {
    const double g = gTp[0][m] / hw;
    const double g2 = g * g;
    const double th = A.tp_alpha * g2, sg = hyd * g2;
    const double om = tauv * gTp[2][m];
    double* pt = A.tp_theta + (size_t)m * plane + po;
    double* ps = A.tp_sigma + (size_t)m * plane + po;
    const double tn = *pt * exp(-th * dt) + om / (A.tp_rhoc * th) * -expm1(-th * dt);
    const double sn2 = *ps * exp(-sg * dt) + om * (A.tp_lambda + lp) / (A.tp_rhoc * sg) * -expm1(-sg * dt);
    const double w = gTp[1][m] / hw;
    tu += w * tn;
    pu += w * sn2;
    if (save) {
      *pt = tn;
      *ps = sn2;
    }
  }
  pu -= lp * tu;
  temp = tu + A.tp_t0;
  return -pu + A.tp_p0;
}

// Regularised Yoffe function: the Yoffe slip-rate function of rise time tau_R convolved with a
// triangle of half width tau_S (Tinti et al. 2005, closed form; Numerical/RegularizedYoffe.h).
__device__ double regularizedYoffe(double t, double tS, double tR) {
  const double k = 2.0 / (M_PI * tR * tS * tS);
  auto c1 = [&] {
    return (0.5 * t + 0.25 * tR) * sqrt(t * (tR - t)) + (t * tR - tR * tR) * asin(sqrt(t / tR)) -
           0.75 * tR * tR * atan(sqrt((tR - t) / t));
  };
  auto c2 = [&] { return 0.375 * M_PI * tR * tR; };
  auto c3 = [&] {
    return (tS - t - 0.5 * tR) * sqrt((t - tS) * (tR - t + tS)) + tR * (2.0 * tR - 2.0 * t + 2.0 * tS) * asin(sqrt((t - tS) / tR)) +
           1.5 * tR * tR * atan(sqrt((tR - t + tS) / (t - tS)));
  };
  auto c4 = [&] {
    return (-tS + 0.5 * t + 0.25 * tR) * sqrt((t - 2.0 * tS) * (tR - t + 2.0 * tS)) -
           tR * (tR - t + 2.0 * tS) * asin(sqrt((t - 2.0 * tS) / tR)) -
           0.75 * tR * tR * atan(sqrt((tR - t + 2.0 * tS) / (t - 2.0 * tS)));
  };
  auto c5 = [&] { return 0.5 * M_PI * tR * (t - tR); };
  auto c6 = [&] { return 0.5 * M_PI * tR * (2.0 * tS - t + tR); };
  if (t <= 0.0 || t >= tR + 2.0 * tS) return 0.0;
  if (t <= tS) return k * (c1() + c2());
  if (tR > 2.0 * tS) {
    if (t <= 2.0 * tS) return k * (c1() - c2() + c3());
    if (t < tR) return k * (c1() + c3() + c4());
    if (t < tR + tS) return k * (c3() + c4() + c5());
    return k * (c4() + c6());
  }
  if (t < tR) return k * (c1() - c2() + c3());
  if (t <= 2.0 * tS) return k * (c5() + c3() - c2());
  if (t < tR + tS) return k * (c3() + c4() + c5());
  return k * (c4() + c6());
}

// FAM 0: rate and state with fast velocity weakening (Newton solve of the slip rate, resampled
// state increment); FAM 1: the other rate-and-state laws, 4 aging, 5 slip, 6 severe velocity
// weakening (state kept as it is); FAM 2: linear slip weakening (law 1: resampled slip rate;
// 2: bimaterial regularised strength; 3: TP proxy state), CpuImpl/LinearSlipWeakening.h:27-170;
// FAM 3: imposed slip rates (7 Yoffe, 8 Gaussian, 9 delta), CpuImpl/ImposedSlipRates.h:21-60.
template <int N, int B, int NP, int FAM, bool TPK>
__global__ void __launch_bounds__(128, 3)
    sei_dr_faces(sei::DrArgs A, const float* __restrict__ V3m, const float* __restrict__ TW,
                 const double* __restrict__ R) {
  constexpr bool RS = FAM <= 1;
  constexpr int TPF = FaceGroup<NP>::kThreads, FPB = FaceGroup<NP>::kFaces;
  constexpr int Bp = (B + 3) / 4 * 4;
  constexpr int kQsel[6] = {0, 3, 5, 6, 7, 8};
  int dsz = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) dsz += (N - i) * (N - i + 1) * (N - i + 2) / 6 * 9;
  __shared__ float sI[FPB][B * 9];
  __shared__ float sJ[FPB][B * 9];
  __shared__ float sG[FPB][NP * 9];
  __shared__ double sD[FPB][TPF];
  __shared__ float sW[FAM == 0 ? kMlpParams : 1];
  const bool useMlp = FAM == 0 && !TPK && A.mlp != nullptr;
  if (useMlp)
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sW[i] = A.mlp[i];
  __syncthreads();
  // face slot and thread of the face (every thread of a face leaves or stays together)
  const int warp = threadIdx.x / TPF, lane = threadIdx.x % TPF;
  const int fi = blockIdx.x * FPB + warp;
  if (fi >= A.face_count) return;
  const int f = A.fidx ? A.fidx[A.face_begin + fi] : A.face_begin + fi;
  if (f < 0 || f >= A.nfaces) return;
  const bool pt = lane < NP;
  const int k = pt ? lane : 0;

  // ---- 1. space-time interpolation of both sides at time point s (six quantities per point),
  // evaluated inside the friction loop so that only one time point is live at a time
  const float* Tf = A.tinvt + (size_t)f * 81;
  auto interpolate = [&](int s, float (&qs)[2][6]) {
#pragma unroll 1
    for (int sd = 0; sd < 2; ++sd) {
      const int slot = sd == 0 ? A.plus_slot[f] : A.minus_slot[f];
      const int combo = sd == 0 ? A.plus_side[f] * 4 : A.minus_side[f] * 4 + A.rel[f];
      const float* d = A.derivs + (size_t)slot * dsz;
      const float* V = V3m + (size_t)combo * NP * B;
      for (int e = lane; e < B * 9; e += TPF) {
        const int l = e % B, q = e / B;
        float v = 0.f;
        int off = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int bi = (N - i) * (N - i + 1) * (N - i + 2) / 6;
          if (l < bi) v = fmaf(A.coll[s][i], __ldg(d + off + l + bi * q), v);
          off += bi * 9;
        }
        sI[warp][q * B + l] = v;
      }
      faceSync<TPF>(warp);
      for (int e = lane; e < B * 9; e += TPF) {
        const int l = e % B, p = e / B;
        float v = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) v = fmaf(sI[warp][q * B + l], __ldg(Tf + q + 9 * p), v);
        sJ[warp][p * B + l] = v;
      }
      faceSync<TPF>(warp);
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        float v = 0.f;
        for (int l = 0; l < B; ++l) v = fmaf(__ldg(V + k * B + l), sJ[warp][kQsel[j] * B + l], v);
        qs[sd][j] = v;
      }
      faceSync<TPF>(warp);
    }
  };

  // ---- 2. friction (lanes < NP own one point each), per time point as the evaluate loop of
  // CpuImpl/BaseFrictionLaw.h:103-137: nucleation, friction, rupture-front and peak outputs
  const size_t po = (size_t)f * NP + k;
  const double* imp = A.imp + (size_t)f * 8;
  const double etap = imp[4], etas = imp[5], invEtaS = imp[6];
  // reciprocal impedances, once per thread: FP64 divisions are costly on this part
  const double rzp = 1.0 / imp[0], rzs = 1.0 / imp[1], rzpn = 1.0 / imp[2], rzsn = 1.0 / imp[3];
  const double a = RS && pt ? A.a[po] : 0.01;
  const double inva = 1.0 / a;  // psi / a as psi * inva: one float64 division per thread, not per solve
  const size_t plane = (size_t)A.nfaces * NP;  // init holds sn0, tau1_0, tau2_0 as [3][nf][npts]
  double sn0 = pt ? A.init[po] : 0.0;
  double t10 = pt ? A.init[plane + po] : 0.0;
  double t20 = pt ? A.init[2 * plane + po] : 0.0;
  const bool nucleating = A.nucleate != 0;
  const double nsn = nucleating && pt ? A.nuc[po] : 0.0;
  const double nt1 = nucleating && pt ? A.nuc[plane + po] : 0.0;
  const double nt2 = nucleating && pt ? A.nuc[2 * plane + po] : 0.0;
  double psiStored = RS && pt ? A.psi[po] : 0.0;
  double psib = psiStored;
  double v1 = pt ? A.v1[po] : 1.0, v2 = pt ? A.v2[po] : 0.0;
  double slip1 = pt ? A.slip1[po] : 0.0, slip2 = pt ? A.slip2[po] : 0.0, slip = pt ? A.slip[po] : 0.0;
  double mu = (FAM == 2 || TPK) && pt ? A.mu[po] : 0.0, tr1 = 0.0, tr2 = 0.0;
  // thermal pressurisation: pressure and temperature of the point, its zone width and diffusivity
  double tpP = TPK && pt ? A.tp_pres[po] : 0.0, tpT = TPK && pt ? A.tp_temp[po] : 0.0;
  const double tpHw = TPK && pt ? A.tp_hw[po] : 1.0, tpHyd = TPK && pt ? A.tp_hyd[po] : 1.0;
  double peak = pt ? A.peak[po] : 0.0, trup = pt ? A.trup[po] : 0.0;
  // slip weakening fields
  const double muS = FAM == 2 && pt ? A.mu_s[po] : 0.0, muD = FAM == 2 && pt ? A.mu_d[po] : 0.0;
  const double dc = FAM == 2 && pt ? A.d_c[po] : 1.0, coh = FAM == 2 && pt ? A.cohesion[po] : 0.0;
  const double tForced = FAM == 2 && pt ? A.t_forced[po] : 0.0;
  double tdyn = FAM == 2 && pt ? A.tdyn[po] : 0.0;
  double reg = FAM == 2 && pt && A.law == 2 ? A.reg[po] : 0.0;
  // imposed slip rates
  const double dir1 = FAM == 3 && pt ? A.dir1[po] : 0.0, dir2 = FAM == 3 && pt ? A.dir2[po] : 0.0;
  const double onset = FAM == 3 && pt ? A.onset[po] : 0.0;
  const double tauS = FAM == 3 && pt ? A.taus[po] : 1.0, tauR = FAM == 3 && pt ? A.taur[po] : 1.0;
  double vmag = sqrt(v1 * v1 + v2 * v2);  // slip-rate magnitude of the previous time point (slip weakening)
  double tStart = (A.time ? *A.time : 0.0) + A.time_offset;
  int iters = 0, firstIters = 0, iters32 = 0;
  const LawInv inv{1.0 / A.v0, 1.0 / A.vw, 1.0 / A.l};
  double isP[6] = {0, 0, 0, 0, 0, 0}, isM[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 1
  for (int s = 0; s < N; ++s) {
    float qc[2][6];
    interpolate(s, qc);
    const double dt = A.deltat[s];
    const double tEnd = tStart + dt;
    // nucleation (FrictionSolverCommon.h:503-531) before the friction of this time point
    if (nucleating && tEnd <= A.t0 + A.s0 && tEnd >= A.s0) {
      const double g = smoothStep(tEnd - A.s0, A.t0) - smoothStep(tEnd - A.s0 - dt, A.t0);
      sn0 += nsn * g;
      t10 += nt1 * g;
      t20 += nt2 * g;
    }
    // precompute stress (etaPDamp = 1): qi order N, T1, T2, U, V, W
    const double fsn = etap * ((double)qc[1][3] - qc[0][3] + qc[0][0] * rzp + qc[1][0] * rzpn);
    const double ft1 = etas * ((double)qc[1][4] - qc[0][4] + qc[0][1] * rzs + qc[1][1] * rzsn);
    const double ft2 = etas * ((double)qc[1][5] - qc[0][5] + qc[0][2] * rzs + qc[1][2] * rzsn);
    const double tt1 = t10 + ft1, tt2 = t20 + ft2;
    const double tau = sqrt(tt1 * tt1 + tt2 * tt2);
    if constexpr (RS) {
      double sn = fsn + sn0 - tpP;  // effective normal stress (RateAndState.h:420-432)
      sn = sn < 0 ? sn : 0.0;
      const double sref = psib;
      vmag = sqrt(v1 * v1 + v2 * v2);  // RateAndState.h:150-153
      vmag = vmag < kAlmostZero ? kAlmostZero : vmag;
      double lsr = vmag;
#pragma unroll 1
      for (int j = 0; j < A.max_outer; ++j) {
        bool conv = true;
        if (pt) {
          NewtonOut r{};
          bool done = false;
          double pe;
          if constexpr (TPK) {
            // the pressure of this pass from the previous pass's stress and friction
            tpP = tpPressure(A, po, plane, tpHw, tpHyd, sn, mu, lsr, dt, false, tpT);
            sn = fsn + sn0 - tpP;
            sn = sn < 0 ? sn : 0.0;
          }
          if constexpr (FAM == 0) {
            psib = stateUpdate(A, inv, a, sref, dt, lsr);
            pe = psib;
          } else {
            psib = slowStateUpdate(A, inv, sref, dt, lsr);
            pe = psiEff(A, inv, psib);
            if (A.law == 6) {
              r = newtonSvw(A, a, psib, sn, tau, invEtaS, vmag);
              (j == 0 ? firstIters : iters) += r.iters;
              done = true;
            }
          }
          const bool net = useMlp && j == 0 && sei_mlp::usable(sn, tau, a);
          if (FAM == 0 && !TPK && (net || A.refine32)) {
            const Solve32 S{(float)(fabs(sn) * a), (float)etas, (float)tau, (float)(psib * inva) - lnPos(2.0 * A.v0)};
            const float u0 = lnPos(vmag);
            float u = u0;
            if (net) {
              // start from the network's guess when its residual is below the plain start's
              // (float32 residuals: the comparison only picks a start)
              const float lg = mlpGuess32(sW, A.mlp_norm, (float)sn, (float)tau, (float)psib, (float)a, (float)A.b);
              const float ug = fminf(fmaxf(lg, kLnGuessMinF), kLnGuessMaxF);
              if (fabsf(h32(S, ug, nullptr)) < fabsf(h32(S, u, nullptr))) u = ug;
            }
            if (A.refine32) {
              int its = 0;
              u = newton32(S, u, its);
              iters32 += its;
            }
            // a start that float arithmetic cannot tell from the previous slip rate is not taken: the
            // previous rate is often the float64 root already (no iteration at all)
            if (!(fabsf(u - u0) <= 2e-6f + 6e-7f * fabsf(u0))) {
              r = newton(A, inv, a, inva, psib, sn, tau, invEtaS, expToDouble(u), true);
              (j == 0 ? firstIters : iters) += r.iters;
              done = r.conv;
            }
          }
          if (!done) {
            r = newton(A, inv, a, inva, pe, sn, tau, invEtaS, vmag, false);
            (j == 0 ? firstIters : iters) += r.iters;
            if (FAM == 0 && A.rec && j == 0 && r.conv && sei_mlp::usable(sn, tau, a)) {
              const unsigned idx = atomicAdd(A.rec_count, 1u);
              if (idx < A.rec_cap) {
                float* o = A.rec + (size_t)idx * 6;
                o[0] = (float)sn;
                o[1] = (float)tau;
                o[2] = (float)psib;
                o[3] = (float)a;
                o[4] = (float)A.b;
                o[5] = (float)log10(r.v);
              }
            }
          }
          lsr = 0.5 * (vmag + r.v);
          conv = fabs(vmag - r.v) < A.state_tol;
          vmag = r.v;
          mu = r.mu;
        }
        if (warpAll(conv)) break;
      }
      if (pt) {
        if constexpr (TPK) {
          // the modes advance with the final pass's slip rate and friction
          tpP = tpPressure(A, po, plane, tpHw, tpHyd, sn, mu, lsr, dt, true, tpT);
          sn = fsn + sn0 - tpP;
          sn = sn < 0 ? sn : 0.0;
        }
        if constexpr (FAM == 0) {
          psib = stateUpdate(A, inv, a, sref, dt, lsr);
          mu = a * arsinhexp(0.5 * inv.v0 * vmag, psib * inva);
        } else {
          psib = slowStateUpdate(A, inv, sref, dt, lsr);
          if (A.law == 6)
            mu = A.f0 + a * vmag / (vmag + A.v0) - A.b * psib / (psib + A.l);
          else
            mu = a * arsinhexp(0.5 * inv.v0 * vmag, psiEff(A, inv, psib) * inva);
        }
        const double strength = -mu * sn;
        slip += vmag * dt;
        const double div = strength + etas * vmag;
        const double vd = vmag / div;
        v1 = vd * tt1;
        v2 = vd * tt2;
        tr1 = ft1 - etas * v1;
        tr2 = ft2 - etas * v2;
        slip1 += v1 * dt;
        slip2 += v2 * dt;
      }
    } else if constexpr (FAM == 3) {
      // the source time function at the time point's end (SourceTimeFunction.cpp)
      const double t = tEnd - onset;
      double stf;
      if (A.law == 7)
        stf = regularizedYoffe(t, tauS, tauR);
      else if (A.law == 8)
        stf = (smoothStep(t, tauS) - smoothStep(t - dt, tauS)) / dt;
      else
        stf = t > 0.0 && t <= dt ? 1.0 / dt : 0.0;
      v1 = dir1 * stf;
      v2 = dir2 * stf;
      tr1 = ft1 - etas * v1;
      tr2 = ft2 - etas * v2;
      vmag = sqrt(v1 * v1 + v2 * v2);
      slip1 += v1 * dt;
      slip2 += v2 * dt;
      slip += vmag * dt;
    } else {
      // strength from the friction coefficient of the previous time point
      const double snt = sn0 + fsn;
      double strength = -coh - mu * (snt < 0.0 ? snt : 0.0);
      if (A.law == 2) {
        const double e = -((vmag > 0.0 ? vmag : 0.0) + A.v_star) * dt / A.prakash_length;
        strength = reg * exp(e) + strength * -expm1(e);
        reg = strength;
      }
      double v = (tau - strength) * invEtaS;
      v = v > 0.0 ? v : 0.0;
      const double div = strength + etas * v;
      v1 = v * tt1 / div;
      v2 = v * tt2 / div;
      tr1 = ft1 - etas * v1;
      tr2 = ft2 - etas * v2;
      slip1 += v1 * dt;
      slip2 += v2 * dt;
      vmag = v;
      // the accumulated slip grows by the slip rate resampled over the face (law 1)
      double rv = v;
      if (A.law == 1) {
        sD[warp][lane] = pt ? v : 0.0;
        faceSync<TPF>(warp);
        rv = 0.0;
        for (int j = 0; j < NP; ++j) rv += R[k * NP + j] * sD[warp][j];
        faceSync<TPF>(warp);
      }
      slip += rv * dt;
      const double ratio = fabs(slip) / dc;
      double state = A.law == 3 ? 1.0 - pow(1.0 + ratio, -A.tp_exponent) : (ratio < 1.0 ? ratio : 1.0);
      double f2;
      if (A.t0 == 0.0) {
        f2 = tEnd >= tForced ? 1.0 : 0.0;
      } else {
        f2 = (tEnd - tForced) / A.t0;
        f2 = f2 < 0.0 ? 0.0 : (f2 > 1.0 ? 1.0 : f2);
      }
      state = state > f2 ? state : f2;
      mu = muS - (muS - muD) * state;
      if (peak > A.healing && v < A.healing) mu = muS;
      if (tdyn < 0.0 && fabs(slip) >= dc) tdyn = tStart;
    }
    if (pt) {
      // rupture front and peak slip rate (FrictionSolverCommon.h:546-592)
      if (trup < 0.0 && vmag > 0.001) trup = tStart;
      peak = vmag > peak ? vmag : peak;
      const double w = A.tweights[s];
      isM[0] += w * fsn;
      isM[1] += w * tr1;
      isM[2] += w * tr2;
      isM[3] += w * (qc[1][3] - (fsn - qc[1][0]) * rzpn);
      isM[4] += w * (qc[1][4] - (tr1 - qc[1][1]) * rzsn);
      isM[5] += w * (qc[1][5] - (tr2 - qc[1][2]) * rzsn);
      isP[0] += w * fsn;
      isP[1] += w * tr1;
      isP[2] += w * tr2;
      isP[3] += w * (qc[0][3] + (fsn - qc[0][0]) * rzp);
      isP[4] += w * (qc[0][4] + (tr1 - qc[0][1]) * rzs);
      isP[5] += w * (qc[0][5] + (tr2 - qc[0][2]) * rzs);
    }
    tStart = tEnd;
  }

  // ---- 3. resample the state-variable increment over the face (fast rate and state; the other
  // rate-and-state laws keep their state as it is, SlowVelocityWeakeningLaw.h:66-72)
  if constexpr (RS) {
    constexpr bool resample = FAM == 0;
    if constexpr (resample) {
      sD[warp][lane] = pt ? psib - psiStored : 0.0;
      faceSync<TPF>(warp);
    }
    if (pt) {
      double v = 0.0;
      if constexpr (resample)
        for (int j = 0; j < NP; ++j) v += R[k * NP + j] * sD[warp][j];
      A.psi[po] = resample ? psiStored + v : psib;
      A.newton_iters[po] += iters + firstIters;
      A.newton_iters[(size_t)A.nfaces * NP + po] += firstIters;
      A.newton_iters[2 * (size_t)A.nfaces * NP + po] += iters32;
    }
  } else if (FAM == 2 && pt) {
    A.tdyn[po] = tdyn;
    if (A.law == 2) A.reg[po] = reg;
  }
  if (pt) {
    if constexpr (TPK) {
      A.tp_pres[po] = tpP;
      A.tp_temp[po] = tpT;
    }
    if (nucleating) {
      A.init[po] = sn0;
      A.init[plane + po] = t10;
      A.init[2 * plane + po] = t20;
    }
    A.peak[po] = peak;
    A.trup[po] = trup;
    A.v1[po] = v1;
    A.v2[po] = v2;
    A.slip1[po] = slip1;
    A.slip2[po] = slip2;
    A.slip[po] = slip;
    A.mu[po] = mu;
    A.trac1[po] = tr1;
    A.trac2[po] = tr2;
  }

  // ---- 4./5. imposed states and nodal flux, plus side then minus side
#pragma unroll 1
  for (int sd = 0; sd < 2; ++sd) {
    const double* is = sd == 0 ? isP : isM;
    float* isOut = (sd == 0 ? A.isp : A.ism) + (size_t)f * 9 * NP;
    const float* fs = (sd == 0 ? A.fsp : A.fsm) + (size_t)f * 81;
    if (pt) {
      float full[9] = {(float)is[0], 0.f, 0.f, (float)is[1], 0.f, (float)is[2], (float)is[3], (float)is[4], (float)is[5]};
#pragma unroll
      for (int q = 0; q < 9; ++q) isOut[q * NP + k] = full[q];
#pragma unroll
      for (int p = 0; p < 9; ++p) {
        float g = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) g = fmaf(full[q], __ldg(fs + q + 9 * p), g);
        sG[warp][k * 9 + p] = g;
      }
    }
    faceSync<TPF>(warp);
    const int cell = sd == 0 ? A.plus_cell[f] : A.minus_cell[f];
    const int combo = sd == 0 ? A.plus_side[f] * 4 : A.minus_side[f] * 4 + A.rel[f];
    const float* W = TW + (size_t)combo * B * NP;
    float* q = A.Q + (size_t)cell * 9 * Bp;
    for (int e = lane; e < B * 9; e += TPF) {
      const int l = e % B, p = e / B;
      float v = 0.f;
      for (int kk = 0; kk < NP; ++kk) v = fmaf(__ldg(W + l * NP + kk), sG[warp][kk * 9 + p], v);
      atomicAdd(q + p * Bp + l, v);  // a cell may have several fault faces, in other CTAs
    }
    faceSync<TPF>(warp);
  }
}

template <int N, int B, int NP>
int launch(const sei::DrArgs& a, const float* v3m, const float* tw, const double* res, void* stream) {
  if (a.face_count <= 0) return 0;
  if (a.law < 0 || a.law > 9 || !a.peak || !a.trup || (a.nucleate && !a.nuc) ||
      (a.law >= 1 && a.law <= 3 && (!a.mu_s || !a.mu_d || !a.d_c || !a.cohesion || !a.t_forced || !a.tdyn)) ||
      (a.law == 2 && !a.reg) || (a.law >= 7 && (!a.dir1 || !a.dir2 || !a.onset || !a.taus || !a.taur)) ||
      (a.tp && ((a.law != 0 && (a.law < 4 || a.law > 6)) || !a.tp_hw || !a.tp_hyd || !a.tp_theta || !a.tp_sigma ||
                !a.tp_temp || !a.tp_pres)))
    return -1;
  constexpr int FPB = FaceGroup<NP>::kFaces;
  const int blocks = (a.face_count + FPB - 1) / FPB;
  cudaStream_t st = (cudaStream_t)stream;
  if (a.law == 0 && a.tp)
    sei_dr_faces<N, B, NP, 0, true><<<blocks, 128, 0, st>>>(a, v3m, tw, res);
  else if (a.law == 0)
    sei_dr_faces<N, B, NP, 0, false><<<blocks, 128, 0, st>>>(a, v3m, tw, res);
  else if (a.law >= 4 && a.law <= 6 && a.tp)
    sei_dr_faces<N, B, NP, 1, true><<<blocks, 128, 0, st>>>(a, v3m, tw, res);
  else if (a.law >= 4 && a.law <= 6)
    sei_dr_faces<N, B, NP, 1, false><<<blocks, 128, 0, st>>>(a, v3m, tw, res);
  else if (a.law >= 7)
    sei_dr_faces<N, B, NP, 3, false><<<blocks, 128, 0, st>>>(a, v3m, tw, res);
  else
    sei_dr_faces<N, B, NP, 2, false><<<blocks, 128, 0, st>>>(a, v3m, tw, res);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

__global__ void sei_dr_advance_time(double* t, double dt) { *t += dt; }

template <typename T>
const T* symbolAddress(const T& sym) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, sym) != cudaSuccess) return nullptr;
  return static_cast<const T*>(p);
}

}  // namespace

namespace sei {

int drNumPoints(int order) { return (order + 1) * (order + 1); }

int launchTpTables(void* stream) {
  sei_tp_tables<<<1, kTpModes, 0, (cudaStream_t)stream>>>();
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchDrAdvanceTime(double* t, double dt, void* stream) {
  sei_dr_advance_time<<<1, 1, 0, (cudaStream_t)stream>>>(t, dt);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launchDrFaces(int order, const DrArgs& a, void* stream) {
  // One thread per face point: orders 4 (25 points), 5 (36) and 6 (49).  Device addresses of
  // the generated tables are looked up here (host code may not take them directly).
  void *v = nullptr, *t = nullptr, *r = nullptr;
  switch (order) {
    case 4:
      if (cudaGetSymbolAddress(&v, sei_dr_o4::kV3m) || cudaGetSymbolAddress(&t, sei_dr_o4::kTW) ||
          cudaGetSymbolAddress(&r, sei_dr_o4::kResample))
        return -1;
      return launch<4, 20, 25>(a, (const float*)v, (const float*)t, (const double*)r, stream);
    case 5:
      if (cudaGetSymbolAddress(&v, sei_dr_o5::kV3m) || cudaGetSymbolAddress(&t, sei_dr_o5::kTW) ||
          cudaGetSymbolAddress(&r, sei_dr_o5::kResample))
        return -1;
      return launch<5, 35, 36>(a, (const float*)v, (const float*)t, (const double*)r, stream);
    case 6:
      if (cudaGetSymbolAddress(&v, sei_dr_o6::kV3m) || cudaGetSymbolAddress(&t, sei_dr_o6::kTW) ||
          cudaGetSymbolAddress(&r, sei_dr_o6::kResample))
        return -1;
      return launch<6, 56, 49>(a, (const float*)v, (const float*)t, (const double*)r, stream);
    default:
      return -1;
  }
}

}  // namespace sei
