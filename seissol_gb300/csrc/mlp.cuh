// Fixed input and output maps of the slip-rate warm-start network (shared by the fault kernel,
// the training kernels and the host normalisation).
//
// The residual of the rate-and-state solve, |sn| a asinh(V exp(psi/a) / (2 V0)) + eta_s V = tau,
// depends on the five raw inputs (normal stress sn, absolute shear traction tau, state variable
// psi, a, b) mostly through the dimensionless groups s = tau / (|sn| a) and f = psi / a: with
// w = ln(V exp(f) / (2 V0)) the locked branch is w = ln sinh(s) and radiation damping lowers it.
// t = s - w = ln(2 V0) + s - f - ln V is ln 2 on the locked branch and grows with slope one in
// z = s - f - ln(|sn| a) once radiation damping dominates (a Lambert-W shape in e^z).  The network
// sees the features (s, f, ln(|sn| a), a, b) and predicts the bounded remainder
// r = t - softplus(z); ln V itself spans ~100 units, r a few.  Normalisation norm[16]: feature
// shifts [0..4], feature scales [5..9], output shift [10], output scale [11], ln(2 V0) [12],
// [13..15] zero.
#pragma once
#include <cmath>

namespace sei_mlp {

constexpr int kHidden = 64;
constexpr int kNorm = 16;
constexpr double kLn10 = 2.302585092994045684;

// The network is neither trained nor evaluated where tau >= 500 |sn| a (among them the opening
// fault, sn = 0): friction is then negligible against the shear traction, the residual is nearly
// linear in V, the plain start converges in a step or two, and such far-out features would only
// stretch the normalisation of the rest.
constexpr double kMaxStressRatio = 500.0;
__host__ __device__ inline bool usable(double sn, double tau, double a) {
  const double an = fabs(sn) * a;
  return an > 1.0 && tau < kMaxStressRatio * an;
}

__host__ __device__ inline void features(double sn, double tau, double psi, double a, double b, double f[5]) {
  double an = fabs(sn) * a;
  an = an > 1.0 ? an : 1.0;  // 1 Pa floor: an opening fault (sn = 0) gives a finite, rejected guess
  f[0] = tau / an;
  f[1] = psi / a;
  f[2] = log(an);
  f[3] = a;
  f[4] = b;
}

// softplus(z) of the features: the fixed part of t.
__host__ __device__ inline double baseline(const double f[5]) {
  const double z = f[0] - f[1] - f[2];
  return z > 30.0 ? z : log1p(exp(z));
}

// Network output r (denormalised) of a sample whose converged slip rate has log10 value lg10v.
__host__ __device__ inline double target(const double f[5], double ln2v0, double lg10v) {
  return ln2v0 + f[0] - f[1] - kLn10 * lg10v - baseline(f);
}

// Natural log of the slip rate for network output r (denormalised).
__host__ __device__ inline double lnSlipRate(const double f[5], double ln2v0, double r) {
  return ln2v0 + f[0] - f[1] - baseline(f) - r;
}

}  // namespace sei_mlp
