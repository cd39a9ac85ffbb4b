// Learned proposal network: constants and device helpers shared by the network
// (mlp.cu) and the chain moves that sample from it (chains.cu).
//
// Per shell the network maps a feature row to a drift direction u (3) and a
// log-scale s (3) of the shell's axis-angle step, from the raw outputs o of the
// last layer:
//     u_d = o_d,  s_d = kSMid + kSHalf * tanh(o_{3+d}),  d = 0..2
// so exp(s) lies in (9e-4, 2.7).  u estimates sigma g_k / T (g_k: the energy
// gradient of a rotation of shell k, sigma: the isotropic step size, T: the
// temperature); the proposal steps along +-u (both signs equally likely).
//
// Feature row of shell k of a state (kMlpInPad bf16 columns):
//   [0, (L+1)^2)            real SH coefficients x_lm (l = 0..L, u = -l..l; x = U c,
//                           Umat of src/spherical_harmonics.jl:445-457) divided by
//                           the shell's norm and multiplied by kFeatScale
//   [(L+1)^2, +8)           the chain's last 8 values of dE / T, clipped to +-10, / 10
//   [(L+1)^2 + 8]           log10(T) / 4 of the candidate's temperature
//   [(L+1)^2 + 9, +24)      the shell's gradient estimates of the chain's last 8
//                           launches (3 each, newest first), clipped to +-8, / 2
//   rest                    zero
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace tp3 {

constexpr int kMlpHist = 8;         // history values per chain
constexpr int kMlpGHist = 8;        // launches of per-shell gradient estimates in a feature row
constexpr int kMlpOut = 6;          // u (3), s (3)
constexpr int kMlpOutPad = 16;      // last layer padded to the smallest MMA N
constexpr double kSMid = -3.0;
constexpr double kSHalf = 4.0;
constexpr float kFeatScale = 8.0f;
// drift of a network step: a sqrt(kDriftGamma) u / sqrt(|u|^2 + kDriftEps^2) in units of
// sigma, a = +-1, |u|^2 summed over the candidate's shells
constexpr double kDriftGamma = 16.0;
constexpr double kDriftEps = 0.1;

__host__ __device__ inline int mlp_n_in(int L) { return (L + 1) * (L + 1) + kMlpHist + 1 + 3 * kMlpGHist; }
__host__ __device__ inline int mlp_n_in_pad(int L) { return (mlp_n_in(L) + 31) / 32 * 32; }

__host__ __device__ inline float mlp_hist_feature(double dE_over_T) {
  double x = dE_over_T;
  if (!(x == x)) x = 10.0;  // NaN: treat as a large uphill step
  x = x > 10.0 ? 10.0 : (x < -10.0 ? -10.0 : x);
  return (float)(x / 10.0);
}

__host__ __device__ inline float mlp_temp_feature(double T) { return (float)(log10(T > 1e-300 ? T : 1e-300) / 4.0); }

__host__ __device__ inline float mlp_grad_feature(float e) {
  float x = e;
  if (!(x == x)) x = 0.f;
  x = x > 8.f ? 8.f : (x < -8.f ? -8.f : x);
  return 0.5f * x;
}

// log of the density of the rotation exp([v]x) under the axis-angle Gaussian
// N(mu, diag(exp(2 s))), up to the Haar factor 1 / (2 (1 - cos|v|)) that is common to
// a move and its reverse: the sum over the preimages v^(|v| + 2 pi n), n = -1, 0, 1, of
// the Gaussian density times ((|v| + 2 pi n) / |v|)^2.
__host__ __device__ inline double rot_logdens(const double v[3], const double mu[3], const double s[3]) {
  const double th = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const double two_pi = 6.283185307179586;
  double lt[3];
  int nt = 0;
  const int nlo = th > 0.0 ? -1 : 0, nhi = th > 0.0 ? 1 : 0;
  for (int n = nlo; n <= nhi; ++n) {
    const double a = th + two_pi * n;
    const double f = th > 0.0 ? a / th : 1.0;
    double q = 0.0, ls = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double z = (v[d] * f - mu[d]) * exp(-s[d]);
      q += z * z;
      ls += s[d];
    }
    lt[nt++] = -0.5 * q - ls - 2.7568155996140185 + 2.0 * log(fabs(f) > 0.0 ? fabs(f) : 1e-300);  // 1.5 log(2 pi)
  }
  double mx = lt[0];
  for (int i = 1; i < nt; ++i) mx = lt[i] > mx ? lt[i] : mx;
  double acc = 0.0;
  for (int i = 0; i < nt; ++i) acc += exp(lt[i] - mx);
  return mx + log(acc);
}

__host__ __device__ inline void mlp_head(const float* o, double u[3], double s[3]) {
  for (int d = 0; d < 3; ++d) {
    u[d] = (double)o[d];
    s[d] = kSMid + kSHalf * tanh((double)o[3 + d]);
  }
}

// drift factor sqrt(gamma) / sqrt(|u|^2 + eps^2) of a candidate whose shells' u have
// squared norm uu
__host__ __device__ inline double drift_factor(double uu) {
  return sqrt(kDriftGamma) / sqrt(uu + kDriftEps * kDriftEps);
}

}  // namespace tp3
