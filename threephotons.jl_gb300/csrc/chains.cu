// Device-resident annealing chains (rotate_all_at_once / evaluate_step of
// src/determination.jl:281-338, 491-515) with the reference's move get_MC_step
// (src/determination.jl:232-241): for every even l in 2..L one rotation
// rtc[l] * random_rotation_step(2l+1, N(0, sigma_l)) * ctr[l] applied to all shells.
//
// random_rotation_step(b, beta) = C^T R(beta) C with C Haar-orthogonal and R a
// rotation by beta in the (1,2) plane (src/utilities.jl:165-190), i.e.
//     M = I + (cos beta - 1)(p p^T + q q^T) + sin beta (q p^T - p q^T)
// where p, q are the first two rows of C: a uniformly random orthonormal pair,
// drawn here by Gram-Schmidt of two Gaussian vectors.  M acts on the real-SH
// coefficients x = U c (U = Umat(l), src/spherical_harmonics.jl:445-457), so one
// shell costs O(2l+1) instead of a dense (2l+1)^2 product.
//
// Batching.  One launch scores B candidates per chain as speculative sequential
// steps: candidate i is the proposal of step (t + i) from the current state with
// the step sizes it would have after i rejections (sigma / f^i) and temperature
// T decay^(i+1).  The chain then takes the first accepted candidate (or none) and
// advances by that many steps, which is exactly the sequential chain's trajectory
// for the same random numbers (a rejected step leaves the state unchanged).
//
// Randomness is Philox4x32-10 keyed by the run seed with counter
// (step, chain, purpose, index), so a step's draws do not depend on the batching
// (the per-shell moves below key their step noise by the launch instead).
// All of it (proposal, scoring, Metropolis test, state update) runs on the device
// from one captured CUDA graph per launch.
//
// Per-shell moves (no reference counterpart; the learned-proposal experiment).
// TP3_MOVE_SHELL_SO3 rotates every shell k by its own exp([v_k]x) with the isotropic
// axis-angle step v_k ~ N(0, sigma^2 I3) (sigma adapted like the reference's step
// sizes), applied with the Wigner-D rotation of rotateStructure
// (src/spherical_harmonics.jl:572-603) to every even l.  Each launch also estimates
// the energy gradient of every shell's rotation from its B candidates, which all
// start from the same state: e_k = (1/B) sum_i ((dE_i - mean dE) / T) w_ik with w_ik
// the candidate's whitened step noise (the Gaussian-smoothing estimator, E[dE w] =
// sigma g to first order); the last kMlpGHist launches' e_k are network features.
// TP3_MOVE_LEARNED draws a candidate from the mixture p * q_net + (1 - p) * q_iso,
// where q_net takes the network's outputs (u_k, s_k) at the current state and draws
// v_k = sigma (a m_k + exp(s_k - mean s) z_k) with a = +-1 equally likely and
// m_k = sqrt(gamma) u_k / sqrt(sum |u|^2 + eps^2): a two-sided step along the
// network's gradient estimate, whose density is symmetric in a.  The candidate is
// accepted with the Metropolis-Hastings rule u < exp(-dE/T) q(x | x') / q(x' | x): the
// reverse density evaluates the network at the proposed state x' for the step -v
// (the rotation densities include the preimages |v| + 2 pi n of the exponential map).
// The network's history inputs (the chain's recent dE/T and gradient estimates) and
// the candidate's temperature are fixed parameters of the step, so every step is an
// exact MH step for exp(-E/T).
// TP3_MOVE_DRIFT is the same mixture without a network: the drift direction u_k is the
// chain's newest gradient estimate e_k and the scales are isotropic (s_k = 0).  The
// drift is a fixed parameter of the step, so the proposal is symmetric and the plain
// Metropolis rule is exact.  It isolates what the trained network adds over its own
// strongest input.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "ctx_internal.h"
#include "mlp.h"
#include "shellrot.cuh"

namespace {

using tp3::kFeatScale;
using tp3::drift_factor;
using tp3::kMlpGHist;
using tp3::kMlpHist;
using tp3::kMlpOutPad;
using tp3::mlp_grad_feature;
using tp3::mlp_head;
using tp3::mlp_hist_feature;
using tp3::mlp_temp_feature;
using tp3::rot_logdens;

constexpr int kPurposeAngle = 0;
constexpr int kPurposePlane = 1;
constexpr int kPurposeAccept = 2;
constexpr int kPurposeComponent = 3;
constexpr int kPurposeNoise = 5;  // + 16 i for candidate i: per-shell steps, keyed by the launch
constexpr int kMaxShells = 64;
constexpr int kMaxL = 62;  // even l <= 62: 2l+1 <= 125 real coefficients per block

struct ChainState {
  double E;
  double T;
  long long step;
  long long accepted;
  int last;      // index of the candidate taken by the last launch, -1 if none
  int launches;  // launches run (keys the network steps' random stream)
};

struct LogRow {  // one evaluated step (the columns of det.out, src/determination.jl:512-514)
  double step, sign, E_new, E, dE, T, ap, sigma_L;
};

struct MoveMeta {  // one logged candidate of a per-shell move
  float dE, T;     // energy change from the launch's start state, candidate temperature
  float acc;       // Metropolis decision with the candidate's own uniform (1 / 0)
  float comp;      // 1 = drawn from the network, 0 = isotropic
  float lr;        // log q(x | x') - log q(x' | x) (0 without the network)
  float sig;       // the candidate's isotropic step size sigma_i
  float tgt;       // (dE - mean over the launch's candidates of dE) / T
};

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c[0];
    const uint64_t p1 = (uint64_t)M1 * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += W0;
    k1 += W1;
  }
}

__device__ inline double u01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }

// Four standard normals (two Box-Muller pairs) for (step, chain, purpose, index).
__device__ inline void normals4(uint64_t seed, long long step, int chain, int purpose, int index, double z[4]) {
  uint32_t c[4] = {(uint32_t)step, (uint32_t)chain, (uint32_t)purpose, (uint32_t)index};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  for (int h = 0; h < 2; ++h) {
    const double r = sqrt(-2.0 * log(u01(c[2 * h])));
    const double a = 6.283185307179586 * u01(c[2 * h + 1]);
    z[2 * h] = r * cos(a);
    z[2 * h + 1] = r * sin(a);
  }
}

__device__ inline int sidx(int l, int m, int LMAX) {  // 0-based seanindex
  const int bigL = LMAX - 1;
  if (m >= 0) return m * (bigL + 1) - (m * (m - 1)) / 2 + (l - m);
  return (bigL * (bigL + 3)) / 2 + 1 + ((bigL + m) * (bigL + m + 1)) / 2 + (l + m);
}

// grid: nch * B; block 32 * warps.  Candidate (chain, i): copy the state, then each
// warp rotates one even l (2..L) of every shell.
__global__ void __launch_bounds__(256) k_propose(const double2* __restrict__ state, double2* __restrict__ cand,
                                                 const ChainState* __restrict__ cs, const double* __restrict__ sigma,
                                                 int nl, int B, int K, int LMAX, int L, double f, uint64_t seed,
                                                 const tp3::RagInfo* __restrict__ rag) {
  if (rag) L = rag[blockIdx.x].L;  // a ragged chain rotates its own orders only
  __shared__ double sp[8][2 * kMaxL + 1], sq[8][2 * kMaxL + 1];
  const int cid = blockIdx.x / B, i = blockIdx.x % B;
  const int ncoef = LMAX * LMAX;
  const double2* src = state + (size_t)cid * K * ncoef;
  double2* dst = cand + (size_t)blockIdx.x * K * ncoef;
  for (int e = threadIdx.x; e < K * ncoef; e += blockDim.x) dst[e] = src[e];
  __syncthreads();
  const long long step = cs[cid].step + i;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int l = 2 * (warp + 1); l <= L; l += 2 * nw) {
    const int d = 2 * l + 1;
    double* p = sp[warp];
    double* q = sq[warp];
    // plane: 2d normals, four per Philox call
    for (int j = lane; 4 * j < 2 * d; j += 32) {
      double z[4];
      normals4(seed, step, cid, kPurposePlane, l * 64 + j, z);
      for (int t = 0; t < 4; ++t) {
        const int idx = 4 * j + t;
        if (idx < d) p[idx] = z[t];
        else if (idx < 2 * d) q[idx - d] = z[t];
      }
    }
    __syncwarp();
    // Gram-Schmidt (FP64, lane-parallel sums)
    double pp = 0.0;
    for (int t = lane; t < d; t += 32) pp += p[t] * p[t];
    for (int o = 16; o > 0; o >>= 1) pp += __shfl_xor_sync(0xffffffffu, pp, o);
    const double ip = 1.0 / sqrt(pp);
    for (int t = lane; t < d; t += 32) p[t] *= ip;
    __syncwarp();
    double pq = 0.0;
    for (int t = lane; t < d; t += 32) pq += p[t] * q[t];
    for (int o = 16; o > 0; o >>= 1) pq += __shfl_xor_sync(0xffffffffu, pq, o);
    for (int t = lane; t < d; t += 32) q[t] -= pq * p[t];
    __syncwarp();
    double qq = 0.0;
    for (int t = lane; t < d; t += 32) qq += q[t] * q[t];
    for (int o = 16; o > 0; o >>= 1) qq += __shfl_xor_sync(0xffffffffu, qq, o);
    const double iq = 1.0 / sqrt(qq);
    for (int t = lane; t < d; t += 32) q[t] *= iq;
    __syncwarp();
    double za[4];
    normals4(seed, step, cid, kPurposeAngle, l, za);
    // step size after i rejections, divided step by step exactly as the sequential chain does
    double sgl = sigma[(size_t)cid * nl + l / 2];
    for (int t = 0; t < i; ++t) sgl /= f;
    const double beta = za[0] * sgl;
    const double cb = cos(beta) - 1.0, sb = sin(beta);
    const double r2 = 0.7071067811865476;
    // one shell per lane
    for (int k = lane; k < K; k += 32) {
      const double2* c = src + (size_t)k * ncoef;
      double2* o = dst + (size_t)k * ncoef;
      // alpha = p . (U c), bet = q . (U c)
      double ar = 0, ai = 0, br = 0, bi = 0;
      for (int u = -l; u <= l; ++u) {
        double xr, xi;
        if (u == 0) {
          const double2 v = c[sidx(l, 0, LMAX)];
          xr = v.x; xi = v.y;
        } else if (u > 0) {
          const double2 a = c[sidx(l, u, LMAX)], b = c[sidx(l, -u, LMAX)];
          const double sg = (u & 1) ? -1.0 : 1.0;
          xr = (a.x + sg * b.x) * r2; xi = (a.y + sg * b.y) * r2;
        } else {
          const double2 a = c[sidx(l, u, LMAX)], b = c[sidx(l, -u, LMAX)];
          const double sg = (u & 1) ? -1.0 : 1.0;  // (-1)^u
          // (i (-1)^u a - i b) / sqrt2
          xr = (-sg * a.y + b.y) * r2; xi = (sg * a.x - b.x) * r2;
        }
        ar += p[u + l] * xr; ai += p[u + l] * xi;
        br += q[u + l] * xr; bi += q[u + l] * xi;
      }
      // y = x + cb (p alpha + q bet) + sb (q alpha - p bet); c' = U^H y
      auto ycomp = [&](int u, double& yr, double& yi) {
        double xr, xi;
        if (u == 0) {
          const double2 v = c[sidx(l, 0, LMAX)];
          xr = v.x; xi = v.y;
        } else if (u > 0) {
          const double2 a = c[sidx(l, u, LMAX)], b = c[sidx(l, -u, LMAX)];
          const double sg = (u & 1) ? -1.0 : 1.0;
          xr = (a.x + sg * b.x) * r2; xi = (a.y + sg * b.y) * r2;
        } else {
          const double2 a = c[sidx(l, u, LMAX)], b = c[sidx(l, -u, LMAX)];
          const double sg = (u & 1) ? -1.0 : 1.0;
          xr = (-sg * a.y + b.y) * r2; xi = (sg * a.x - b.x) * r2;
        }
        const double pu = p[u + l], qu = q[u + l];
        yr = xr + cb * (pu * ar + qu * br) + sb * (qu * ar - pu * br);
        yi = xi + cb * (pu * ai + qu * bi) + sb * (qu * ai - pu * bi);
      };
      for (int m = 0; m <= l; ++m) {
        if (m == 0) {
          double yr, yi;
          ycomp(0, yr, yi);
          o[sidx(l, 0, LMAX)] = make_double2(yr, yi);
        } else {
          double ypr, ypi, ymr, ymi;
          ycomp(m, ypr, ypi);
          ycomp(-m, ymr, ymi);
          // c_m = (y_m + i y_-m)/sqrt2 ; c_-m = (-1)^m (y_m - i y_-m)/sqrt2
          const double sg = (m & 1) ? -1.0 : 1.0;
          o[sidx(l, m, LMAX)] = make_double2((ypr - ymi) * r2, (ypi + ymr) * r2);
          o[sidx(l, -m, LMAX)] = make_double2(sg * (ypr + ymi) * r2, sg * (ypi - ymr) * r2);
        }
      }
    }
    __syncwarp();
  }
}

// grid: ceil(nch / 128); block 128.  Metropolis over the speculative candidates.
// lr (per candidate log q(x|x') - log q(x'|x)) switches to the Metropolis-Hastings
// rule; without it the rule is the reference's (dE < 0, or dE > 0 and u < exp(-dE/T)).
// hist (nullable): the chain's last kMlpHist values of dE/T, newest last.
// meta (nullable): per-candidate log row of the launch's ring slot.
// sig_lo: first step-size index updated on accept/reject (0 for per-shell moves).
__global__ void k_select(ChainState* __restrict__ cs, double* __restrict__ sigma, const double* __restrict__ Ecand,
                         int nch, int nl, int B, double f, double decay, uint64_t seed, LogRow* __restrict__ log,
                         int logcap, int Lmax_index, const double* __restrict__ lr, float* __restrict__ hist,
                         const int* __restrict__ comp, MoveMeta* __restrict__ meta,
                         long long* __restrict__ launch_ctr, int meta_cap, int sig_lo) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const long long launch = launch_ctr ? *launch_ctr : 0;
  if (c < nch) {
    ChainState st = cs[c];
    const double E0 = st.E, T0 = st.T;
    const long long s0 = st.step;
    double* sg = sigma + (size_t)c * nl;
    double sig_i = sg[0];  // sigma_0 / f^i of candidate i (per-shell moves)
    st.last = -1;
    double dEmean = 0.0;
    if (meta) {
      int nf = 0;
      for (int i = 0; i < B; ++i) {
        const double d = Ecand[(size_t)c * B + i] - E0;
        if (isfinite(d)) { dEmean += d; ++nf; }
      }
      dEmean = nf > 0 ? dEmean / nf : 0.0;
    }
    for (int i = 0; i < B; ++i) {
      if (i > 0) sig_i /= f;
      const long long s = s0 + i;  // this step's index (0-based)
      double T = T0;
      for (int t = 0; t <= i; ++t) T *= decay;
      const double En = Ecand[(size_t)c * B + i];
      const double dE = En - E0;
      const double ap = exp(-dE / T);
      uint32_t ctr[4] = {(uint32_t)s, (uint32_t)c, (uint32_t)kPurposeAccept, 0u};
      philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
      const double u = u01(ctr[0]);
      bool acc;
      if (lr) {
        const double a = -dE / T + lr[(size_t)c * B + i];
        acc = a > 0.0 || u < exp(a);
      } else {
        acc = dE < 0.0 || (dE > 0.0 && u < ap);
      }
      if (meta) {
        MoveMeta mm;
        mm.dE = (float)dE; mm.T = (float)T; mm.acc = acc ? 1.f : 0.f;
        mm.comp = comp ? (float)comp[(size_t)c * B + i] : 0.f;
        mm.lr = lr ? (float)lr[(size_t)c * B + i] : 0.f;
        mm.sig = (float)sig_i;
        mm.tgt = (float)((dE - dEmean) / T);
        meta[((size_t)(launch % meta_cap) * nch + c) * B + i] = mm;
      }
      if (st.last >= 0) continue;  // past the taken step: logged only
      double sign = 0.0;
      if (acc) {
        sign = dE < 0.0 ? 1.0 : -1.0;
        for (int l = sig_lo; l < nl; ++l) sg[l] *= f;
        st.E = En;
      } else {
        for (int l = sig_lo; l < nl; ++l) sg[l] /= f;
      }
      if (hist) {
        float* hc = hist + (size_t)c * kMlpHist;
        for (int t = 0; t + 1 < kMlpHist; ++t) hc[t] = hc[t + 1];
        hc[kMlpHist - 1] = (float)(dE / T);
      }
      st.T = T;
      st.step = s + 1;
      if (log && logcap > 0) {
        LogRow r;
        r.step = (double)(s + 1); r.sign = sign; r.E_new = En; r.E = st.E; r.dE = dE; r.T = T; r.ap = ap;
        r.sigma_L = sg[Lmax_index];
        log[(size_t)c * logcap + (size_t)(s % logcap)] = r;
      }
      if (acc) {
        st.accepted += 1;
        st.last = i;
        if (!meta) break;
      }
    }
    st.launches += 1;
    cs[c] = st;
  }
}

// Feature rows of the proposal network (layout in mlp.h).  grid: nch * nb * K blocks
// (row = (chain, candidate i < nb, shell)), block 128.  coef: per-row source set,
// src_per_chain ? state[chain] : cand[chain * B + i].  X (nullable): rows of stride
// xs; logf (nullable): the i = 0 rows also go to the launch's log slot.  rag
// (nullable, ragged chains): a chain's coefficient features stop at its own L (the
// columns of higher orders, which its model does not have, are zero).
__global__ void __launch_bounds__(128) k_features(const double2* __restrict__ coef, int src_per_chain, int nch, int nb,
                                                  int B, int K, int LMAX, int L, const ChainState* __restrict__ cs,
                                                  double decay, const float* __restrict__ hist,
                                                  const float* __restrict__ ghist,
                                                  __nv_bfloat16* __restrict__ X, int xs,
                                                  __nv_bfloat16* __restrict__ logf,
                                                  const long long* __restrict__ launch_ctr, int log_cap,
                                                  const tp3::RagInfo* __restrict__ rag) {
  __shared__ float red[4];
  __shared__ float sx[(kMaxL + 1) * (kMaxL + 1)];
  const int row = blockIdx.x;
  const int k = row % K, ci = row / K, i = ci % nb, c = ci / nb;
  const int ncoef = LMAX * LMAX;
  const double2* src = coef + ((size_t)(src_per_chain ? c : c * B + i) * K + k) * ncoef;
  const int nf = (L + 1) * (L + 1);
  const int Lc = rag ? rag[(size_t)c * B + i].L : L;  // the chain's own orders
  const double r2 = 0.7071067811865476;
  float ss = 0.f;
  for (int t = threadIdx.x; t < nf; t += blockDim.x) {
    int l = 0;
    while ((l + 1) * (l + 1) <= t) ++l;
    const int u = t - l * l - l;  // -l..l
    double x;
    if (l > Lc) {
      x = 0.0;
    } else if (u == 0) {
      x = src[tp3::sean0(l, 0, LMAX)].x;
    } else if (u > 0) {  // (c_u + (-1)^u c_-u) / sqrt2
      const double2 a = src[tp3::sean0(l, u, LMAX)], b = src[tp3::sean0(l, -u, LMAX)];
      x = (a.x + ((u & 1) ? -b.x : b.x)) * r2;
    } else {  // (i (-1)^u c_u - i c_-u) / sqrt2, real part
      const double2 a = src[tp3::sean0(l, u, LMAX)], b = src[tp3::sean0(l, -u, LMAX)];
      x = (((u & 1) ? a.y : -a.y) + b.y) * r2;
    }
    sx[t] = (float)x;
    ss += (float)(x * x);
  }
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  const float nrm = red[0] + red[1] + red[2] + red[3];
  const float scale = nrm > 0.f ? kFeatScale / sqrtf(nrm) : 0.f;
  double T = cs[c].T;
  for (int t = 0; t <= i; ++t) T *= decay;
  const float tf = mlp_temp_feature(T);
  const float* hc = hist + (size_t)c * kMlpHist;
  __nv_bfloat16* xr = X ? X + (size_t)row * xs : nullptr;
  __nv_bfloat16* lr = nullptr;
  if (logf && i == 0) lr = logf + (((size_t)(*launch_ctr % log_cap) * nch + c) * K + k) * xs;
  for (int t = threadIdx.x; t < xs; t += blockDim.x) {
    float v = 0.f;
    if (t < nf) v = sx[t] * scale;
    else if (t < nf + kMlpHist) v = mlp_hist_feature((double)hc[t - nf]);
    else if (t == nf + kMlpHist) v = tf;
    else if (t < nf + kMlpHist + 1 + 3 * kMlpGHist) {
      const int q = t - nf - kMlpHist - 1, lag = q / 3, d = q - 3 * lag;
      v = mlp_grad_feature(ghist[(((size_t)c * kMlpGHist + lag) * K + k) * 3 + d]);
    }
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    if (xr) xr[t] = b;
    if (lr) lr[t] = b;
  }
}

// The network proposes relative to the candidate's isotropic step size sigma_i: for
// head outputs (u_k, s^_k) of the K shells, the drift is m_k = sigma_i f u_k with
// f = drift_factor(sum_k |u_k|^2) and the log-scale s_k = log sigma_i + s^_k - mean_k s^_k,
// so the network sets the direction of the step and how its noise is shared between
// shells and axes while the chain's adapted sigma sets its size.
__device__ inline void shell_scale_mean(const double (*hs)[3], int K, double m[3]) {
  m[0] = m[1] = m[2] = 0.0;
  for (int k = 0; k < K; ++k)
    for (int d = 0; d < 3; ++d) m[d] += hs[k][d];
  for (int d = 0; d < 3; ++d) m[d] /= K;
}

__device__ inline double shell_drift_factor(const double (*hu)[3], int K) {
  double uu = 0.0;
  for (int k = 0; k < K; ++k)
    for (int d = 0; d < 3; ++d) uu += hu[k][d] * hu[k][d];
  return drift_factor(uu);
}

__device__ inline void shell_params(const double hu[3], const double hs[3], const double m[3], double sg, double df,
                                    double ls, double mu[3], double s[3]) {
  for (int d = 0; d < 3; ++d) {
    mu[d] = sg * df * hu[d];
    s[d] = ls + hs[d] - m[d];
  }
}

__device__ inline double logaddexp(double a, double b) {
  const double m = a > b ? a : b;
  if (m == -INFINITY) return m;
  return m + log(exp(a - m) + exp(b - m));
}

// Per-shell proposal.  grid: nch * B (candidate (chain, i)); block 128.
// O (nullable): raw network outputs at the current state, rows (chain, i, shell).
// Writes the candidate's coefficients, its steps v [cand][K][3], its whitened step
// noise w [cand][K][3] (float), the component drawn, and
// lq[cand] = (log q(x'|x) of the network's drift +m, of -m, of the isotropic step),
// each summed over shells.
__global__ void __launch_bounds__(128) k_propose_shell(const double2* __restrict__ state, double2* __restrict__ cand,
                                                       const ChainState* __restrict__ cs,
                                                       const double* __restrict__ sigma, int nl, int B, int K, int LMAX,
                                                       int L, double f, uint64_t seed, const float* __restrict__ O,
                                                       const float* __restrict__ G, double p_net,
                                                       double* __restrict__ vout,
                                                       float* __restrict__ wout, int* __restrict__ comp,
                                                       double* __restrict__ lq, const double* __restrict__ delta,
                                                       const int* __restrict__ doff, float* __restrict__ vlog,
                                                       const long long* __restrict__ launch_ctr, int log_cap, int nch,
                                                       const tp3::RagInfo* __restrict__ rag) {
  __shared__ double2 xs[4][2 * tp3::kMaxRotL + 1], ys[4][2 * tp3::kMaxRotL + 1];
  if (rag) L = rag[blockIdx.x].L;
  __shared__ double eul[kMaxShells][3];
  __shared__ double red[3][128];
  __shared__ double hu[kMaxShells][3], hs[kMaxShells][3];
  const int cid = blockIdx.x / B, i = blockIdx.x % B;
  const int ncoef = LMAX * LMAX;
  const double2* src = state + (size_t)cid * K * ncoef;
  double2* dst = cand + (size_t)blockIdx.x * K * ncoef;
  const long long step = cs[cid].step + i;
  double sg = sigma[(size_t)cid * nl];
  for (int t = 0; t < i; ++t) sg /= f;
  uint32_t pc[4] = {(uint32_t)step, (uint32_t)cid, (uint32_t)kPurposeComponent, 0u};
  philox4x32_10(pc, (uint32_t)seed, (uint32_t)(seed >> 32));
  const bool drift = O != nullptr || G != nullptr;  // network or gradient-history drift
  const bool use_net = drift && u01(pc[0]) < p_net;
  // Per-shell steps draw their noise (and a network step its side) from a stream keyed
  // by the launch, not the step: the speculative candidates of one launch are
  // re-proposed at the same step numbers by the next, and the gradient-history inputs
  // are built from the previous launches' noise, so step-keyed draws would repeat noise
  // that the history (and the drift built on it) already depends on.  Each taken step
  // still sees a fresh draw, so the chain is a sequential chain with its own stream.
  const int launch = cs[cid].launches;
  const int pnet_i = kPurposeNoise + 16 * i;
  uint32_t pa[4] = {(uint32_t)launch, (uint32_t)cid, (uint32_t)pnet_i, (uint32_t)kMaxShells};
  philox4x32_10(pa, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double a = u01(pa[0]) < 0.5 ? -1.0 : 1.0;  // side of the network's two-sided drift
  const double ls = log(sg);
  double smean[3] = {0, 0, 0}, df = 0.0;
  if (drift) {
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      if (O) {
        mlp_head(O + ((size_t)blockIdx.x * K + k) * kMlpOutPad, hu[k], hs[k]);
      } else {
        // newest gradient estimate of shell k (history slot 0), isotropic scales
        const float* g = G + ((size_t)cid * kMlpGHist * K + k) * 3;
        for (int d = 0; d < 3; ++d) {
          hu[k][d] = isfinite(g[d]) ? (double)g[d] : 0.0;
          hs[k][d] = 0.0;
        }
      }
    }
    __syncthreads();
    shell_scale_mean(hs, K, smean);
    df = shell_drift_factor(hu, K);
  }
  double lp = 0.0, lm = 0.0, liso = 0.0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double z[4];
    normals4(seed, launch, cid, pnet_i, k, z);
    double mu[3] = {0, 0, 0}, s[3] = {ls, ls, ls}, v[3], w[3];
    if (drift) shell_params(hu[k], hs[k], smean, sg, df, ls, mu, s);
    for (int d = 0; d < 3; ++d) {
      v[d] = use_net ? a * mu[d] + exp(s[d]) * z[d] : sg * z[d];
      w[d] = use_net ? z[d] * exp(ls - s[d]) : z[d];
    }
    const double si[3] = {ls, ls, ls}, zero[3] = {0, 0, 0};
    liso += rot_logdens(v, zero, si);
    if (drift) {
      const double mneg[3] = {-mu[0], -mu[1], -mu[2]};
      lp += rot_logdens(v, mu, s);
      lm += rot_logdens(v, mneg, s);
    }
    double* vo = vout + ((size_t)blockIdx.x * K + k) * 3;
    float* wo = wout + ((size_t)blockIdx.x * K + k) * 3;
    for (int d = 0; d < 3; ++d) { vo[d] = v[d]; wo[d] = (float)w[d]; }
    if (vlog) {
      float* vl = vlog + (((size_t)(*launch_ctr % log_cap) * nch * B + blockIdx.x) * K + k) * 3;
      vl[0] = (float)v[0]; vl[1] = (float)v[1]; vl[2] = (float)v[2];
    }
    tp3::axis_angle_euler(v[0], v[1], v[2], eul[k][0], eul[k][1], eul[k][2]);
  }
  red[0][threadIdx.x] = lp;
  red[1][threadIdx.x] = lm;
  red[2][threadIdx.x] = liso;
  for (int e = threadIdx.x; e < K * ncoef; e += blockDim.x) dst[e] = src[e];
  __syncthreads();
  for (int h = 64; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; ++q) lq[(size_t)blockIdx.x * 3 + q] = red[q][0];
    comp[blockIdx.x] = use_net ? 1 : 0;
  }
  // rotate every even l >= 2 of every shell (l = 0 is invariant)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nord = L / 2;
  for (int item = warp; item < K * nord; item += nw) {
    const int k = item / nord, l = L - 2 * (item % nord);
    tp3::rotate_order_warp(src + (size_t)k * ncoef, dst + (size_t)k * ncoef, l, LMAX, eul[k][0], eul[k][1],
                           eul[k][2], delta + doff[l], xs[warp], ys[warp], lane);
  }
}

// grid: nch * B; block 64.  O2: raw network outputs at the proposed states.
// lr[cand] = log q(x | x') - log q(x' | x) for the mixture p q_net + (1 - p) q_iso,
// q_net = (q(. ; +m) + q(. ; -m)) / 2.
__global__ void k_mh_ratio(const float* __restrict__ O2, const double* __restrict__ v, const double* __restrict__ lq,
                           int K, double p_net, const ChainState* __restrict__ cs, const double* __restrict__ sigma,
                           int nl, int B, double f, double* __restrict__ lr) {
  __shared__ double red[2][64];
  __shared__ double hu[kMaxShells][3], hs[kMaxShells][3];
  const int cid = blockIdx.x / B, i = blockIdx.x % B;
  double sg = sigma[(size_t)cid * nl];
  for (int t = 0; t < i; ++t) sg /= f;
  const double ls = log(sg);
  for (int k = threadIdx.x; k < K; k += blockDim.x)
    mlp_head(O2 + ((size_t)blockIdx.x * K + k) * kMlpOutPad, hu[k], hs[k]);
  __syncthreads();
  double smean[3];
  shell_scale_mean(hs, K, smean);
  const double df = shell_drift_factor(hu, K);
  double rp = 0.0, rm = 0.0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double mu[3], s[3];
    shell_params(hu[k], hs[k], smean, sg, df, ls, mu, s);
    const double* vk = v + ((size_t)blockIdx.x * K + k) * 3;
    const double rv[3] = {-vk[0], -vk[1], -vk[2]};
    const double mneg[3] = {-mu[0], -mu[1], -mu[2]};
    rp += rot_logdens(rv, mu, s);
    rm += rot_logdens(rv, mneg, s);
  }
  red[0][threadIdx.x] = rp;
  red[1][threadIdx.x] = rm;
  __syncthreads();
  for (int h = 32; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      red[0][threadIdx.x] += red[0][threadIdx.x + h];
      red[1][threadIdx.x] += red[1][threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double* q = lq + (size_t)blockIdx.x * 3;
    const double ln2 = 0.6931471805599453;
    const double fnet = logaddexp(q[0], q[1]) - ln2, fiso = q[2];
    const double rnet = logaddexp(red[0][0], red[1][0]) - ln2;
    const double lp = log(p_net), lq1 = p_net < 1.0 ? log1p(-p_net) : -INFINITY;
    // the isotropic density is symmetric: q_iso(x | x') = q_iso(x' | x)
    lr[blockIdx.x] = logaddexp(lp + rnet, lq1 + fiso) - logaddexp(lp + fnet, lq1 + fiso);
  }
}

// Gradient estimate of the launch from its B candidates (all drawn at the chain's
// start state): e_k = (1/n) sum_i ((dE_i - mean dE) / T1) w_ik over the n candidates
// with a finite energy, T1 = the first candidate's temperature; shifted into the
// chain's history ghist [nch][kMlpGHist][K][3] (newest first).  Runs before k_select
// (reads the start energy and temperature).  grid: nch; block 128.
__global__ void k_grad_hist(const ChainState* __restrict__ cs, const double* __restrict__ Ecand,
                            const float* __restrict__ w, int B, int K, double decay, float* __restrict__ ghist) {
  const int c = blockIdx.x;
  const double E0 = cs[c].E, T1 = cs[c].T * decay;
  double mean = 0.0;
  int nf = 0;
  for (int i = 0; i < B; ++i) {
    const double d = Ecand[(size_t)c * B + i] - E0;
    if (isfinite(d)) { mean += d; ++nf; }
  }
  mean = nf > 0 ? mean / nf : 0.0;
  float* g = ghist + (size_t)c * kMlpGHist * K * 3;
  for (int q = threadIdx.x; q < K * 3; q += blockDim.x) {
    double e = 0.0;
    for (int i = 0; i < B; ++i) {
      const double d = Ecand[(size_t)c * B + i] - E0;
      if (isfinite(d)) e += (d - mean) * (double)w[((size_t)c * B + i) * K * 3 + q];
    }
    e = nf > 0 ? e / (nf * T1) : 0.0;
    for (int t = kMlpGHist - 1; t > 0; --t) g[(size_t)t * K * 3 + q] = g[(size_t)(t - 1) * K * 3 + q];
    g[q] = (float)e;
  }
}

// grid: nch; block 32.  sigma[c][0] = s0 (per-shell step size).
__global__ void k_set_sigma0(double* sigma, int nl, int nch, double s0) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nch) sigma[(size_t)c * nl] = s0;
}

// Training rows from the move log.  grid: n * K blocks (row = (pick, shell)), block 128.
__global__ void k_log_gather(const long long* __restrict__ idx, int K, int nch, int B, int xs, int tcol,
                             const __nv_bfloat16* __restrict__ logf, const float* __restrict__ vlog,
                             const MoveMeta* __restrict__ meta, __nv_bfloat16* __restrict__ X, float* __restrict__ V,
                             float* __restrict__ M) {
  const int row = blockIdx.x;
  const int k = row % K, j = row / K;
  const long long pos = idx[j];                 // candidate position in the ring
  const long long sc = pos / B;                 // (slot, chain)
  const __nv_bfloat16* f = logf + ((size_t)sc * K + k) * xs;
  const MoveMeta mm = meta[pos];
  const __nv_bfloat16 tb = __float2bfloat16_rn(mlp_temp_feature((double)mm.T));
  for (int t = threadIdx.x; t < xs; t += blockDim.x) X[(size_t)row * xs + t] = t == tcol ? tb : f[t];
  if (threadIdx.x < 3) V[(size_t)row * 3 + threadIdx.x] = vlog[((size_t)pos * K + k) * 3 + threadIdx.x] / mm.sig;
  if (k == 0 && threadIdx.x == 0) {
    float* mr = M + (size_t)j * 7;
    mr[0] = mm.dE; mr[1] = mm.T; mr[2] = mm.acc; mr[3] = mm.comp; mr[4] = mm.lr; mr[5] = mm.sig; mr[6] = mm.tgt;
  }
}

// grid: nch; block 256.  Adopt the accepted candidate; advance the launch counter
// of the move log (read by this launch's earlier kernels).
__global__ void k_commit(double2* __restrict__ state, const double2* __restrict__ cand,
                         const ChainState* __restrict__ cs, int B, int n, long long* __restrict__ launch_ctr) {
  const int c = blockIdx.x;
  if (launch_ctr && c == 0 && threadIdx.x == 0) *launch_ctr += 1;
  const int sel = cs[c].last;
  if (sel < 0) return;
  const double2* src = cand + ((size_t)c * B + sel) * n;
  double2* dst = state + (size_t)c * n;
  for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = src[e];
}

}  // namespace

struct tp3_chains {
  tp3_ctx* ctx = nullptr;
  int nch = 0, B = 0, K = 0, LMAX = 0, L = 0, nl = 0, ncoef = 0, logcap = 0;
  double f = 1.02, decay = 0.99;
  uint64_t seed = 0;
  double2* d_state = nullptr;
  double2* d_cand = nullptr;
  double* d_Ecand = nullptr;
  ChainState* d_cs = nullptr;
  double* d_sigma = nullptr;
  LogRow* d_log = nullptr;
  float* d_hist = nullptr;      // [nch][kMlpHist] dE/T history, newest last
  float* d_ghist = nullptr;     // [nch][kMlpGHist][K][3] per-shell gradient estimates, newest first
  tp3::RagInfo* d_rag = nullptr;  // [nch*B] per-candidate limits of ragged chains (null: the context's shape)
  int* d_lkh = nullptr;           // [nch*B][3] (L, K, histogram) per candidate
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_gen = -1;   // context scratch generation the graph was captured against
  int graph_mode = -1;  // evaluation mode baked into the graph
  bool dirty = false;   // move settings changed since the capture
  // per-shell moves
  int kind = TP3_MOVE_REFERENCE;
  double p_net = 0.0;
  tp3_mlp* net = nullptr;
  double* d_v = nullptr;        // [nch*B][K][3] axis-angle steps
  double* d_lq = nullptr;       // [nch*B][3] forward log densities (network +m, -m, isotropic)
  float* d_w = nullptr;         // [nch*B][K][3] whitened step noise
  double* d_lr = nullptr;       // [nch*B] log q(x|x') - log q(x'|x)
  int* d_comp = nullptr;        // [nch*B] component drawn
  // move log (training data): ring of mlog_cap launches
  int mlog_cap = 0;
  int xs = 0;                   // feature row stride (bf16)
  long long* d_launch = nullptr;
  __nv_bfloat16* d_lfeat = nullptr;  // [cap][nch][K][xs]
  float* d_lv = nullptr;             // [cap][nch][B][K][3]
  MoveMeta* d_lmeta = nullptr;       // [cap][nch][B]
};

namespace {

void chains_free(tp3_chains* h) {
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  cudaFree(h->d_state); cudaFree(h->d_cand); cudaFree(h->d_Ecand); cudaFree(h->d_cs); cudaFree(h->d_sigma);
  cudaFree(h->d_log); cudaFree(h->d_hist); cudaFree(h->d_ghist); cudaFree(h->d_w); cudaFree(h->d_v); cudaFree(h->d_lq); cudaFree(h->d_lr); cudaFree(h->d_comp);
  cudaFree(h->d_launch); cudaFree(h->d_lfeat); cudaFree(h->d_lv); cudaFree(h->d_lmeta);
  cudaFree(h->d_rag); cudaFree(h->d_lkh);
}

// one launch: propose B candidates per chain, score them, accept/reject, commit
int chains_enqueue(tp3_chains* h) {
  tp3_ctx* c = h->ctx;
  const int n = h->nch * h->B;
  cudaError_t e;
  const bool shell = h->kind != TP3_MOVE_REFERENCE;
  const bool net = h->kind == TP3_MOVE_LEARNED;
  const bool mlog = shell && h->mlog_cap > 0;
  long long* lctr = h->d_launch;
  if (!shell) {
    k_propose<<<n, 256, 0, c->stream>>>(h->d_state, h->d_cand, h->d_cs, h->d_sigma, h->nl, h->B, h->K, h->LMAX, h->L,
                                        h->f, h->seed, h->d_rag);
  } else {
    const float* O = nullptr;
    __nv_bfloat16* X = net ? tp3::mlp_input(h->net) : nullptr;
    if (net || mlog)
      k_features<<<h->nch * (net ? h->B : 1) * h->K, 128, 0, c->stream>>>(
          h->d_state, 1, h->nch, net ? h->B : 1, h->B, h->K, h->LMAX, h->L, h->d_cs, h->decay, h->d_hist, h->d_ghist,
          X, h->xs, mlog ? h->d_lfeat : nullptr, lctr, h->mlog_cap, h->d_rag);
    if (net) {
      if ((e = cudaGetLastError()) != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "features");
      if (int r = tp3::mlp_forward_raw(h->net, n * h->K, &O)) return r;
    }
    k_propose_shell<<<n, 128, 0, c->stream>>>(h->d_state, h->d_cand, h->d_cs, h->d_sigma, h->nl, h->B, h->K, h->LMAX,
                                              h->L, h->f, h->seed, O,
                                              h->kind == TP3_MOVE_DRIFT ? h->d_ghist : nullptr, h->p_net, h->d_v,
                                              h->d_w, h->d_comp, h->d_lq,
                                              c->d_delta,
                                              c->d_doff, mlog ? h->d_lv : nullptr, lctr, h->mlog_cap, h->nch,
                                              h->d_rag);
    if (net) {
      k_features<<<n * h->K, 128, 0, c->stream>>>(h->d_cand, 0, h->nch, h->B, h->B, h->K, h->LMAX, h->L, h->d_cs,
                                                   h->decay, h->d_hist, h->d_ghist, X, h->xs, nullptr, lctr,
                                                   h->mlog_cap, h->d_rag);
      if ((e = cudaGetLastError()) != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "features");
      if (int r = tp3::mlp_forward_raw(h->net, n * h->K, &O)) return r;
      k_mh_ratio<<<n, 64, 0, c->stream>>>(O, h->d_v, h->d_lq, h->K, h->p_net, h->d_cs, h->d_sigma, h->nl, h->B, h->f,
                                          h->d_lr);
    }
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "propose");
  if (int r = tp3::ctx_run_energy(c, n, h->d_cand, h->d_Ecand, h->d_rag)) return r;
  if (shell) k_grad_hist<<<h->nch, 128, 0, c->stream>>>(h->d_cs, h->d_Ecand, h->d_w, h->B, h->K, h->decay, h->d_ghist);
  k_select<<<(h->nch + 127) / 128, 128, 0, c->stream>>>(
      h->d_cs, h->d_sigma, h->d_Ecand, h->nch, h->nl, h->B, h->f, h->decay, h->seed, h->d_log, h->logcap,
      shell ? 0 : h->nl - 1, net ? h->d_lr : nullptr, h->d_hist, shell ? h->d_comp : nullptr,
      mlog ? h->d_lmeta : nullptr, lctr, h->mlog_cap, shell ? 0 : 1);
  k_commit<<<h->nch, 256, 0, c->stream>>>(h->d_state, h->d_cand, h->d_cs, h->B, h->K * h->ncoef, mlog ? lctr : nullptr);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "select/commit");
  return TP3_OK;
}

// Capture one launch into a CUDA graph (profiling events are kept out of it).  The
// graph holds the context's scratch pointers and evaluation mode, so it is
// re-captured when either changes.
int capture(tp3_chains* h) {
  tp3_ctx* ctx = h->ctx;
  if (h->exec) { cudaGraphExecDestroy(h->exec); h->exec = nullptr; }
  if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
  const bool prof = ctx->prof;
  ctx->prof = false;
  cudaStream_t cap = ctx->stream;
  bool graph_ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  int r = graph_ok ? chains_enqueue(h) : TP3_OK;
  if (graph_ok) {
    cudaGraph_t g = nullptr;
    cudaError_t ec = cudaStreamEndCapture(cap, &g);
    if (r == TP3_OK && ec == cudaSuccess && g && cudaGraphInstantiate(&h->exec, g, 0) == cudaSuccess) {
      h->graph = g;
    } else {
      if (g) cudaGraphDestroy(g);
      h->exec = nullptr;
    }
  }
  ctx->prof = prof;
  cudaGetLastError();
  h->graph_gen = ctx->scratch_gen;
  h->graph_mode = ctx->mode;
  h->dirty = false;
  return r;
}

}  // namespace

extern "C" {

static int chains_create(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                         double initial_stepsize, double stepsizefactor, double temperature_decay, uint64_t seed,
                         int log_capacity, const int* lkh, tp3_chains** out);

int tp3_chains_create(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                      double initial_stepsize, double stepsizefactor, double temperature_decay, uint64_t seed,
                      int log_capacity, tp3_chains** out) {
  return chains_create(ctx, nchains, ncand, coeff0, T0, initial_stepsize, stepsizefactor, temperature_decay, seed,
                       log_capacity, nullptr, out);
}

int tp3_chains_create_ragged(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                             double initial_stepsize, double stepsizefactor, double temperature_decay, uint64_t seed,
                             int log_capacity, const int* chain_lkh, tp3_chains** out) {
  if (!chain_lkh) return tp3::ctx_fail(ctx, TP3_ERR_ARG, "chain_lkh is NULL");
  return chains_create(ctx, nchains, ncand, coeff0, T0, initial_stepsize, stepsizefactor, temperature_decay, seed,
                       log_capacity, chain_lkh, out);
}

static int chains_create(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                         double initial_stepsize, double stepsizefactor, double temperature_decay, uint64_t seed,
                         int log_capacity, const int* lkh, tp3_chains** out) {
  if (int r = tp3::ctx_check(ctx)) return r;
  if (!out || !coeff0 || !T0 || nchains < 1 || ncand < 1 || log_capacity < 0)
    return tp3::ctx_fail(ctx, TP3_ERR_ARG, "bad chain arguments");
  if (!(stepsizefactor > 0.0) || !(temperature_decay > 0.0))
    return tp3::ctx_fail(ctx, TP3_ERR_ARG, "step-size factor and temperature decay must be positive");
  if (ctx->b.L > kMaxL) return tp3::ctx_fail(ctx, TP3_ERR_UNSUPPORTED, "chains need L <= 62");
  if (!lkh && !ctx->has_hist) return tp3::ctx_fail(ctx, TP3_ERR_NO_HISTOGRAM, "tp3_set_histogram has not been called");
  if (lkh && ctx->nhist == 0) return tp3::ctx_fail(ctx, TP3_ERR_NO_HISTOGRAM, "tp3_set_histograms has not been called");
  *out = nullptr;
  tp3_chains* h = new tp3_chains();
  h->ctx = ctx;
  h->nch = nchains; h->B = ncand; h->K = ctx->b.K; h->LMAX = ctx->b.LMAX; h->L = ctx->b.L;
  h->nl = ctx->b.L / 2 + 1; h->ncoef = h->LMAX * h->LMAX; h->logcap = log_capacity;
  h->f = stepsizefactor; h->decay = temperature_decay; h->seed = seed;
  const size_t nst = (size_t)nchains * h->K * h->ncoef;
  cudaError_t e;
  if ((e = cudaMalloc(&h->d_state, nst * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_cand, nst * ncand * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_Ecand, (size_t)nchains * ncand * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_cs, (size_t)nchains * sizeof(ChainState))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_sigma, (size_t)nchains * h->nl * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_hist, (size_t)nchains * kMlpHist * sizeof(float))) != cudaSuccess ||
      (e = cudaMemset(h->d_hist, 0, (size_t)nchains * kMlpHist * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_ghist, (size_t)nchains * kMlpGHist * h->K * 3 * sizeof(float))) != cudaSuccess ||
      (e = cudaMemset(h->d_ghist, 0, (size_t)nchains * kMlpGHist * h->K * 3 * sizeof(float))) != cudaSuccess ||
      (log_capacity > 0 && (e = cudaMalloc(&h->d_log, (size_t)nchains * log_capacity * sizeof(LogRow))) != cudaSuccess)) {
    chains_free(h);
    delete h;
    cudaGetLastError();
    return tp3::ctx_fail(ctx, TP3_ERR_ALLOC, std::string("chain allocation: ") + cudaGetErrorString(e));
  }
  if (int r = tp3::ctx_ensure_cap(ctx, nchains * ncand)) { chains_free(h); delete h; return r; }
  // initial state and energies
  if ((e = cudaMemcpy(h->d_state, coeff0, nst * sizeof(double2), cudaMemcpyHostToDevice)) != cudaSuccess) {
    chains_free(h); delete h;
    return tp3::ctx_cuda_fail(ctx, e, "chain upload");
  }
  const tp3::RagInfo* rag0 = nullptr;
  if (lkh) {
    // per-candidate limits [nch * B], then the chains' own [nch] for the initial energies
    const size_t nc = (size_t)nchains * ncand;
    std::vector<int> hl(3 * (nc + nchains));
    for (size_t i = 0; i < nc + nchains; ++i) {
      const size_t c = i < nc ? i / ncand : i - nc;
      for (int j = 0; j < 3; ++j) hl[3 * i + j] = lkh[3 * c + j];
    }
    if ((e = cudaMalloc(&h->d_lkh, hl.size() * sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_rag, (nc + nchains) * sizeof(tp3::RagInfo))) != cudaSuccess ||
        (e = cudaMemcpy(h->d_lkh, hl.data(), hl.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) {
      chains_free(h); delete h;
      cudaGetLastError();
      return tp3::ctx_fail(ctx, TP3_ERR_ALLOC, std::string("ragged limits: ") + cudaGetErrorString(e));
    }
    if (int r = tp3::ctx_make_rag(ctx, (int)(nc + nchains), h->d_lkh, h->d_rag)) { chains_free(h); delete h; return r; }
    rag0 = h->d_rag + nc;
  }
  double* dE0 = h->d_Ecand;  // scratch for the initial energies
  if (int r = tp3::ctx_run_energy(ctx, nchains, h->d_state, dE0, rag0)) { chains_free(h); delete h; return r; }
  std::vector<double> E0(nchains);
  if ((e = cudaMemcpyAsync(E0.data(), dE0, nchains * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) {
    chains_free(h); delete h;
    return tp3::ctx_cuda_fail(ctx, e, "initial energies");
  }
  if (int r = tp3::ctx_check_device_error(ctx)) { chains_free(h); delete h; return r; }
  std::vector<ChainState> cs(nchains);
  std::vector<double> sig((size_t)nchains * h->nl);
  for (int i = 0; i < nchains; ++i) {
    cs[i].E = E0[i]; cs[i].T = T0[i]; cs[i].step = 0; cs[i].accepted = 0; cs[i].last = -1; cs[i].launches = 0;
    // stepsizes[l] = initial_stepsize * (l - 1), l = 2:2:L (src/determination.jl:295)
    for (int il = 0; il < h->nl; ++il) sig[(size_t)i * h->nl + il] = il == 0 ? 0.0 : initial_stepsize * (2 * il - 1);
  }
  if ((e = cudaMemcpy(h->d_cs, cs.data(), cs.size() * sizeof(ChainState), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(h->d_sigma, sig.data(), sig.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (log_capacity > 0 && (e = cudaMemset(h->d_log, 0, (size_t)nchains * log_capacity * sizeof(LogRow))) != cudaSuccess)) {
    chains_free(h); delete h;
    return tp3::ctx_cuda_fail(ctx, e, "chain state upload");
  }
  int r = capture(h);
  if (r != TP3_OK) { chains_free(h); delete h; return r; }
  *out = h;
  return TP3_OK;
}

void tp3_chains_destroy(tp3_chains* h) {
  if (!h) return;
  if (h->ctx) {
    cudaSetDevice(h->ctx->device);
    cudaStreamSynchronize(h->ctx->stream);
  }
  chains_free(h);
  delete h;
}

int tp3_chains_run(tp3_chains* h, int launches) {
  if (!h) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  if (launches < 0) return tp3::ctx_fail(c, TP3_ERR_ARG, "launches must be >= 0");
  if (int r = tp3::ctx_ensure_cap(c, h->nch * h->B)) return r;
  if (h->graph_gen != c->scratch_gen || h->graph_mode != c->mode || h->dirty) {
    if (int r = capture(h)) return r;
  }
  for (int i = 0; i < launches; ++i) {
    if (h->exec) {
      cudaError_t e = cudaGraphLaunch(h->exec, c->stream);
      if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "graph launch");
    } else if (int r = chains_enqueue(h)) {
      return r;
    }
  }
  return TP3_OK;
}

int tp3_chains_state(tp3_chains* h, double* E, double* T, double* sigma, int64_t* steps, int64_t* accepted) {
  if (!h) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "chain sync");
  if (int r = tp3::ctx_check_device_error(c)) return r;
  std::vector<ChainState> cs(h->nch);
  if ((e = cudaMemcpy(cs.data(), h->d_cs, cs.size() * sizeof(ChainState), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return tp3::ctx_cuda_fail(c, e, "chain state read");
  if (sigma && (e = cudaMemcpy(sigma, h->d_sigma, (size_t)h->nch * h->nl * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return tp3::ctx_cuda_fail(c, e, "chain sigma read");
  for (int i = 0; i < h->nch; ++i) {
    if (E) E[i] = cs[i].E;
    if (T) T[i] = cs[i].T;
    if (steps) steps[i] = cs[i].step;
    if (accepted) accepted[i] = cs[i].accepted;
  }
  return TP3_OK;
}

int tp3_chains_coeff(tp3_chains* h, double* coeff) {
  if (!h || !coeff) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(coeff, h->d_state, (size_t)h->nch * h->K * h->ncoef * sizeof(double2), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "chain coefficients read");
  return TP3_OK;
}

int tp3_chains_log(tp3_chains* h, int chain, double* rows, int64_t* nrows) {
  if (!h || !rows || !nrows || chain < 0 || chain >= h->nch) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  *nrows = 0;
  if (h->logcap == 0) return TP3_OK;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  std::vector<LogRow> buf(h->logcap);
  if (e == cudaSuccess)
    e = cudaMemcpy(buf.data(), h->d_log + (size_t)chain * h->logcap, h->logcap * sizeof(LogRow), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "chain log read");
  ChainState cs;
  if ((e = cudaMemcpy(&cs, h->d_cs + chain, sizeof(ChainState), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return tp3::ctx_cuda_fail(c, e, "chain state read");
  const long long n = cs.step < h->logcap ? cs.step : h->logcap;
  const long long first = cs.step - n;
  for (long long i = 0; i < n; ++i) {
    const LogRow& r = buf[(size_t)((first + i) % h->logcap)];
    std::memcpy(rows + 8 * i, &r, sizeof(LogRow));
  }
  *nrows = n;
  return TP3_OK;
}

int tp3_chains_snapshot(tp3_chains* h, void* buf, size_t capacity, size_t* bytes) {
  if (!h || !bytes) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  const size_t nst = (size_t)h->nch * h->K * h->ncoef * sizeof(double2);
  const size_t ncs = (size_t)h->nch * sizeof(ChainState);
  const size_t nsg = (size_t)h->nch * h->nl * sizeof(double);
  const size_t nhs = (size_t)h->nch * kMlpHist * sizeof(float);
  const size_t ngh = (size_t)h->nch * kMlpGHist * h->K * 3 * sizeof(float);
  const size_t hdr = 8 * sizeof(int64_t);
  const size_t need = hdr + nst + ncs + nsg + nhs + ngh;
  *bytes = need;
  if (!buf) return TP3_OK;
  if (capacity < need) return tp3::ctx_fail(c, TP3_ERR_ARG, "snapshot buffer too small");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "snapshot sync");
  int64_t head[8] = {0x54503343484e31LL, h->nch, h->K, h->LMAX, h->L, (int64_t)h->seed, 0, 0};
  std::memcpy(head + 6, &h->f, sizeof(double));
  std::memcpy(head + 7, &h->decay, sizeof(double));
  uint8_t* p = (uint8_t*)buf;
  std::memcpy(p, head, hdr);
  if ((e = cudaMemcpy(p + hdr, h->d_state, nst, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(p + hdr + nst, h->d_cs, ncs, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(p + hdr + nst + ncs, h->d_sigma, nsg, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(p + hdr + nst + ncs + nsg, h->d_hist, nhs, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(p + hdr + nst + ncs + nsg + nhs, h->d_ghist, ngh, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return tp3::ctx_cuda_fail(c, e, "snapshot copy");
  return TP3_OK;
}

int tp3_chains_restore(tp3_chains* h, const void* buf, size_t bytes) {
  if (!h || !buf) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  const size_t nst = (size_t)h->nch * h->K * h->ncoef * sizeof(double2);
  const size_t ncs = (size_t)h->nch * sizeof(ChainState);
  const size_t nsg = (size_t)h->nch * h->nl * sizeof(double);
  const size_t nhs = (size_t)h->nch * kMlpHist * sizeof(float);
  const size_t ngh = (size_t)h->nch * kMlpGHist * h->K * 3 * sizeof(float);
  const size_t hdr = 8 * sizeof(int64_t);
  if (bytes != hdr + nst + ncs + nsg + nhs + ngh) return tp3::ctx_fail(c, TP3_ERR_ARG, "snapshot size does not match these chains");
  int64_t head[8];
  std::memcpy(head, buf, hdr);
  double f, decay;
  std::memcpy(&f, head + 6, sizeof(double));
  std::memcpy(&decay, head + 7, sizeof(double));
  if (head[0] != 0x54503343484e31LL || head[1] != h->nch || head[2] != h->K || head[3] != h->LMAX || head[4] != h->L ||
      (uint64_t)head[5] != h->seed || f != h->f || decay != h->decay)
    return tp3::ctx_fail(c, TP3_ERR_ARG, "snapshot belongs to differently configured chains");
  const uint8_t* p = (const uint8_t*)buf;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_state, p + hdr, nst, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_cs, p + hdr + nst, ncs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_sigma, p + hdr + nst + ncs, nsg, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_hist, p + hdr + nst + ncs + nsg, nhs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_ghist, p + hdr + nst + ncs + nsg + nhs, ngh, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "restore copy");
  return TP3_OK;
}

int tp3_chains_set_move(tp3_chains* h, int kind, double sigma0, double p_net, tp3_mlp* net) {
  if (!h) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  if (kind != TP3_MOVE_REFERENCE && kind != TP3_MOVE_SHELL_SO3 && kind != TP3_MOVE_LEARNED &&
      kind != TP3_MOVE_DRIFT)
    return tp3::ctx_fail(c, TP3_ERR_ARG, "unknown move kind");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "set move sync");
  if (kind != TP3_MOVE_REFERENCE) {
    if (!(sigma0 > 0.0) || !std::isfinite(sigma0)) return tp3::ctx_fail(c, TP3_ERR_ARG, "sigma0 must be positive");
    if (h->K > kMaxShells) return tp3::ctx_fail(c, TP3_ERR_UNSUPPORTED, "per-shell moves need K <= 64");
    if (int r = tp3::ctx_ensure_rot_tables(c, h->L)) return r;
    const size_t nc = (size_t)h->nch * h->B;
    if (!h->d_v && ((e = cudaMalloc(&h->d_v, nc * h->K * 3 * sizeof(double))) != cudaSuccess ||
                    (e = cudaMalloc(&h->d_lq, nc * 3 * sizeof(double))) != cudaSuccess ||
                    (e = cudaMalloc(&h->d_w, nc * h->K * 3 * sizeof(float))) != cudaSuccess ||
                    (e = cudaMalloc(&h->d_lr, nc * sizeof(double))) != cudaSuccess ||
                    (e = cudaMalloc(&h->d_comp, nc * sizeof(int))) != cudaSuccess)) {
      cudaGetLastError();
      return tp3::ctx_fail(c, TP3_ERR_ALLOC, std::string("move buffers: ") + cudaGetErrorString(e));
    }
    k_set_sigma0<<<(h->nch + 31) / 32, 32, 0, c->stream>>>(h->d_sigma, h->nl, h->nch, sigma0);
    if ((e = cudaGetLastError()) != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "set sigma0");
  }
  if (kind == TP3_MOVE_LEARNED) {
    if (!net) return tp3::ctx_fail(c, TP3_ERR_ARG, "learned moves need a network");
    if (!(p_net > 0.0 && p_net <= 1.0)) return tp3::ctx_fail(c, TP3_ERR_ARG, "p_net must be in (0, 1]");
    if (tp3::mlp_n_in_of(net) != tp3::mlp_n_in(h->L))
      return tp3::ctx_fail(c, TP3_ERR_ARG, "network input width is not (L+1)^2 + 33");
    if (tp3::mlp_max_rows(net) < h->nch * h->B * h->K)
      return tp3::ctx_fail(c, TP3_ERR_ARG, "network max_rows < chains x candidates x shells");
  }
  if (kind == TP3_MOVE_DRIFT && !(p_net > 0.0 && p_net <= 1.0))
    return tp3::ctx_fail(c, TP3_ERR_ARG, "p_net must be in (0, 1]");
  h->kind = kind;
  h->p_net = (kind == TP3_MOVE_LEARNED || kind == TP3_MOVE_DRIFT) ? p_net : 0.0;
  h->net = kind == TP3_MOVE_LEARNED ? net : nullptr;
  h->xs = tp3::mlp_n_in_pad(h->L);
  h->dirty = true;
  return TP3_OK;
}

int tp3_chains_enable_move_log(tp3_chains* h, int launches) {
  if (!h) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  if (launches < 1) return tp3::ctx_fail(c, TP3_ERR_ARG, "launch capacity must be >= 1");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "move log sync");
  cudaFree(h->d_lfeat); cudaFree(h->d_lv); cudaFree(h->d_lmeta);
  h->d_lfeat = nullptr; h->d_lv = nullptr; h->d_lmeta = nullptr;
  h->xs = tp3::mlp_n_in_pad(h->L);
  const size_t slots = (size_t)launches * h->nch;
  if ((!h->d_launch && (e = cudaMalloc(&h->d_launch, sizeof(long long))) != cudaSuccess) ||
      (e = cudaMalloc(&h->d_lfeat, slots * h->K * h->xs * sizeof(__nv_bfloat16))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_lv, slots * h->B * h->K * 3 * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_lmeta, slots * h->B * sizeof(MoveMeta))) != cudaSuccess) {
    cudaGetLastError();
    h->mlog_cap = 0;
    h->dirty = true;
    return tp3::ctx_fail(c, TP3_ERR_ALLOC, std::string("move log: ") + cudaGetErrorString(e));
  }
  if ((e = cudaMemset(h->d_launch, 0, sizeof(long long))) != cudaSuccess)
    return tp3::ctx_cuda_fail(c, e, "move log reset");
  h->mlog_cap = launches;
  h->dirty = true;
  return TP3_OK;
}

int tp3_chains_move_log_count(tp3_chains* h, int64_t* candidates) {
  if (!h || !candidates) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  *candidates = 0;
  if (h->mlog_cap == 0) return TP3_OK;
  long long n = 0;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(&n, h->d_launch, sizeof(long long), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "move log count");
  *candidates = (int64_t)(n < h->mlog_cap ? n : h->mlog_cap) * h->nch * h->B;
  return TP3_OK;
}

int tp3_chains_move_log_gather(tp3_chains* h, int n, const int64_t* d_idx, void* d_x, float* d_v, float* d_meta) {
  if (!h) return TP3_ERR_ARG;
  tp3_ctx* c = h->ctx;
  if (int r = tp3::ctx_check(c)) return r;
  if (h->mlog_cap == 0) return tp3::ctx_fail(c, TP3_ERR_ARG, "move log not enabled");
  if (n < 1 || !d_idx || !d_x || !d_v || !d_meta) return tp3::ctx_fail(c, TP3_ERR_ARG, "bad gather arguments");
  const int tcol = (h->L + 1) * (h->L + 1) + kMlpHist;
  k_log_gather<<<n * h->K, 128, 0, c->stream>>>((const long long*)d_idx, h->K, h->nch, h->B, h->xs, tcol, h->d_lfeat,
                                                 h->d_lv, h->d_lmeta, (__nv_bfloat16*)d_x, d_v, d_meta);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "move log gather");
  return TP3_OK;
}

int tp3_chains_graph(const tp3_chains* h, int* captured) {
  if (!h || !captured) return TP3_ERR_ARG;
  *captured = h->exec != nullptr;
  return TP3_OK;
}

}  // extern "C"
