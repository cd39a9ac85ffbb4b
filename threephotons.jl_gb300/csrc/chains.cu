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
// (step, chain, purpose, index), so a step's draws do not depend on the batching.
// All of it (proposal, scoring, Metropolis test, state update) runs on the device
// from one captured CUDA graph per launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "ctx_internal.h"

namespace {

constexpr int kPurposeAngle = 0;
constexpr int kPurposePlane = 1;
constexpr int kPurposeAccept = 2;
constexpr int kMaxL = 62;  // even l <= 62: 2l+1 <= 125 real coefficients per block

struct ChainState {
  double E;
  double T;
  long long step;
  long long accepted;
  int last;  // index of the candidate taken by the last launch, -1 if none
  int pad;
};

struct LogRow {  // one evaluated step (the columns of det.out, src/determination.jl:512-514)
  double step, sign, E_new, E, dE, T, ap, sigma_L;
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
                                                 int nl, int B, int K, int LMAX, int L, double f, uint64_t seed) {
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
__global__ void k_select(ChainState* __restrict__ cs, double* __restrict__ sigma, const double* __restrict__ Ecand,
                         int nch, int nl, int B, double f, double decay, uint64_t seed, LogRow* __restrict__ log,
                         int logcap, int Lmax_index) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nch) return;
  ChainState st = cs[c];
  double* sg = sigma + (size_t)c * nl;
  st.last = -1;
  for (int i = 0; i < B; ++i) {
    const long long s = st.step;  // this step's index (0-based)
    const double T = st.T * decay;
    const double En = Ecand[(size_t)c * B + i];
    const double dE = En - st.E;
    const double ap = exp(-dE / T);
    uint32_t ctr[4] = {(uint32_t)s, (uint32_t)c, (uint32_t)kPurposeAccept, 0u};
    philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u = u01(ctr[0]);
    const bool acc = dE < 0.0 || (dE > 0.0 && u < ap);
    double sign = 0.0;
    if (acc) {
      sign = dE < 0.0 ? 1.0 : -1.0;
      for (int l = 1; l < nl; ++l) sg[l] *= f;
      st.E = En;
    } else {
      for (int l = 1; l < nl; ++l) sg[l] /= f;
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
      break;
    }
  }
  cs[c] = st;
}

// grid: nch; block 256.  Adopt the accepted candidate.
__global__ void k_commit(double2* __restrict__ state, const double2* __restrict__ cand,
                         const ChainState* __restrict__ cs, int B, int n) {
  const int c = blockIdx.x;
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
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_gen = -1;   // context scratch generation the graph was captured against
  int graph_mode = -1;  // evaluation mode baked into the graph
};

namespace {

void chains_free(tp3_chains* h) {
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  cudaFree(h->d_state); cudaFree(h->d_cand); cudaFree(h->d_Ecand); cudaFree(h->d_cs); cudaFree(h->d_sigma);
  cudaFree(h->d_log);
}

// one launch: propose B candidates per chain, score them, accept/reject, commit
int chains_enqueue(tp3_chains* h) {
  tp3_ctx* c = h->ctx;
  const int n = h->nch * h->B;
  k_propose<<<n, 256, 0, c->stream>>>(h->d_state, h->d_cand, h->d_cs, h->d_sigma, h->nl, h->B, h->K, h->LMAX, h->L,
                                      h->f, h->seed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "propose");
  if (int r = tp3::ctx_run_energy(c, n, h->d_cand, h->d_Ecand)) return r;
  k_select<<<(h->nch + 127) / 128, 128, 0, c->stream>>>(h->d_cs, h->d_sigma, h->d_Ecand, h->nch, h->nl, h->B, h->f,
                                                          h->decay, h->seed, h->d_log, h->logcap, h->nl - 1);
  k_commit<<<h->nch, 256, 0, c->stream>>>(h->d_state, h->d_cand, h->d_cs, h->B, h->K * h->ncoef);
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
  return r;
}

}  // namespace

extern "C" {

int tp3_chains_create(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                      double initial_stepsize, double stepsizefactor, double temperature_decay, uint64_t seed,
                      int log_capacity, tp3_chains** out) {
  if (int r = tp3::ctx_check(ctx)) return r;
  if (!out || !coeff0 || !T0 || nchains < 1 || ncand < 1 || log_capacity < 0)
    return tp3::ctx_fail(ctx, TP3_ERR_ARG, "bad chain arguments");
  if (!(stepsizefactor > 0.0) || !(temperature_decay > 0.0))
    return tp3::ctx_fail(ctx, TP3_ERR_ARG, "step-size factor and temperature decay must be positive");
  if (ctx->b.L > kMaxL) return tp3::ctx_fail(ctx, TP3_ERR_UNSUPPORTED, "chains need L <= 62");
  if (!ctx->has_hist) return tp3::ctx_fail(ctx, TP3_ERR_NO_HISTOGRAM, "tp3_set_histogram has not been called");
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
  double* dE0 = h->d_Ecand;  // scratch for the initial energies
  if (int r = tp3::ctx_run_energy(ctx, nchains, h->d_state, dE0)) { chains_free(h); delete h; return r; }
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
    cs[i].E = E0[i]; cs[i].T = T0[i]; cs[i].step = 0; cs[i].accepted = 0; cs[i].last = -1; cs[i].pad = 0;
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
  if (h->graph_gen != c->scratch_gen || h->graph_mode != c->mode) {
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
  const size_t hdr = 8 * sizeof(int64_t);
  const size_t need = hdr + nst + ncs + nsg;
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
      (e = cudaMemcpy(p + hdr + nst + ncs, h->d_sigma, nsg, cudaMemcpyDeviceToHost)) != cudaSuccess)
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
  const size_t hdr = 8 * sizeof(int64_t);
  if (bytes != hdr + nst + ncs + nsg) return tp3::ctx_fail(c, TP3_ERR_ARG, "snapshot size does not match these chains");
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
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "restore copy");
  return TP3_OK;
}

int tp3_chains_graph(const tp3_chains* h, int* captured) {
  if (!h || !captured) return TP3_ERR_ARG;
  *captured = h->exec != nullptr;
  return TP3_OK;
}

}  // extern "C"
