// Plain FP32 path: one proposal = gather -> direct coupling -> SIMT angular
// contraction with the Bayes terms fused into its epilogue -> FP64 finalize.
//
// This is the straightforward GPU form of the reference computation
// (src/correlations.jl:157-226; src/cuda_kernel.cu:14-43 + cublasSgemm at
// src/cuda.jl:88), kept as the comparison baseline for the tensor-core path:
//   * coupling: T[ki][lt] = sum_{j in lt} w_j Re(c_k1[i1] c_k2[i2] c_k3[i3]),
//     one thread per (shell triple, l-triple), the l-triple's 3j terms read as
//     warp-uniform broadcasts (the reference's As loop, without materialising the
//     basislen x klength PA matrix);
//   * angular: c3[ki][g] = sum_lt T[ki][lt] F[g][lt] over the full N x 2N grid,
//     FP32 FMA, 64 x 64 register-tiled;
//   * Bayes: per slab, Sp = sum_g max(c3, 1e-30) and Sql = sum_g q^[g] log max(c3, 1e-30)
//     (q^ = the L1-normalised histogram slab); E = sum_ki tf (Qs log Sp - Sql), which
//     equals sum_ki tf * (-sum_g q^ log p^) of correlations.jl:210-220 with Qs = sum_g q^.
#include <cuda_bf16.h>

#include "internal.h"

#include <cstdint>

namespace tp3 {

namespace {

__global__ void k_gather(int n, int K, int nc, int ncoef, const int* __restrict__ csean,
                         const double2* __restrict__ coeff, float2* __restrict__ cc) {
  const int64_t total = (int64_t)n * K * nc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % nc);
    const int64_t pk = i / nc;  // prop * K + k
    const double2 v = coeff[pk * ncoef + csean[c]];
    cc[i] = make_float2((float)v.x, (float)v.y);
  }
}

// grid: (ceil(klength/32), ceil(n_lt/32), n); block 256; dyn smem K*nc float2
__global__ void __launch_bounds__(256) k_couple_direct(
    const float2* __restrict__ cc, int K, int nc, const float* __restrict__ w,
    const uint32_t* __restrict__ idx, const int2* __restrict__ lt, int n_lt,
    const int4* __restrict__ kl, int klength, float* __restrict__ T, int ldT, int64_t T_stride) {
  extern __shared__ float2 sc[];
  __shared__ float tile[32][33];
  const int prop = blockIdx.z;
  const float2* src = cc + (int64_t)prop * K * nc;
  for (int i = threadIdx.x; i < K * nc; i += blockDim.x) sc[i] = src[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ki0 = blockIdx.x * 32, lt0 = blockIdx.y * 32;
  const int ki = ki0 + lane;
  const int4 k = kl[ki < klength ? ki : klength - 1];
  const float2* c1 = sc + k.x * nc;
  const float2* c2 = sc + k.y * nc;
  const float2* c3 = sc + k.z * nc;
#pragma unroll 1
  for (int r = 0; r < 4; ++r) {
    const int t = lt0 + warp + 8 * r;
    float acc = 0.f;
    if (t < n_lt) {
      const int2 js = lt[t];
      for (int j = js.x; j < js.x + js.y; ++j) {
        const uint32_t id = idx[j];
        const float wj = w[j];
        const float2 a = c1[id & 1023u], b = c2[(id >> 10) & 1023u], c = c3[(id >> 20) & 1023u];
        const float abr = a.x * b.x - a.y * b.y;
        const float abi = a.x * b.y + a.y * b.x;
        acc = fmaf(wj, abr * c.x - abi * c.y, acc);
      }
    }
    tile[lane][warp + 8 * r] = acc;
  }
  __syncthreads();
  float* Tp = T + (int64_t)prop * T_stride;
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int row = e >> 5, col = e & 31;
    if (ki0 + row < klength && lt0 + col < n_lt) Tp[(int64_t)(ki0 + row) * ldT + lt0 + col] = tile[row][col];
  }
}

// grid: (ceil(klength/64), ncg, n); block 256 (16 x 16 threads, 4 x 4 per thread).
// STORE: write c3 rows (out[prop][ki][g]); otherwise accumulate Bayes partials.
template <bool STORE>
__global__ void __launch_bounds__(256) k_angular_plain(
    const float* __restrict__ T, int ldT, int64_t T_stride, const float* __restrict__ F, int Kdim,
    int klength, int G, int cols_per_group, const float* __restrict__ q, double2* __restrict__ part,
    int ncg, float* __restrict__ out) {
  __shared__ __align__(16) float As[16][64 + 4];
  __shared__ __align__(16) float Bs[16][64 + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int prop = blockIdx.z, cg = blockIdx.y;
  const int r0 = blockIdx.x * 64;
  const float* Tp = T + (int64_t)prop * T_stride;
  const int cbeg = cg * cols_per_group;
  const int cend = min(G, cbeg + cols_per_group);
  // compensated (Kahan) per-row sums
  float Sp[4] = {0.f, 0.f, 0.f, 0.f}, Sql[4] = {0.f, 0.f, 0.f, 0.f};
  float Cp[4] = {0.f, 0.f, 0.f, 0.f}, Cq[4] = {0.f, 0.f, 0.f, 0.f};
  // loader mapping: 64 rows x 16 k = 256 float4
  const int lrow = tid >> 2, lk = (tid & 3) * 4;
  for (int c0 = cbeg; c0 < cend; c0 += 64) {
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < Kdim; k0 += 16) {
      const float4 av = *reinterpret_cast<const float4*>(Tp + (int64_t)(r0 + lrow) * ldT + k0 + lk);
      const int gcol = min(c0 + lrow, G - 1);
      const float4 bv = *reinterpret_cast<const float4*>(F + (int64_t)gcol * ldT + k0 + lk);
      As[lk + 0][lrow] = av.x; As[lk + 1][lrow] = av.y; As[lk + 2][lrow] = av.z; As[lk + 3][lrow] = av.w;
      Bs[lk + 0][lrow] = bv.x; Bs[lk + 1][lrow] = bv.y; Bs[lk + 2][lrow] = bv.z; Bs[lk + 3][lrow] = bv.w;
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < 16; ++kk) {
        const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
        const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
        const float ar[4] = {a.x, a.y, a.z, a.w}, br[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(ar[i], br[j], acc[i][j]);
      }
      __syncthreads();
    }
    const int col = c0 + tx * 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = r0 + ty * 4 + i;
      if (row >= klength) continue;
      if (STORE) {
        float* o = out + ((int64_t)prop * klength + row) * G;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (col + j < cend) o[col + j] = acc[i][j];
      } else {
        const float* qr = q + (int64_t)row * G;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (col + j < cend) {
            const float p = fmaxf(acc[i][j], 1e-30f);
            const float y1 = p - Cp[i];
            const float t1 = Sp[i] + y1;
            Cp[i] = (t1 - Sp[i]) - y1;
            Sp[i] = t1;
            const float y2 = qr[col + j] * __logf(p) - Cq[i];
            const float t2 = Sql[i] + y2;
            Cq[i] = (t2 - Sql[i]) - y2;
            Sql[i] = t2;
          }
        }
      }
    }
  }
  if (STORE) return;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    double sp = (double)Sp[i] - (double)Cp[i], sq = (double)Sql[i] - (double)Cq[i];
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
      sp += __shfl_xor_sync(0xffffffffu, sp, off);
      sq += __shfl_xor_sync(0xffffffffu, sq, off);
    }
    const int row = r0 + ty * 4 + i;
    if (tx == 0 && row < klength)
      part[((int64_t)prop * ncg + cg) * klength + row] = make_double2(sp, sq);
  }
}

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// grid: n; block 256.  Deterministic compensated sum of the per-slab energies.
__global__ void __launch_bounds__(256) k_finalize(const double2* __restrict__ part, int ncg, int klength,
                                                  const double* __restrict__ Qs,
                                                  const double* __restrict__ tf, int mult,
                                                  double* __restrict__ E) {
  __shared__ double ss[256], sc[256];
  const int prop = blockIdx.x;
  const double2* pp = part + (int64_t)prop * ncg * klength;
  double s = 0.0, c = 0.0;
  for (int ki = threadIdx.x; ki < klength; ki += blockDim.x) {
    double sp = 0.0, sq = 0.0;
    for (int g = 0; g < ncg; ++g) {
      const double2 v = pp[(int64_t)g * klength + ki];
      sp += v.x;
      sq += v.y;
    }
    const double e = tf[ki] * (Qs[ki] * log((double)mult * sp) - sq);
    double t, err;
    two_sum(s, e, t, err);
    s = t;
    c += err;
  }
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      double t, err;
      two_sum(ss[threadIdx.x], ss[threadIdx.x + h], t, err);
      ss[threadIdx.x] = t;
      sc[threadIdx.x] += sc[threadIdx.x + h] + err;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) E[prop] = ss[0] + sc[0];
}

}  // namespace


int plain_ncg(const DevTables& t) {
  // about 512 grid columns per block, at least one group
  int ncg = (t.G + 511) / 512;
  return ncg < 1 ? 1 : ncg;
}

cudaError_t launch_gather(const DevTables& t, int n, const double2* coeff, CoeffLayout lay, float2* cc,
                          cudaStream_t s) {
  const int64_t total = (int64_t)n * t.K * t.nc;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  k_gather<<<blocks, 256, 0, s>>>(n, t.K, t.nc, lay.stride, lay.map, coeff, cc);
  return cudaGetLastError();
}

cudaError_t launch_couple_direct(const DevTables& t, int n, const float2* cc, float* T, cudaStream_t s) {
  const size_t smem = (size_t)t.K * t.nc * sizeof(float2);
  dim3 grid((t.klength + 31) / 32, (t.n_lt + 31) / 32, n);
  k_couple_direct<<<grid, 256, smem, s>>>(cc, t.K, t.nc, t.w, t.idx, t.lt, t.n_lt, t.kl, t.klength, T,
                                          t.n_ltp, (int64_t)t.klp * t.n_ltp);
  return cudaGetLastError();
}

cudaError_t launch_angular_plain(const DevTables& t, int n, const float* T, const float* q,
                                 double2* part, int ncg, float* c3out, cudaStream_t s) {
  const int cpg = ((t.G + ncg - 1) / ncg + 63) / 64 * 64;
  dim3 grid((t.klength + 63) / 64, ncg, n);
  // lambda = 0: A = T [klp][n_ltp] against F; otherwise A = H [klp][nqp] against the cosine table
  const bool hform = t.nqp > 0;
  const int kd = hform ? t.nqp : t.n_ltp;
  const float* tab = hform ? t.Cq : t.Ffull;
  const int64_t Ts = (int64_t)t.klp * kd;
  if (c3out)
    k_angular_plain<true><<<grid, 256, 0, s>>>(T, kd, Ts, tab, kd, t.klength, t.G, cpg, nullptr, nullptr, ncg,
                                               c3out);
  else
    k_angular_plain<false><<<grid, 256, 0, s>>>(T, kd, Ts, tab, kd, t.klength, t.G, cpg, q, part, ncg, nullptr);
  return cudaGetLastError();
}

// grid: (ceil(klength/32), ceil(nq/8), n); block 256 (warp w: pair q0 + w; lane: shell triple).
// H[ki][q] = sum_{j with (m2, m3) = +-q} w_j Y(l1,m1,th_k1) Y(l2,m2,th_k2) Y(l3,m3,th_k3) T[ki][lt(j)]
// (lambda != 0: the Legendre factors depend on the shells, so the angular stage contracts
// over Fourier pairs (m2, m3) instead of l-triples; src/correlations.jl:137-148, 182).
__global__ void __launch_bounds__(256) k_build_H(const float* __restrict__ T, int n_ltp, int64_t T_stride,
                                                 const float* __restrict__ Ytab, int K, int nc,
                                                 const float* __restrict__ w, const uint32_t* __restrict__ idx,
                                                 const int* __restrict__ lt_of_j, const int* __restrict__ qstart,
                                                 const int* __restrict__ qlist, int nq, const int4* __restrict__ kl,
                                                 int klength, float* __restrict__ H, int nqp, int64_t H_stride) {
  extern __shared__ float sm[];
  float* sY = sm;                      // [K][nc]
  float* sT = sm + (size_t)K * nc;     // [32][n_ltp + 1]: an odd row stride keeps the lanes'
                                       // reads of one l-triple in different banks
  const int rs = n_ltp + 1;
  const int prop = blockIdx.z;
  const int ki0 = blockIdx.x * 32;
  for (int i = threadIdx.x; i < K * nc; i += blockDim.x) sY[i] = Ytab[i];
  const float* Tp = T + (int64_t)prop * T_stride;
  for (int i = threadIdx.x; i < 32 * n_ltp; i += blockDim.x) {
    const int r = i / n_ltp, c = i - r * n_ltp;
    sT[r * rs + c] = ki0 + r < klength ? Tp[(int64_t)(ki0 + r) * n_ltp + c] : 0.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int q = blockIdx.y * 8 + warp;
  const int ki = ki0 + lane;
  if (q >= nq || ki >= klength) return;
  const int4 k = kl[ki];
  const float* y1 = sY + k.x * nc;
  const float* y2 = sY + k.y * nc;
  const float* y3 = sY + k.z * nc;
  const float* trow = sT + lane * rs;
  float acc = 0.f;
  for (int e = qstart[q]; e < qstart[q + 1]; ++e) {
    const int j = qlist[e];
    const uint32_t id = idx[j];
    acc = fmaf(w[j] * y1[id & 1023u] * y2[(id >> 10) & 1023u] * y3[(id >> 20) & 1023u], trow[lt_of_j[j]], acc);
  }
  H[(int64_t)prop * H_stride + (int64_t)ki * nqp + q] = acc;
}

cudaError_t launch_build_H(const DevTables& t, int n, const float* T, float* H, cudaStream_t s) {
  const size_t smem = ((size_t)t.K * t.nc + 32 * (size_t)(t.n_ltp + 1)) * sizeof(float);
  dim3 grid((t.klength + 31) / 32, (t.nq + 7) / 8, n);
  k_build_H<<<grid, 256, smem, s>>>(T, t.n_ltp, (int64_t)t.klp * t.n_ltp, t.Ytab, t.K, t.nc, t.w, t.idx, t.lt_of_j,
                                    t.qstart, t.qlist, t.nq, t.kl, t.klength, H, t.nqp, (int64_t)t.klp * t.nqp);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DevTables& t, int n, const double2* part, int ncg, const double* Qs,
                            int mult, double* E, cudaStream_t s) {
  k_finalize<<<n, 256, 0, s>>>(part, ncg, t.klength, Qs, t.tf, mult, E);
  return cudaGetLastError();
}

// Tensor-core path at lambda != 0: the Fourier-pair operand H of a batch, written as the
// angular kernel's split A operand.  grid: (klength, ceil(n / PB)); block kHWarps warps;
// PB = 32 PPL proposals per block, PPL per lane.  One block = one shell triple ki:
//   H[prop][ki][q] = sum_{j with (m2, m3) = +-q} T[prop][ki][lt(j)] w_j Y1 Y2 Y3,
// the Legendre product of entry j at the triple's three shells formed once per block and
// applied to all PB proposals.  T rows are staged transposed (l-triple major, proposals
// fastest, row stride PB + 2 or PB + 1 so the lanes' loads and the transposing stores
// stay in distinct banks), with the triple's three Legendre rows.  Warps take pairs q;
// per pair, the lanes first form the products of up to kHChunk entries (independent
// 16-byte entry loads, packed indices / w / l-triple in pair order) into the warp's
// buffer, then stream them as broadcasts against the staged T.  Results go through a
// 64-pair tile in shared memory and leave as rows of consecutive pairs, split into
// hi + lo (bf16, or tf32-rounded fp32 + fp32 remainder).  Pair columns nq..KP-1 are zero.
constexpr int kHWarps = 16;
constexpr int kHChunk = 128;

template <int PPL>
__global__ void __launch_bounds__(kHWarps * 32, 1) k_build_H_split(
    const float* __restrict__ T32, int ldT, int64_t Tstride, int n, int n_lt, const float* __restrict__ Ytab, int nc,
    const int4* __restrict__ qent, const int* __restrict__ qstart, int nq, const int4* __restrict__ kl, int klp, int KP,
    int tf32, void* __restrict__ Hhi, void* __restrict__ Hlo) {
  constexpr int PB = 32 * PPL;
  constexpr int RS = PB + (PPL == 2 ? 2 : 1);
  constexpr int HS = PB + 1;
  extern __shared__ float smh[];
  float* Ts = smh;                     // [n_lt][RS]
  float* Hs = Ts + (size_t)n_lt * RS;  // [64][HS]
  // [kHWarps][kHChunk] (P, T-row offset bits), 16-byte aligned for the float4 reads
  float2* Pb = reinterpret_cast<float2*>(smh + (((size_t)n_lt * RS + 64 * HS + 3) & ~(size_t)3));
  float* Ys = reinterpret_cast<float*>(Pb + kHWarps * kHChunk);  // [3][nc]
  const int ki = blockIdx.x, p0 = blockIdx.y * PB;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int4 k = kl[ki];
  for (int i = threadIdx.x; i < 3 * nc; i += blockDim.x) {
    const int r = i / nc, cix = i - r * nc;
    Ys[i] = Ytab[(size_t)(r == 0 ? k.x : r == 1 ? k.y : k.z) * nc + cix];
  }
  for (int i = threadIdx.x; i < n_lt * PB; i += blockDim.x) {
    const int pr = i / n_lt, l = i - pr * n_lt;
    Ts[l * RS + pr] = p0 + pr < n ? T32[(int64_t)(p0 + pr) * Tstride + (int64_t)ki * ldT + l] : 0.f;
  }
  __syncthreads();
  float2* pw = Pb + warp * kHChunk;
  for (int qb = 0; qb < KP; qb += 64) {
    for (int qq = warp; qq < 64; qq += kHWarps) {
      const int q = qb + qq;
      // two accumulator sets (even / odd entries) per proposal of the lane
      float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
      if (q < nq) {
        const int e1 = qstart[q + 1];
        for (int e0 = qstart[q]; e0 < e1; e0 += kHChunk) {
          const int cnt = min(kHChunk, e1 - e0);
          const int cnt8 = (cnt + 7) & ~7;
          // products and the l-triple's T-row offset (in floats); padding entries are 0
#pragma unroll 4
          for (int i = lane; i < cnt8; i += 32) {
            float P = 0.f;
            int off = 0;
            if (i < cnt) {
              const int4 en = qent[e0 + i];
              const uint32_t id = (uint32_t)en.x;
              P = __int_as_float(en.y) * Ys[id & 1023u] * Ys[nc + ((id >> 10) & 1023u)] *
                  Ys[2 * nc + ((id >> 20) & 1023u)];
              off = en.z * RS;
            }
            pw[i] = make_float2(P, __int_as_float(off));
          }
          __syncwarp();
          const float4* pw4 = reinterpret_cast<const float4*>(pw);
          for (int i = 0; i < cnt8; i += 8) {
            float pv[8];
            int po[8];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float4 v = pw4[i / 2 + u];
              pv[2 * u] = v.x;
              po[2 * u] = __float_as_int(v.y);
              pv[2 * u + 1] = v.z;
              po[2 * u + 1] = __float_as_int(v.w);
            }
            if (PPL == 2) {
              float2 tv[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) tv[u] = *reinterpret_cast<const float2*>(Ts + po[u] + 2 * lane);
#pragma unroll
              for (int u = 0; u < 8; u += 2) {
                a0 = fmaf(pv[u], tv[u].x, a0);
                a1 = fmaf(pv[u], tv[u].y, a1);
                b0 = fmaf(pv[u + 1], tv[u + 1].x, b0);
                b1 = fmaf(pv[u + 1], tv[u + 1].y, b1);
              }
            } else {
              float tv[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) tv[u] = Ts[po[u] + lane];
#pragma unroll
              for (int u = 0; u < 8; u += 2) {
                a0 = fmaf(pv[u], tv[u], a0);
                b0 = fmaf(pv[u + 1], tv[u + 1], b0);
              }
            }
          }
          __syncwarp();
        }
      }
      Hs[qq * HS + PPL * lane] = a0 + b0;
      if (PPL == 2) Hs[qq * HS + 2 * lane + 1] = a1 + b1;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < PB * 64; i += blockDim.x) {
      const int pr = i >> 6, qq = i & 63, q = qb + qq;
      if (p0 + pr >= n || q >= KP) continue;
      const float v = q < nq ? Hs[qq * HS + pr] : 0.f;
      const size_t o = ((size_t)(p0 + pr) * klp + ki) * KP + q;
      if (tf32) {
        uint32_t h;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
        const float hf = __uint_as_float(h);
        reinterpret_cast<float*>(Hhi)[o] = hf;
        reinterpret_cast<float*>(Hlo)[o] = v - hf;
      } else {
        const __nv_bfloat16 hb = __float2bfloat16_rn(v);
        reinterpret_cast<__nv_bfloat16*>(Hhi)[o] = hb;
        reinterpret_cast<__nv_bfloat16*>(Hlo)[o] = __float2bfloat16_rn(v - __bfloat162float(hb));
      }
    }
    __syncthreads();
  }
}

size_t build_H_split_smem(const DevTables& t, int ppl) {
  const int PB = 32 * ppl;
  const size_t pbo = ((size_t)t.n_lt * (PB + (ppl == 2 ? 2 : 1)) + 64 * (size_t)(PB + 1) + 3) & ~(size_t)3;
  return (pbo + 2 * (size_t)kHWarps * kHChunk + 3 * (size_t)t.nc) * sizeof(float);
}

cudaError_t launch_build_H_split(const DevTables& t, int KP, int n, const float* T32, void* Hhi, void* Hlo, bool tf32,
                                 cudaStream_t s) {
  const int ppl = build_H_split_smem(t, 2) <= (size_t)kPlainMaxSmem ? 2 : 1;
  const size_t smem = build_H_split_smem(t, ppl);
  if (smem > (size_t)kPlainMaxSmem) return cudaErrorInvalidConfiguration;
  const dim3 grid(t.klength, (n + 32 * ppl - 1) / (32 * ppl));
  const int64_t Ts = (int64_t)t.klp * t.n_ltp;
  if (ppl == 2)
    k_build_H_split<2><<<grid, kHWarps * 32, smem, s>>>(T32, t.n_ltp, Ts, n, t.n_lt, t.Ytab, t.nc, t.qent, t.qstart,
                                                        t.nq, t.kl, t.klp, KP, tf32 ? 1 : 0, Hhi, Hlo);
  else
    k_build_H_split<1><<<grid, kHWarps * 32, smem, s>>>(T32, t.n_ltp, Ts, n, t.n_lt, t.Ytab, t.nc, t.qent, t.qstart,
                                                        t.nq, t.kl, t.klp, KP, tf32 ? 1 : 0, Hhi, Hlo);
  return cudaGetLastError();
}

cudaError_t plain_configure() {
  const cudaFuncAttribute ds = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_couple_direct, ds, kPlainMaxSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_build_H, ds, kPlainMaxSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_build_H_split<1>, ds, kPlainMaxSmem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_build_H_split<2>, ds, kPlainMaxSmem)) != cudaSuccess)
    return e;
  return cudaSuccess;
}

}  // namespace tp3
