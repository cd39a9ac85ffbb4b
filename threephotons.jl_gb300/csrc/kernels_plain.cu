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
  float* sT = sm + (size_t)K * nc;     // [32][n_ltp]
  const int prop = blockIdx.z;
  const int ki0 = blockIdx.x * 32;
  for (int i = threadIdx.x; i < K * nc; i += blockDim.x) sY[i] = Ytab[i];
  const float* Tp = T + (int64_t)prop * T_stride;
  for (int i = threadIdx.x; i < 32 * n_ltp; i += blockDim.x) {
    const int r = i / n_ltp, c = i - r * n_ltp;
    sT[i] = ki0 + r < klength ? Tp[(int64_t)(ki0 + r) * n_ltp + c] : 0.f;
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
  const float* trow = sT + lane * n_ltp;
  float acc = 0.f;
  for (int e = qstart[q]; e < qstart[q + 1]; ++e) {
    const int j = qlist[e];
    const uint32_t id = idx[j];
    acc = fmaf(w[j] * y1[id & 1023u] * y2[(id >> 10) & 1023u] * y3[(id >> 20) & 1023u], trow[lt_of_j[j]], acc);
  }
  H[(int64_t)prop * H_stride + (int64_t)ki * nqp + q] = acc;
}

cudaError_t launch_build_H(const DevTables& t, int n, const float* T, float* H, cudaStream_t s) {
  const size_t smem = ((size_t)t.K * t.nc + 32 * (size_t)t.n_ltp) * sizeof(float);
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

cudaError_t plain_configure() {
  cudaError_t e = cudaFuncSetAttribute(k_couple_direct, cudaFuncAttributeMaxDynamicSharedMemorySize, kPlainMaxSmem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_build_H, cudaFuncAttributeMaxDynamicSharedMemorySize, kPlainMaxSmem);
}

}  // namespace tp3
