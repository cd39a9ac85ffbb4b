// Stage (a) as two barrier-free kernels (the "split" coupling variant).
//
// The pair-factorised coupling (see kernels_tc.cu) has two phases per (l1, l2) block:
//   phase 1  D[(k1,k2)][l3][m3] = sum_m1 w(l1 m1 l2 m2 l3 m3) c_k1[l1,m1] c_k2[l2,m2]
//   phase 2  T[(k1,k2,k3)][(l1,l2,l3)] = Re sum_m3 D[(k1,k2)][l3][m3] c_k3[l3,m3]
// In one kernel the phases are separated by block-wide barriers, and uneven item costs
// leave warps waiting.  Here each phase is its own kernel and D goes through global
// memory; proposals are processed in sub-batches small enough that D stays resident
// in the 126 MB L2 between the two launches.  Neither kernel has a barrier after its
// initial shared-memory fill, and both fit two CTAs per SM.
//   k_couple_d: grid (pair blocks, proposals in the sub-batch); items (m3, shell pair),
//               lanes of a warp share m3 (broadcast 3j reads, equal loop trip counts).
//   k_couple_t: grid (pair blocks, k1, proposals); items (l3, 4 x 4 tile of (k2, k3)).
// Real-function coefficients (sym flag from k_gather_sym): only m3 >= 0 of D is formed
// and T = Re(D[0] c[0]) + 2 sum_{m3>0} Re(D[m3] c[m3]).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace tp3 {
namespace {

constexpr int kThreadsD = 256;
constexpr int kThreadsT = 256;

__device__ __forceinline__ int ki_of(int k1, int k2, int k3) {
  return k1 * (k1 + 1) * (k1 + 2) / 6 + k2 * (k2 + 1) / 2 + k3;
}

// One CTA = one work unit (pair block, m3 range) of one proposal: all shell pairs for
// m3 in [m3lo, m3hi].  Shared memory: the coefficients of l1 and l2 of every shell and
// the unit's 3j rows.
template <int MAXS>
__global__ void __launch_bounds__(kThreadsD, 3) k_couple_d(
    const float2* __restrict__ cc, int K, int nc, const int* __restrict__ coff,
    const PairBlock* __restrict__ pbs, const int* __restrict__ eofs, const float* __restrict__ wtab,
    const int4* __restrict__ units_sym, int n_units_sym, const int4* __restrict__ units_gen, int n_units_gen,
    const long long* __restrict__ doff, long long dstride, const int* __restrict__ symflags,
    float2* __restrict__ Dg, int prop0) {
  extern __shared__ __align__(16) float smf[];
  const int prop = prop0 + blockIdx.y;
  const bool sym = symflags[prop] != 0;
  if ((int)blockIdx.x >= (sym ? n_units_sym : n_units_gen)) return;
  const int4 u = (sym ? units_sym : units_gen)[blockIdx.x];  // (pb, m3lo, m3hi, -)
  const PairBlock pb = pbs[u.x];
  const int l1 = pb.l1, l2 = pb.l2, nl3 = pb.nl3, nl3p = pb.nl3p, l3min = pb.l3min, M = pb.M, SD = pb.SD;
  const int d1 = 2 * l1 + 1, d2 = 2 * l2 + 1;
  float2* s1 = reinterpret_cast<float2*>(smf);        // [K][d1]  c_k[l1, m1 + l1]
  float2* s2 = s1 + (size_t)K * d1;                    // [K][d2]  c_k[l2, m2 + l2]
  float* sw = reinterpret_cast<float*>(s2 + (size_t)K * d2);
  sw = reinterpret_cast<float*>(((uintptr_t)sw + 15) & ~(uintptr_t)15);
  const float2* src = cc + (size_t)prop * K * nc;
  const int o1 = coff[l1 >> 1], o2 = coff[l2 >> 1];
  for (int i = threadIdx.x; i < K * d1; i += blockDim.x) s1[i] = src[(i / d1) * nc + o1 + i % d1];
  for (int i = threadIdx.x; i < K * d2; i += blockDim.x) s2[i] = src[(i / d2) * nc + o2 + i % d2];
  // the unit's 3j rows: e = m3 + M in [m3lo + M, m3hi + M], contiguous in the block
  const int wbeg = eofs[pb.eofs + u.y + M];
  const int wend = (u.z + M + 1 <= 2 * M) ? eofs[pb.eofs + u.z + M + 1] : pb.wcount;
  {
    const float* wsrc = wtab + pb.wofs + wbeg;
    for (int i = threadIdx.x; i < wend - wbeg; i += blockDim.x) sw[i] = wsrc[i];
  }
  __syncthreads();
  const int npairs = K * (K + 1) / 2;
  float2* Dblk = Dg + (size_t)blockIdx.y * dstride + doff[u.x];
  const int nm3 = u.z - u.y + 1;
  const int items = npairs * nm3;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int eo = it / npairs, p = it - eo * npairs;
    // heaviest first: the m3 closest to zero
    int m3;
    if (u.y >= 0) m3 = u.y + eo;
    else if (u.z <= 0) m3 = u.z - eo;
    else m3 = (eo & 1) ? -((eo + 1) >> 1) : (eo >> 1);  // range straddles 0 (general path)
    if (m3 < u.y || m3 > u.z) continue;
    int k1 = (int)((sqrtf(8.f * p + 1.f) - 1.f) * 0.5f);
    while (k1 * (k1 + 1) / 2 > p) --k1;
    while ((k1 + 1) * (k1 + 2) / 2 <= p) ++k1;
    const int k2 = p - k1 * (k1 + 1) / 2;
    const int m1lo = max(-l1, -l2 - m3), m1hi = min(l1, l2 - m3);
    const float2* wr = reinterpret_cast<const float2*>(sw + (eofs[pb.eofs + m3 + M] - wbeg));
    const float2* c1 = s1 + k1 * d1 + l1;
    const float2* c2 = s2 + k2 * d2 + l2 - m3;
    const int wstep = nl3p >> 1;
    float ar[MAXS], ai[MAXS];
#pragma unroll
    for (int s = 0; s < MAXS; ++s) { ar[s] = 0.f; ai[s] = 0.f; }
    for (int m1 = m1lo; m1 <= m1hi; ++m1, wr += wstep) {
      const float2 a = c1[m1];
      const float2 b = c2[-m1];
      const float xr = a.x * b.x - a.y * b.y;
      const float xi = a.x * b.y + a.y * b.x;
#pragma unroll
      for (int s2 = 0; s2 < (MAXS + 1) / 2; ++s2) {
        if (2 * s2 < nl3) {
          const float2 wv = wr[s2];
          ar[2 * s2] = fmaf(wv.x, xr, ar[2 * s2]);
          ai[2 * s2] = fmaf(wv.x, xi, ai[2 * s2]);
          if (2 * s2 + 1 < MAXS) {
            ar[2 * s2 + 1] = fmaf(wv.y, xr, ar[2 * s2 + 1]);
            ai[2 * s2 + 1] = fmaf(wv.y, xi, ai[2 * s2 + 1]);
          }
        }
      }
    }
    float2* d = Dblk + (size_t)p * SD;
    int dofs = 0;
#pragma unroll
    for (int s = 0; s < MAXS; ++s) {
      if (s < nl3) {
        const int l3 = l3min + 2 * s;
        if (m3 >= -l3 && m3 <= l3) d[dofs + m3 + l3] = make_float2(ar[s], ai[s]);
        dofs += 2 * l3 + 1;
      }
    }
  }
}

__global__ void __launch_bounds__(kThreadsT, 2) k_couple_t(
    const float2* __restrict__ cc, int K, int nc, int ncp, const int* __restrict__ coff,
    const PairBlock* __restrict__ pbs, const long long* __restrict__ doff, long long dstride,
    const int* __restrict__ symflags, const float2* __restrict__ Dg, int prop0, int klp, int KP,
    void* __restrict__ Thi, void* __restrict__ Tlo, bool tf32, float* __restrict__ T32, int ldT32) {
  extern __shared__ __align__(16) float smf[];
  const int k1 = K - 1 - (int)blockIdx.y;
  const int sub = blockIdx.z;
  const int prop = prop0 + sub;
  const PairBlock pb = pbs[blockIdx.x];
  const bool sym = symflags[prop] != 0;
  const int nk = k1 + 1;
  const int SD = pb.SD;
  float2* sc = reinterpret_cast<float2*>(smf);  // [nk][ncp]
  float2* sD = sc + (size_t)nk * ncp;           // [nk][SD]: pairs (k1, 0..k1)
  const float2* src = cc + (size_t)prop * K * nc;
  for (int i = threadIdx.x; i < nk * nc; i += blockDim.x) {
    const int k = i / nc, c = i - k * nc;
    sc[k * ncp + c] = src[i];
  }
  const float2* Drows = Dg + (size_t)sub * dstride + doff[blockIdx.x] + (size_t)(k1 * (k1 + 1) / 2) * SD;
  for (int i = threadIdx.x; i < nk * SD; i += blockDim.x) sD[i] = Drows[i];
  __syncthreads();
  const int nl3 = pb.nl3, l3min = pb.l3min;
  const int nq = (k1 + 4) >> 2;
  const int tiles = nq * (nq + 1) / 2;
  const int items = tiles * nl3;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int s = nl3 - 1 - it / tiles;  // largest l3 first
    int t = it % tiles;
    int ra = 0;
    while (t > ra) { t -= ra + 1; ++ra; }
    const int rb = t;
    const int l3 = l3min + 2 * s;
    const int dofs = s * (2 * l3min + 2 * s - 1);
    const int off3 = coff[l3 >> 1] + l3;
    const float2* drow[4];
    const float2* crow[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      drow[i] = sD + (size_t)min(4 * ra + i, k1) * SD + dofs + l3;
      crow[i] = sc + min(4 * rb + i, k1) * ncp + off3;
    }
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int m3 = sym ? 1 : -l3; m3 <= l3; ++m3) {
      float2 x[4], y[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { x[i] = drow[i][m3]; y[i] = crow[i][m3]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(x[i].x, y[j].x, fmaf(-x[i].y, y[j].y, acc[i][j]));
    }
    if (sym) {
      float2 x[4], y[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { x[i] = drow[i][0]; y[i] = crow[i][0]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(x[i].x, y[j].x, fmaf(-x[i].y, y[j].y, 2.f * acc[i][j]));
    }
    const int lt = pb.lt_base + s;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k2 = 4 * ra + i;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k3 = 4 * rb + j;
        if (k2 <= k1 && k3 <= k2) {
          const int ki = ki_of(k1, k2, k3);
          const float v = acc[i][j];
          const size_t o = ((size_t)prop * klp + ki) * KP + lt;
          if (tf32) {
            uint32_t h;
            asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
            reinterpret_cast<float*>(Thi)[o] = __uint_as_float(h);
            reinterpret_cast<float*>(Tlo)[o] = v - __uint_as_float(h);
          } else {
            const __nv_bfloat16 hi = __float2bfloat16_rn(v);
            reinterpret_cast<__nv_bfloat16*>(Thi)[o] = hi;
            reinterpret_cast<__nv_bfloat16*>(Tlo)[o] = __float2bfloat16_rn(v - __bfloat162float(hi));
          }
          if (T32) T32[((size_t)prop * klp + ki) * ldT32 + lt] = v;
        }
      }
    }
  }
}

}  // namespace

size_t couple_split_smem_d(const DevTables& t, const TcTables& tc) {
  return (size_t)t.K * (2 * tc.dmax + 1) * 2 * sizeof(float2) + 16 + (size_t)tc.unit_wmax * sizeof(float);
}

size_t couple_split_smem_t(const DevTables& t, const TcTables& tc) {
  return (size_t)t.K * (tc.ncp + tc.SDmax) * sizeof(float2);
}

cudaError_t couple_split_configure(const DevTables& t, const TcTables& tc) {
  cudaError_t e;
  const int sd = (int)couple_split_smem_d(t, tc), st = (int)couple_split_smem_t(t, tc);
  if ((e = cudaFuncSetAttribute(k_couple_d<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, sd)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_d<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, sd)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_d<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, sd)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_d<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, sd)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_d<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, sd)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_t, cudaFuncAttributeMaxDynamicSharedMemorySize, st)) != cudaSuccess)
    return e;
  return cudaSuccess;
}

cudaError_t launch_couple_split(const DevTables& t, const TcTables& tc, int n, const float2* cc, const int* sym,
                                float2* Dg, void* Thi, void* Tlo, bool tf32, float* T32, cudaStream_t s) {
  const size_t sd = couple_split_smem_d(t, tc), st = couple_split_smem_t(t, tc);
  for (int p0 = 0; p0 < n; p0 += tc.dsub) {
    const int m = n - p0 < tc.dsub ? n - p0 : tc.dsub;
    dim3 gd(tc.n_units_sym > tc.n_units_gen ? tc.n_units_sym : tc.n_units_gen, m);
#define TP3_D(S) \
  k_couple_d<S><<<gd, kThreadsD, sd, s>>>(cc, t.K, t.nc, tc.coff, tc.pbs, tc.eofs, tc.wtab, tc.units_sym, \
                                          tc.n_units_sym, tc.units_gen, tc.n_units_gen, tc.doff, tc.dstride, sym, Dg, p0)
    if (tc.maxs <= 4) TP3_D(4);
    else if (tc.maxs <= 8) TP3_D(8);
    else if (tc.maxs <= 10) TP3_D(10);
    else if (tc.maxs <= 12) TP3_D(12);
    else TP3_D(16);
#undef TP3_D
    dim3 gt(tc.n_pb, t.K, m);
    k_couple_t<<<gt, kThreadsT, st, s>>>(cc, t.K, t.nc, tc.ncp, tc.coff, tc.pbs, tc.doff, tc.dstride, sym, Dg, p0,
                                         t.klp, tc.KP, Thi, Tlo, tf32, T32, t.n_ltp);
  }
  return cudaGetLastError();
}

}  // namespace tp3
