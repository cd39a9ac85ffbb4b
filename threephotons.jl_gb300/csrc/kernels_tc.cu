// Fast path: pair-factorised coupling (SIMT FP32) -> tcgen05 angular contraction
// with BF16 hi/lo split operands (three MMA passes, FP32 accumulation in TMEM) and
// the Bayes log-likelihood fused into the TMEM epilogue -> FP64 finalize.
//
// Stage (a), coupling.  For one (l1, l2) pair block and one shell k1, all shells
// k2 <= k1 and every m3:
//     D[k2][l3][m3] = sum_m1 w(l1 m1 l2 m2 l3 m3) c_k1[l1,m1] c_k2[l2,m2],  m2 = -m3 - m1
// then for every k3 <= k2
//     T[(k1,k2,k3)][(l1,l2,l3)] = Re sum_m3 D[k2][l3][m3] c_k3[l3,m3]
// which is the reference's As sum (src/correlations.jl:169-172; src/cuda_kernel.cu:31-37)
// regrouped so that each product c_k1 c_k2 is formed once per pair of shells and
// reused by every l3 and every k3.  T is written as a BF16 pair (hi, lo = bf16(T - hi)).
//
// Stage (b)+(c), angular + Bayes.  At lambda = 0 the model correlation on the unique
// grid points u of the symmetry fold is c3[ki][u] = sum_lt T[ki][lt] F[u][lt]
// (F = w Y Y Y cos(m2 alpha + m3 beta) summed per l-triple; the reference's B * PA of
// src/correlations.jl:182 / src/cuda.jl:88 regrouped).  One CTA owns 128 shell triples
// (TMEM lanes) and all unique grid points (TMEM columns, two halves of 256).  Operand
// tiles are staged by TMA (64-byte swizzle) through a 4-deep mbarrier ring; one thread
// issues tcgen05.mma (M=128, N=256, K=16) for hi*hi, hi*lo and lo*hi.  Eight epilogue
// warps read the accumulator with tcgen05.ld, clamp at 1e-30 (src/correlations.jl:203)
// and accumulate Sp = sum p and Sql = sum q~ log p with the folded histogram q~, so
// c3 never reaches global memory.  Every mbarrier wait is bounded; on timeout the
// kernel records TP3_ERR_TIMEOUT in *err, skips the remaining work and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/tp3.h"
#include "internal.h"
#include "tc_prims.cuh"

namespace tp3 {

// ---------------------------------------------------------------------------
// Stage (a): pair-factorised coupling
// ---------------------------------------------------------------------------
namespace {

// T as an operand pair of the split-precision contraction: BF16 hi + bf16(v - hi), or
// TF32 hi (round to nearest, ties away) + the FP32 remainder.
__device__ __forceinline__ void store_split(void* hi, void* lo, size_t i, float v, bool tf32) {
  if (tf32) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    const float hf = __uint_as_float(h);
    reinterpret_cast<float*>(hi)[i] = hf;
    reinterpret_cast<float*>(lo)[i] = v - hf;
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    reinterpret_cast<__nv_bfloat16*>(hi)[i] = h;
    reinterpret_cast<__nv_bfloat16*>(lo)[i] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

__device__ __forceinline__ int ki_index(int k1, int k2, int k3) {
  return k1 * (k1 + 1) * (k1 + 2) / 6 + k2 * (k2 + 1) / 2 + k3;
}

// Coefficients of a real function satisfy c[l,-m] = (-1)^m conj(c[l,m]) (intensities
// are real; the reference's moves rtc * R * ctr with real orthogonal R preserve it).
// grid: n; block 256.  Converts one proposal's FP64 seanindex-ordered coefficients to
// the compact FP32 layout and sets sym[prop] = 1 when every shell satisfies the
// relation to 1e-10 of the shell's largest coefficient; the m < 0 entries are then
// rebuilt from m >= 0 so the relation holds exactly in FP32.
__global__ void __launch_bounds__(256) k_gather_sym(int K, int nc, int ncoef, const int* __restrict__ csean,
                                                    const int* __restrict__ cm, const int* __restrict__ cmir,
                                                    const double2* __restrict__ coeff, float2* __restrict__ cc,
                                                    int* __restrict__ sym, const int* __restrict__ cl,
                                                    const RagInfo* __restrict__ rag, int* __restrict__ err) {
  const int prop = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const double2* cp = coeff + (size_t)prop * K * ncoef;
#ifdef TP3_DEBUG
  {  // the coefficient maps stay inside a shell's coefficients and the compact layout
    int maps_ok = 1;
    for (int c = threadIdx.x; c < nc; c += blockDim.x)
      maps_ok &= csean[c] >= 0 && csean[c] < ncoef && cmir[c] >= 0 && cmir[c] < nc;
    if (!TP3_DCHECK(__syncthreads_and(maps_ok) != 0, err)) K = 0;  // nothing is read or written
  }
#endif
  int ok = 1;
  for (int k = warp; k < K; k += nw) {
    const double2* ck = cp + (size_t)k * ncoef;
    double amax = 0.0;
    for (int c = lane; c < nc; c += 32) {
      const double2 a = ck[csean[c]];
      amax = fmax(amax, fabs(a.x) + fabs(a.y));
    }
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    const double tol = 1e-10 * amax;
    for (int c = lane; c < nc; c += 32) {
      const int m = cm[c];
      if (m < 0) continue;
      const double2 a = ck[csean[c]];
      if (m == 0) {
        ok &= fabs(a.y) <= tol;
      } else {
        const double2 b = ck[csean[cmir[c]]];
        const double sg = (m & 1) ? -1.0 : 1.0;
        ok &= fabs(b.x - sg * a.x) + fabs(b.y + sg * a.y) <= tol;
      }
    }
  }
  const int s = __syncthreads_and(ok);
  float2* out = cc + (size_t)prop * K * nc;
  for (int i = threadIdx.x; i < K * nc; i += blockDim.x) {
    const int k = i / nc, c = i - k * nc;
    const int m = cm[c];
    const double2* ck = cp + (size_t)k * ncoef;
    float2 v;
    if (s && m < 0) {
      const double2 a = ck[csean[cmir[c]]];
      const double sg = (m & 1) ? -1.0 : 1.0;
      v = make_float2((float)(sg * a.x), (float)(-sg * a.y));
    } else {
      const double2 a = ck[csean[c]];
      v = make_float2((float)a.x, (s && m == 0) ? 0.f : (float)a.y);
    }
    if (rag && (cl[c] > rag[prop].L || k >= rag[prop].K)) v = make_float2(0.f, 0.f);  // absent orders / shells
    out[i] = v;
  }
  if (threadIdx.x == 0) sym[prop] = s;
}

// One CTA = one (l1, l2) pair block of one proposal; it loops over chunks of shell
// pairs (k1, k2 <= k1), each chunk a run of whole k1 values.
// Shared memory: coefficients [K][ncp] (ncp odd: conflict-free strided float2 reads),
// the block's 3j table [e][m1][nl3p] (when W_SMEM), and D [pairs in chunk][SDp].
// Phase 1: item = (m3, pair); the lanes of a warp share m3, so they share the m1
//          range and read the 3j values as broadcasts.
// Phase 2: item = (k1, l3, 4 x 4 tile of (k2, k3)) with k3 <= k2.
// grid: (n_pb, n); block kCoupleThreads.
constexpr int kCoupleThreads = 512;
constexpr int kCoupleThreadsSmall = 256;  // the two-CTA-per-SM tilings

template <int MAXS, bool W_SMEM, int THREADS>
__global__ void __launch_bounds__(THREADS, kCoupleThreads / THREADS) k_couple_pair(
    const float2* __restrict__ cc, int K, int nc, int ncp, const int* __restrict__ coff,
    const PairBlock* __restrict__ pbs, const int* __restrict__ eofs, const float* __restrict__ wtab,
    const int2* __restrict__ chunks_gen, int nchunks_gen, int pmax_gen, int SDp,
    const int2* __restrict__ chunks_sym, int nchunks_sym, int pmax_sym, int SDhp, int wsmem, int klp, int KP,
    const int* __restrict__ symflags, void* __restrict__ Thi, void* __restrict__ Tlo, bool tf32out,
    float* __restrict__ T32, int ldT32, const RagInfo* __restrict__ rag) {
  extern __shared__ __align__(16) float smf[];
  const int prop = blockIdx.y;
  int Kp = K;
  if (rag) {
    const RagInfo ri = rag[prop];
    Kp = ri.K;
    const PairBlock pb0 = pbs[blockIdx.x];
    if (pb0.l1 > ri.L || pb0.l2 > ri.L) {
      // absent orders: the block's l-triples are zero for this proposal's scored rows
      for (int i = threadIdx.x; i < ri.klen * pb0.nl3; i += blockDim.x) {
        const int ki = i / pb0.nl3, sj = i - ki * pb0.nl3;
        store_split(Thi, Tlo, ((size_t)prop * klp + ki) * KP + pb0.lt_base + sj, 0.f, tf32out);
        if (T32) T32[((size_t)prop * klp + ki) * ldT32 + pb0.lt_base + sj] = 0.f;
      }
      return;
    }
  }
  // real-function coefficients: only m3 >= 0 of D is formed, D[-m3] = (-1)^m3 conj(D[m3])
  // and T = Re(D[0] c[0]) + 2 sum_{m3 > 0} Re(D[m3] c[m3]); D rows then hold m3 = 0..l3
  // only (row length SDhp instead of SDp), so a chunk holds about twice the shell pairs.
  const bool sym = symflags[prop] != 0;
  const int2* chunks = sym ? chunks_sym : chunks_gen;
  const int nchunks = sym ? nchunks_sym : nchunks_gen;
  const int pmax = sym ? pmax_sym : pmax_gen;
  const int rowD = sym ? SDhp : SDp;
  const PairBlock pb = pbs[blockIdx.x];
  float2* sc = reinterpret_cast<float2*>(smf);                 // [K][ncp]
  float* sw = smf + (2 * (size_t)K * ncp + 3) / 4 * 4;          // [wsmem], 16-byte aligned
  float2* sD = reinterpret_cast<float2*>(sw + (W_SMEM ? wsmem : 0));  // [2][pmax][rowD]
  const float2* src = cc + (size_t)prop * K * nc;
  for (int i = threadIdx.x; i < K * nc; i += blockDim.x) {
    const int k = i / nc, c = i - k * nc;
    sc[k * ncp + c] = src[i];
  }
  const float* wblk = wtab + pb.wofs;
  if (W_SMEM) {
    const float4* w4 = reinterpret_cast<const float4*>(wblk);
    float4* s4 = reinterpret_cast<float4*>(sw);
    for (int i = threadIdx.x; i < pb.wcount / 4; i += blockDim.x) s4[i] = w4[i];
  }
  __syncthreads();
  const float* wsrc = W_SMEM ? sw : wblk;

  const int l1 = pb.l1, l2 = pb.l2, nl3 = pb.nl3, nl3p = pb.nl3p, l3min = pb.l3min, M = pb.M;
  const int off1 = coff[l1 >> 1] + l1, off2 = coff[l2 >> 1] + l2;
  // D is double-buffered: phase 2 of chunk ch and phase 1 of chunk ch+1 need no
  // barrier between them, so one __syncthreads per chunk suffices and uneven items
  // of the two phases overlap across warps.
  int done = 0;  // chunks processed (parity of the D buffer)
  for (int ch = 0; ch < nchunks; ++ch) {
    const int k1hi = chunks[ch].x, k1lo = chunks[ch].y;
    if (k1lo >= Kp) continue;  // shells beyond this proposal's K: rows not scored
    float2* Dbuf = sD + (size_t)(done & 1) * pmax * rowD;
    ++done;
    int npairs = 0;
    for (int k1 = k1hi; k1 >= k1lo; --k1) npairs += k1 + 1;
    // ---- phase 1: longest diagonals (small |m3|) first ----
    const int items1 = npairs * (sym ? M + 1 : 2 * M + 1);
    for (int it = threadIdx.x; it < items1; it += blockDim.x) {
      const int eo = it / npairs, p = it - eo * npairs;
      const int m3 = sym ? eo : ((eo & 1) ? -((eo + 1) >> 1) : (eo >> 1));
      const int e = m3 + M;
      int k1 = k1hi, q = p;
      while (q > k1) { q -= k1 + 1; --k1; }
      const int k2 = q;
      const int m1lo = max(-l1, -l2 - m3), m1hi = min(l1, l2 - m3);
      const float* wp = wsrc + eofs[pb.eofs + e];
      const float2* c1 = sc + k1 * ncp + off1;
      const float2* c2 = sc + k2 * ncp + off2 - m3;
      float ar[MAXS], ai[MAXS];
#pragma unroll
      for (int s = 0; s < MAXS; ++s) { ar[s] = 0.f; ai[s] = 0.f; }
      for (int m1 = m1lo; m1 <= m1hi; ++m1) {
        const float2 a = c1[m1];
        const float2 b = c2[-m1];
        const float xr = a.x * b.x - a.y * b.y;
        const float xi = a.x * b.y + a.y * b.x;
        const float2* wr = reinterpret_cast<const float2*>(wp + (m1 - m1lo) * nl3p);
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
      float2* d = Dbuf + (size_t)p * rowD;
      int dofs = 0;
#pragma unroll
      for (int s = 0; s < MAXS; ++s) {
        if (s < nl3) {
          const int l3 = l3min + 2 * s;
          if (sym) {
            if (m3 <= l3) d[dofs + m3] = make_float2(ar[s], ai[s]);
            dofs += l3 + 1;
          } else {
            if (m3 >= -l3 && m3 <= l3) d[dofs + m3 + l3] = make_float2(ar[s], ai[s]);
            dofs += 2 * l3 + 1;
          }
        }
      }
    }
    __syncthreads();
    // ---- phase 2: largest l3 first ----
    int items2 = 0;
    for (int k1 = k1hi; k1 >= k1lo; --k1) {
      const int nq = (k1 + 4) >> 2;
      items2 += nq * (nq + 1) / 2 * nl3;
    }
    for (int it = threadIdx.x; it < items2; it += blockDim.x) {
      int k1 = k1hi, q = it, pbase = 0;
      for (;;) {
        const int nq = (k1 + 4) >> 2;
        const int cnt = nq * (nq + 1) / 2 * nl3;
        if (q < cnt) break;
        q -= cnt;
        pbase += k1 + 1;
        --k1;
      }
      const int nq = (k1 + 4) >> 2;
      const int tiles = nq * (nq + 1) / 2;
      const int s = nl3 - 1 - q / tiles;
      int t = q % tiles;
      int ra = 0;
      while (t > ra) { t -= ra + 1; ++ra; }
      const int rb = t;  // k2 quad ra, k3 quad rb <= ra
      const int l3 = l3min + 2 * s;
      // row offset of l3: sum_{j<s} (l3_j + 1) (m3 >= 0 rows) or sum_{j<s} (2 l3_j + 1), centred
      const int dofs = sym ? s * (l3min + s) : s * (2 * l3min + 2 * s - 1) + l3min + 2 * s;
      const int off3 = coff[l3 >> 1] + l3;
      const float2* drow[4];
      const float2* crow[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k2 = min(4 * ra + i, k1);
        const int k3 = min(4 * rb + i, k1);
        drow[i] = Dbuf + (size_t)(pbase + k2) * rowD + dofs;
        crow[i] = sc + k3 * ncp + off3;
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
            const int ki = ki_index(k1, k2, k3);
            const float v = acc[i][j];
            store_split(Thi, Tlo, ((size_t)prop * klp + ki) * KP + lt, v, tf32out);
            if (T32) T32[((size_t)prop * klp + ki) * ldT32 + lt] = v;
          }
        }
      }
    }
  }
}


// Warp-local form of the pair coupling (no CTA barrier after the loads).  One CTA =
// one (l1, l2) pair block of one proposal; its warps take work units from a shared
// counter.  A unit is one shell k1 and a quad of k2 (k2 = 4q .. 4q+3, <= k1): the warp
// forms D for those (up to) four shell pairs and every m3 / l3 in its own shared-memory
// buffer (phase 1: lanes own (m3, pair) items, so lanes with one m3 read the same 3j row),
// then contracts D with every k3-quad <= q (phase 2: lanes own (l3, k3-quad) items and
// read the unit's D rows as broadcasts).  Both phases synchronise only the warp.
// grid: (n_pb, n); block kCoupleThreads.
template <int MAXS, bool W_SMEM, int THREADS>
__global__ void __launch_bounds__(THREADS, kCoupleThreads / THREADS) k_couple_warp(
    const float2* __restrict__ cc, int K, int nc, int ncp, const int* __restrict__ coff,
    const PairBlock* __restrict__ pbs, const int* __restrict__ eofs, const float* __restrict__ wtab, int SDp,
    int SDhp, int wsmem, int klp, int KP, const int* __restrict__ symflags, void* __restrict__ Thi,
    void* __restrict__ Tlo, bool tf32out, float* __restrict__ T32, int ldT32, const RagInfo* __restrict__ rag) {
  extern __shared__ __align__(16) float smf[];
  __shared__ int s_next, s_total;
  __shared__ int s_ustart[64];  // first unit index of each k1 (units ordered by k1 descending)
  __shared__ int s_eofs[64];    // the block's per-m3 3j row offsets (2 M + 1 <= 61)
  __shared__ int s_coff[32];    // coefficient offset of each even order
  const int prop = blockIdx.y;
  int Kp = K;
  const PairBlock pb = pbs[blockIdx.x];
  if (rag) {
    const RagInfo ri = rag[prop];
    Kp = ri.K;
    if (pb.l1 > ri.L || pb.l2 > ri.L) {
      for (int i = threadIdx.x; i < ri.klen * pb.nl3; i += blockDim.x) {
        const int ki = i / pb.nl3, sj = i - ki * pb.nl3;
        store_split(Thi, Tlo, ((size_t)prop * klp + ki) * KP + pb.lt_base + sj, 0.f, tf32out);
        if (T32) T32[((size_t)prop * klp + ki) * ldT32 + pb.lt_base + sj] = 0.f;
      }
      return;
    }
  }
  const bool sym = symflags[prop] != 0;
  const int rowD = sym ? SDhp : SDp;
  float2* sc = reinterpret_cast<float2*>(smf);                  // [K][ncp]
  float* sw = smf + (2 * (size_t)K * ncp + 3) / 4 * 4;           // [wsmem]
  float2* sD = reinterpret_cast<float2*>(sw + (W_SMEM ? wsmem : 0));  // [warps][4][rowD]
  const float2* src = cc + (size_t)prop * K * nc;
  for (int i = threadIdx.x; i < Kp * nc; i += blockDim.x) {
    const int k = i / nc, c = i - k * nc;
    sc[k * ncp + c] = src[i];
  }
  const float* wblk = wtab + pb.wofs;
  if (W_SMEM) {
    const float4* w4 = reinterpret_cast<const float4*>(wblk);
    float4* s4 = reinterpret_cast<float4*>(sw);
    for (int i = threadIdx.x; i < pb.wcount / 4; i += blockDim.x) s4[i] = w4[i];
  }
  for (int e = threadIdx.x; e <= 2 * pb.M; e += blockDim.x) s_eofs[e] = eofs[pb.eofs + e];
  // orders used by this block: l1, l2 and l3 <= M (all <= L, so coff has entries up to L / 2)
  for (int e = threadIdx.x; e <= max(max(pb.l1, pb.l2), pb.M) >> 1; e += blockDim.x) s_coff[e] = coff[e];
  if (threadIdx.x == 0) {
    int u = 0;
    for (int k1 = Kp - 1; k1 >= 0; --k1) {
      s_ustart[k1] = u;
      u += (k1 + 4) >> 2;
    }
    s_total = u;
    s_next = 0;
  }
  __syncthreads();
  const float* wsrc = W_SMEM ? sw : wblk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this proposal's T rows (klp x KP elements, within int range per proposal)
  const size_t tbase = (size_t)prop * klp * KP;
  void* ThiP = tf32out ? (void*)((float*)Thi + tbase) : (void*)((__nv_bfloat16*)Thi + tbase);
  void* TloP = tf32out ? (void*)((float*)Tlo + tbase) : (void*)((__nv_bfloat16*)Tlo + tbase);
  float* T32P = T32 ? T32 + (size_t)prop * klp * ldT32 : nullptr;
  float2* Dw = sD + (size_t)warp * 4 * rowD;
  const int l1 = pb.l1, l2 = pb.l2, nl3 = pb.nl3, nl3p = pb.nl3p, l3min = pb.l3min, M = pb.M;
  const int off1 = s_coff[l1 >> 1] + l1, off2 = s_coff[l2 >> 1] + l2;
  const int nm3 = sym ? M + 1 : 2 * M + 1;
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&s_next, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= s_total) break;
    // decode unit u (k1 descending, then q ascending)
    int k1 = Kp - 1;
    while (k1 > 0 && s_ustart[k1 - 1] <= u) --k1;
    const int q = u - s_ustart[k1];
    const int np = min(4, k1 - 4 * q + 1);
    // ---- phase 1: D[i][l3][m3] for the unit's pairs (k1, 4q + i) ----
    const int nI = nm3 * np;
    for (int it = lane; it < nI; it += 32) {
      // it / np for np in 1..4 without a division (exact for it < 2^15)
      const int eo = np == 4 ? it >> 2 : (np == 2 ? it >> 1 : (np == 1 ? it : (it * 43691) >> 17));
      const int i = it - eo * np;
      const int m3 = sym ? eo : ((eo & 1) ? -((eo + 1) >> 1) : (eo >> 1));
      const int e = m3 + M;
      const int k2 = 4 * q + i;
      const int m1lo = max(-l1, -l2 - m3), m1hi = min(l1, l2 - m3);
      const float* wp = wsrc + s_eofs[e];
      const float2* c1 = sc + k1 * ncp + off1;
      const float2* c2 = sc + k2 * ncp + off2 - m3;
      float ar[MAXS], ai[MAXS];
#pragma unroll
      for (int s = 0; s < MAXS; ++s) { ar[s] = 0.f; ai[s] = 0.f; }
#pragma unroll 2
      for (int m1 = m1lo; m1 <= m1hi; ++m1) {
        const float2 a = c1[m1];
        const float2 b = c2[-m1];
        const float xr = a.x * b.x - a.y * b.y;
        const float xi = a.x * b.y + a.y * b.x;
        const float2* wr = reinterpret_cast<const float2*>(wp + (m1 - m1lo) * nl3p);
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
      float2* d = Dw + (size_t)i * rowD;
      int dofs = 0;
#pragma unroll
      for (int s = 0; s < MAXS; ++s) {
        if (s < nl3) {
          const int l3 = l3min + 2 * s;
          if (sym) {
            if (m3 <= l3) d[dofs + m3] = make_float2(ar[s], ai[s]);
            dofs += l3 + 1;
          } else {
            if (m3 >= -l3 && m3 <= l3) d[dofs + m3 + l3] = make_float2(ar[s], ai[s]);
            dofs += 2 * l3 + 1;
          }
        }
      }
    }
    __syncwarp();
    // ---- phase 2: T for (k1, k2 in the quad, k3-quad rb <= q, l3) ----
    // A unit has only nl3 (q + 1) items; when they fill less than the warp, g = 2 or 4
    // lanes share an item, each summing every g-th m3, and combine by shuffles.
    const int nI2 = nl3 * (q + 1);
    int lg = 0;
    while (lg < 2 && (nI2 << (lg + 1)) <= 32) ++lg;
    const int g = 1 << lg, nI2g = nI2 << lg;
    // it / (q + 1) as a multiply-shift: exact for it < 2^16 / (q + 1) (it < 16 * 16 here)
    const int d1 = q + 1, rcp = (65536 + d1 - 1) / d1;
    const int t3 = k1 * (k1 + 1) * (k1 + 2) / 6;  // first shell triple of k1
    for (int base = 0; base < nI2g; base += 32) {
      const int itl = base + lane;
      const bool active = itl < nI2g;
      const int it = active ? itl >> lg : 0, seg = itl & (g - 1);
      const int sq = (it * rcp) >> 16;
      const int s = nl3 - 1 - sq;  // largest l3 first
      const int rb = it - sq * d1;
      const int l3 = l3min + 2 * s;
      const int dofs = sym ? s * (l3min + s) : s * (2 * l3min + 2 * s - 1) + l3min + 2 * s;
      const int off3 = s_coff[l3 >> 1] + l3;
      const float2* drow[4];
      const float2* crow[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        drow[i] = Dw + (size_t)min(i, np - 1) * rowD + dofs;
        crow[i] = sc + min(4 * rb + i, k1) * ncp + off3;
      }
      float acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
      if (active) {
#pragma unroll 2
        for (int m3 = (sym ? 1 : -l3) + seg; m3 <= l3; m3 += g) {
          float2 x[4], y[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) { x[i] = drow[i][m3]; y[i] = crow[i][m3]; }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(x[i].x, y[j].x, fmaf(-x[i].y, y[j].y, acc[i][j]));
        }
      }
      for (int o = 1; o < g; o <<= 1)
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] += __shfl_xor_sync(0xffffffffu, acc[i][j], o);
      if (!active || seg != 0) continue;
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
        const int k2 = 4 * q + i;
        if (k2 > k1) continue;
        const int row0 = t3 + k2 * (k2 + 1) / 2 + 4 * rb;  // shell triple (k1, k2, 4 rb)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (4 * rb + j <= k2) {
            const int ki = row0 + j;
            const float v = acc[i][j];
            store_split(ThiP, TloP, (size_t)(ki * KP + lt), v, tf32out);
            if (T32P) T32P[ki * ldT32 + lt] = v;
          }
        }
      }
    }
    __syncwarp();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Stage (b)+(c): tcgen05 angular contraction + fused Bayes epilogue
// ---------------------------------------------------------------------------
namespace {

constexpr int kStages = 4;
constexpr int kBK = 32;                       // K elements per stage: 64 bytes of bf16 (16 of tf32)
constexpr int kBM = 128;                      // shell triples per CTA (TMEM lanes)
constexpr int kBN = 256;                      // grid columns per MMA (one TMEM half)
constexpr int kABytes = kBM * kBK * 2;        // 8 KB
constexpr int kBBytes = kBN * kBK * 2;        // 16 KB
constexpr int kStageBytes = 2 * kABytes + 2 * kBBytes;  // 48 KB
constexpr int kEpiWarps = 8;
constexpr int kThreads = 64 + 32 * kEpiWarps;  // producer warp, MMA warp, 8 epilogue warps
// Instruction descriptor: F32 accumulator, both operands K-major, M = 128, N = 256;
// operand format 1 = BF16 (kind::f16), 2 = TF32 (kind::tf32).
__host__ __device__ constexpr uint32_t idesc_m128_n256(uint32_t fmt) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(kBN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

struct TcSmemHeader {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t tmem_full[2];
  uint32_t tmem_base;
  int abort_flag;
  float part_sp[2][kBM];
  float part_sq[2][kBM];
};

// grid: (klp / 128, n); block kThreads; dyn smem = 1 KB alignment slack + stages + header.
// STORE: write c3 (all four images of every unique point) instead of the Bayes terms.
// AMN (BF16 only): T is order-major, [prop][lt][ki]; each stage's A tile arrives as two
// 64-shell-triple boxes (128-byte swizzle) and is read as an MN-major operand.
template <bool STORE, bool TF32, bool AMN>
__global__ void __launch_bounds__(kThreads, 1) k_angular_tc(
    const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
    const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo, int klp, int KP,
    int Gu, int nhalf, int klength, const float* __restrict__ qt, const double* __restrict__ Qs,
    const double* __restrict__ tf, int mult, double* __restrict__ Eslab, float* __restrict__ c3out,
    const int* __restrict__ u_to_g, int N, int* __restrict__ err, const RagInfo* __restrict__ rag) {
  extern __shared__ uint8_t smem_raw[];
  if (rag) {
    // ragged batch: tiles past the proposal's scored shell triples do no work, and
    // the Bayes terms read the proposal's own histogram
    const RagInfo ri = rag[blockIdx.y];
    if ((int)blockIdx.x * kBM >= ri.klen) return;
    qt += (size_t)ri.hist * klp * Gu;
    Qs += (size_t)ri.hist * klength;
  }
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* stages = base;
  TcSmemHeader* hd = (TcSmemHeader*)(base + kStages * kStageBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int prop = blockIdx.y;
  const int mtile = blockIdx.x;
  const int row0 = prop * klp + mtile * kBM;  // row coordinate in the A tensor
  constexpr int kbk = TF32 ? kBK / 2 : kBK;  // K elements in one 64-byte row
  const int nk = KP / kbk;
  const uint32_t tcols = nhalf == 2 ? 512u : 256u;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&hd->full[s], 1);
      mbar_init(&hd->empty[s], 1);
    }
    mbar_init(&hd->tmem_full[0], 1);
    mbar_init(&hd->tmem_full[1], 1);
    hd->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&hd->tmem_base)),
                 "r"(tcols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = hd->tmem_base;
  volatile int* abort_flag = &hd->abort_flag;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0;
      int last[kStages];
#pragma unroll
      for (int s = 0; s < kStages; ++s) last[s] = -1;
      for (int h = 0; h < nhalf && !*abort_flag; ++h) {
        for (int kc = 0; kc < nk; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (uint32_t)((it / kStages) & 1);
          if (!mbar_wait(&hd->empty[s], ph ^ 1u, abort_flag, err)) break;
          last[s] = it;
          uint8_t* st = stages + s * kStageBytes;
          mbar_expect_tx(&hd->full[s], kStageBytes);
          if (AMN) {
            const int y = prop * KP + kc * kbk;  // order row of T[lt][ki]
#pragma unroll
            for (int g = 0; g < 2; ++g) {
              tma_load_2d(st + g * (kABytes / 2), &tmA_hi, &hd->full[s], mtile * kBM + g * 64, y);
              tma_load_2d(st + kABytes + g * (kABytes / 2), &tmA_lo, &hd->full[s], mtile * kBM + g * 64, y);
            }
          } else {
            tma_load_2d(st, &tmA_hi, &hd->full[s], kc * kbk, row0);
            tma_load_2d(st + kABytes, &tmA_lo, &hd->full[s], kc * kbk, row0);
          }
          tma_load_2d(st + 2 * kABytes, &tmB_hi, &hd->full[s], kc * kbk, h * kBN);
          tma_load_2d(st + 2 * kABytes + kBBytes, &tmB_lo, &hd->full[s], kc * kbk, h * kBN);
        }
      }
      if (*abort_flag) {
        // let this CTA's copies in flight land before its shared memory is released
        for (int s = 0; s < kStages; ++s) {
          if (last[s] < 0) continue;
          const long long t0 = clock64();
          while (!mbar_try_wait(&hd->full[s], (uint32_t)((last[s] / kStages) & 1)) &&
                 clock64() - t0 < kTimeoutCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_m128_n256(TF32 ? 2u : 1u) | (AMN ? (1u << 15) : 0u);  // bit 15: A MN-major
      int it = 0;
      for (int h = 0; h < nhalf && !*abort_flag; ++h) {
        const uint32_t dt = tmem + (uint32_t)(h * kBN);
        for (int kc = 0; kc < nk; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (uint32_t)((it / kStages) & 1);
          if (!mbar_wait(&hd->full[s], ph, abort_flag, err)) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(stages + s * kStageBytes);
          const uint64_t ahi = AMN ? smem_desc_mn_sw128(st, kABytes / 2) : smem_desc_sw64(st);
          const uint64_t alo = AMN ? smem_desc_mn_sw128(st + kABytes, kABytes / 2) : smem_desc_sw64(st + kABytes);
          const uint64_t bhi = smem_desc_sw64(st + 2 * kABytes), blo = smem_desc_sw64(st + 2 * kABytes + kBBytes);
          // two MMA K-steps per stage (K = 16 bf16 or K = 8 tf32 each): 32 bytes along a
          // K-major row, or 16 rows of 128 bytes (2 KB) of an MN-major tile
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint64_t dk = (uint64_t)(ks * 2);  // +32 bytes, in 16-byte descriptor units
            const uint64_t da = AMN ? (uint64_t)(ks * 128) : dk;  // +2048 bytes for MN-major A
            mma_issue<TF32>(dt, ahi + da, bhi + dk, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
            mma_issue<TF32>(dt, ahi + da, blo + dk, idesc, 1u);
            mma_issue<TF32>(dt, alo + da, bhi + dk, idesc, 1u);
          }
          mma_commit(&hd->empty[s]);
        }
        mma_commit(&hd->tmem_full[h]);
      }
    }
  } else {
    // ---------------- epilogue: 8 warps ----------------
    const int ew = warp - 2;
    const int quarter = warp & 3;           // TMEM lane quarter this warp may access
    const int cblk = ew >> 2;               // which 128-column block of each half
    const int r = quarter * 32 + lane;      // row inside the tile
    const int ki = mtile * kBM + r;
    // compensated (Kahan) sums: Sp and Sql are differences of large, nearly equal
    // energies once combined, so their rounding sets the precision of dE
    float sp = 0.f, sq = 0.f, csp = 0.f, csq = 0.f;
    for (int h = 0; h < nhalf; ++h) {
      if (!mbar_wait(&hd->tmem_full[h], 0u, abort_flag, err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int cc = 0; cc < 4; ++cc) {
        const int col = h * kBN + cblk * 128 + cc * 32;
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)col, v);
        if (STORE) {
          if (ki < klength) {
            float* o = c3out + ((size_t)prop * klength + ki) * (size_t)(2 * N * N);
#pragma unroll 4
            for (int j = 0; j < 32; ++j) {
              const int u = col + j;
              if (u < Gu) {
                const int g = u_to_g[u];
                const int a = g % N, b = g / N;
                o[g] = v[j];
                if (mult == 4) {
                  o[a + N * (b + N)] = v[j];
                  o[(N - 1 - a) + N * (N - 1 - b)] = v[j];
                  o[(N - 1 - a) + N * (2 * N - 1 - b)] = v[j];
                }
              }
            }
          }
        } else {
          const float* qrow = qt + ((size_t)mtile * Gu) * kBM + r;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int u = col + j;
            if (u < Gu) {
              const float p = fmaxf(v[j], 1e-30f);
              const float y1 = p - csp;
              const float t1 = sp + y1;
              csp = (t1 - sp) - y1;
              sp = t1;
              const float y2 = qrow[(size_t)u * kBM] * __logf(p) - csq;
              const float t2 = sq + y2;
              csq = (t2 - sq) - y2;
              sq = t2;
            }
          }
        }
      }
    }
    if (!STORE) {
      hd->part_sp[cblk][r] = sp - csp;
      hd->part_sq[cblk][r] = sq - csq;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (!STORE && warp >= 2 && warp < 6) {
    const int r = (warp & 3) * 32 + lane;
    const int ki = mtile * kBM + r;
    if (ki < klength && !*abort_flag) {
      const double Sp = (double)hd->part_sp[0][r] + (double)hd->part_sp[1][r];
      const double Sq = (double)hd->part_sq[0][r] + (double)hd->part_sq[1][r];
      Eslab[(size_t)prop * klength + ki] = tf[ki] * (Qs[ki] * log((double)mult * Sp) - Sq);
    }
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols) : "memory");
  }
}

// Persistent schedule of the same contraction (Bayes terms only).  A unit is one
// (proposal, 128-shell-triple tile, 256-column half of the grid), half fastest; CTA c
// takes units c, c + gridDim.x, ...  TMEM holds two 256-column accumulators: the i-th
// unit of a CTA accumulates into buffer i & 1, so the epilogue warps drain one unit
// while the MMA warp fills the other.  tmem_full[b] (one arrival, tcgen05.commit) hands
// a buffer to the epilogue; tmem_empty[b] (one arrival per epilogue warp) hands it back.
// The epilogue writes compensated partial sums per (row, half, column block) to
// part [prop][klp][nhalf halves][2 blocks][Sp, Sql]; k_finalize_parts forms the slab
// terms.  STORE: the epilogue writes c3 instead (all images of every unique point).
// Any number of halves (the unfolded 2N^2-point grid of lambda != 0 has 8 at N = 32).
template <bool STORE, bool TF32, bool AMN>
__global__ void __launch_bounds__(kThreads, 1) k_angular_tp(
    const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
    const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo, int klp, int KP,
    int Gu, int nhalf, int nunits, const float* __restrict__ qt, float* __restrict__ part, int* __restrict__ err,
    const RagInfo* __restrict__ rag, int klength, float* __restrict__ c3out, const int* __restrict__ u_to_g, int N,
    int mult) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t tmem_empty[2];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* stages = base;
  TcSmemHeader* hd = (TcSmemHeader*)(base + kStages * kStageBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nmt = klp / kBM;
  constexpr int kbk = TF32 ? kBK / 2 : kBK;
  const int nk = KP / kbk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&hd->full[s], 1);
      mbar_init(&hd->empty[s], 1);
    }
    mbar_init(&hd->tmem_full[0], 1);
    mbar_init(&hd->tmem_full[1], 1);
    mbar_init(&tmem_empty[0], kEpiWarps);
    mbar_init(&tmem_empty[1], kEpiWarps);
    hd->abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&hd->tmem_base)),
                 "r"(512u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = hd->tmem_base;
  volatile int* abort_flag = &hd->abort_flag;

  // unit -> (prop, mtile, h); false for tiles past a ragged proposal's scored triples
  auto decode = [&](int u, int& prop, int& mtile, int& h) -> bool {
    h = u % nhalf;
    const int tile = u / nhalf;
    mtile = tile % nmt;
    prop = tile / nmt;
    return !rag || mtile * kBM < rag[prop].klen;
  };

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0;
      int last[kStages];
#pragma unroll
      for (int s = 0; s < kStages; ++s) last[s] = -1;
      for (int u = blockIdx.x; u < nunits && !*abort_flag; u += gridDim.x) {
        int prop, mtile, h;
        if (!decode(u, prop, mtile, h)) continue;
        const int row0 = prop * klp + mtile * kBM;
        for (int kc = 0; kc < nk; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (uint32_t)((it / kStages) & 1);
          if (!mbar_wait(&hd->empty[s], ph ^ 1u, abort_flag, err)) break;
          last[s] = it;
          uint8_t* st = stages + s * kStageBytes;
          mbar_expect_tx(&hd->full[s], kStageBytes);
          if (AMN) {
            const int y = prop * KP + kc * kbk;
#pragma unroll
            for (int g = 0; g < 2; ++g) {
              tma_load_2d(st + g * (kABytes / 2), &tmA_hi, &hd->full[s], mtile * kBM + g * 64, y);
              tma_load_2d(st + kABytes + g * (kABytes / 2), &tmA_lo, &hd->full[s], mtile * kBM + g * 64, y);
            }
          } else {
            tma_load_2d(st, &tmA_hi, &hd->full[s], kc * kbk, row0);
            tma_load_2d(st + kABytes, &tmA_lo, &hd->full[s], kc * kbk, row0);
          }
          tma_load_2d(st + 2 * kABytes, &tmB_hi, &hd->full[s], kc * kbk, h * kBN);
          tma_load_2d(st + 2 * kABytes + kBBytes, &tmB_lo, &hd->full[s], kc * kbk, h * kBN);
        }
      }
      if (*abort_flag) {
        for (int s = 0; s < kStages; ++s) {
          if (last[s] < 0) continue;
          const long long t0 = clock64();
          while (!mbar_try_wait(&hd->full[s], (uint32_t)((last[s] / kStages) & 1)) &&
                 clock64() - t0 < kTimeoutCycles) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_m128_n256(TF32 ? 2u : 1u) | (AMN ? (1u << 15) : 0u);
      int it = 0, i = 0;
      for (int u = blockIdx.x; u < nunits && !*abort_flag; u += gridDim.x) {
        int prop, mtile, h;
        if (!decode(u, prop, mtile, h)) continue;
        const int b = i & 1;
        // the buffer's previous unit (i - 2) must have been read out by the epilogue
        if (!mbar_wait(&tmem_empty[b], (uint32_t)(((i >> 1) & 1) ^ 1), abort_flag, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dt = tmem + (uint32_t)(b * kBN);
        bool ok = true;
        for (int kc = 0; kc < nk; ++kc, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (uint32_t)((it / kStages) & 1);
          if (!mbar_wait(&hd->full[s], ph, abort_flag, err)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(stages + s * kStageBytes);
          const uint64_t ahi = AMN ? smem_desc_mn_sw128(st, kABytes / 2) : smem_desc_sw64(st);
          const uint64_t alo = AMN ? smem_desc_mn_sw128(st + kABytes, kABytes / 2) : smem_desc_sw64(st + kABytes);
          const uint64_t bhi = smem_desc_sw64(st + 2 * kABytes), blo = smem_desc_sw64(st + 2 * kABytes + kBBytes);
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint64_t dk = (uint64_t)(ks * 2);
            const uint64_t da = AMN ? (uint64_t)(ks * 128) : dk;
            mma_issue<TF32>(dt, ahi + da, bhi + dk, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
            mma_issue<TF32>(dt, ahi + da, blo + dk, idesc, 1u);
            mma_issue<TF32>(dt, alo + da, bhi + dk, idesc, 1u);
          }
          mma_commit(&hd->empty[s]);
        }
        if (!ok) break;
        mma_commit(&hd->tmem_full[b]);
        ++i;
      }
    }
  } else {
    // ---------------- epilogue: 8 warps ----------------
    const int ew = warp - 2;
    const int quarter = warp & 3;
    const int cblk = ew >> 2;
    const int r = quarter * 32 + lane;
    int i = 0;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
      int prop, mtile, h;
      if (!decode(u, prop, mtile, h)) continue;
      const int b = i & 1;
      if (!mbar_wait(&hd->tmem_full[b], (uint32_t)((i >> 1) & 1), abort_flag, err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const float* qrow =
          STORE ? nullptr : qt + (rag ? (size_t)rag[prop].hist * klp * Gu : 0) + ((size_t)mtile * Gu) * kBM + r;
      const int ki = mtile * kBM + r;
      float sp = 0.f, sq = 0.f, csp = 0.f, csq = 0.f;
      for (int cc = 0; cc < 4; ++cc) {
        const int col = cblk * 128 + cc * 32;  // column inside the half
        const int u0 = h * kBN + col;          // unique grid point of column 0
        float v[32];
        if (STORE) {
          tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * kBN + col), v);
          if (ki < klength) {
            float* o = c3out + ((size_t)prop * klength + ki) * (size_t)(2 * N * N);
#pragma unroll 4
            for (int j = 0; j < 32; ++j) {
              const int u = u0 + j;
              if (u < Gu) {
                const int g = u_to_g[u];
                const int a = g % N, bb = g / N;
                o[g] = v[j];
                if (mult == 4) {
                  o[a + N * (bb + N)] = v[j];
                  o[(N - 1 - a) + N * (N - 1 - bb)] = v[j];
                  o[(N - 1 - a) + N * (2 * N - 1 - bb)] = v[j];
                }
              }
            }
          }
          continue;
        }
        float q[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) q[j] = u0 + j < Gu ? qrow[(size_t)(u0 + j) * kBM] : 0.f;
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * kBN + col), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          if (u0 + j < Gu) {
            const float p = fmaxf(v[j], 1e-30f);
            const float y1 = p - csp;
            const float t1 = sp + y1;
            csp = (t1 - sp) - y1;
            sp = t1;
            const float y2 = q[j] * __logf(p) - csq;
            const float t2 = sq + y2;
            csq = (t2 - sq) - y2;
            sq = t2;
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tmem_empty[b])) : "memory");
      if (!STORE)
        reinterpret_cast<float2*>(part)[(((size_t)prop * klp + ki) * nhalf + h) * 2 + cblk] =
            make_float2(sp - csp, sq - csq);
      ++i;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
  }
}

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// grid: n; block 256.  Deterministic compensated sum of per-slab energies (the first
// rag[prop].klen slabs of a ragged batch).
__global__ void __launch_bounds__(256) k_finalize_slabs(const double* __restrict__ Eslab, int klength,
                                                        double* __restrict__ E, const RagInfo* __restrict__ rag) {
  __shared__ double ss[256], sc[256];
  const int prop = blockIdx.x;
  const double* e = Eslab + (size_t)prop * klength;
  const int nk = rag ? rag[prop].klen : klength;
  double s = 0.0, c = 0.0;
  for (int ki = threadIdx.x; ki < nk; ki += blockDim.x) {
    double t, err;
    two_sum(s, e[ki], t, err);
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

// grid: (ceil(klength / 256), n); block 256.  Slab terms tf (Qs log(mult Sp) - Sql) in
// FP64 from the persistent kernel's partial sums [klp][nhalf][2][2] per proposal, one
// thread per shell triple; k_finalize_slabs then adds them in its fixed order.
__global__ void __launch_bounds__(256) k_slab_terms(const float* __restrict__ part, int klp, int klength, int nhalf,
                                                    const double* __restrict__ Qs, const double* __restrict__ tf,
                                                    int mult, double* __restrict__ Eslab,
                                                    const RagInfo* __restrict__ rag) {
  const int prop = blockIdx.y;
  const int ki = blockIdx.x * blockDim.x + threadIdx.x;
  int nk = klength;
  if (rag) {
    nk = rag[prop].klen;
    Qs += (size_t)rag[prop].hist * klength;
  }
  if (ki >= nk) return;
  const float4* p4 = reinterpret_cast<const float4*>(part) + ((size_t)prop * klp + ki) * nhalf;
  double Sp = 0.0, Sq = 0.0;
  for (int h = 0; h < nhalf; ++h) {
    const float4 a = p4[h];  // (Sp, Sql) of column blocks 0 and 1
    Sp += (double)a.x + (double)a.z;
    Sq += (double)a.y + (double)a.w;
  }
  Eslab[(size_t)prop * klength + ki] = tf[ki] * (Qs[ki] * log((double)mult * Sp) - Sq);
}

}  // namespace

size_t tc_smem_bytes() { return 1024 + (size_t)kStages * kStageBytes + sizeof(TcSmemHeader); }

cudaError_t tc_configure() {
  cudaError_t e;
  const int smem = (int)tc_smem_bytes();
  const cudaFuncAttribute ds = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if ((e = cudaFuncSetAttribute(k_angular_tc<false, false, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tc<true, false, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tc<false, true, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tc<true, true, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tc<false, false, true>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tc<true, false, true>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tp<false, false, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tp<false, true, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tp<false, false, true>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tp<true, false, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tp<true, true, false>, ds, smem)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_angular_tp<true, false, true>, ds, smem)) != cudaSuccess)
    return e;
  const int cs = kCoupleMaxDynSmem, css = kCoupleSmallSmem;
#define TP3_CP_ATTR(S, W)                                                                                    \
  if ((e = cudaFuncSetAttribute(k_couple_pair<S, W, kCoupleThreads>,                                         \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, cs)) != cudaSuccess ||          \
      (e = cudaFuncSetAttribute(k_couple_pair<S, W, kCoupleThreads / 2>,                                     \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, css)) != cudaSuccess)           \
    return e;
  TP3_CP_ATTR(4, true) TP3_CP_ATTR(8, true) TP3_CP_ATTR(10, true) TP3_CP_ATTR(12, true) TP3_CP_ATTR(16, true)
  TP3_CP_ATTR(4, false) TP3_CP_ATTR(8, false) TP3_CP_ATTR(10, false) TP3_CP_ATTR(12, false)
  TP3_CP_ATTR(16, false)
#undef TP3_CP_ATTR
#define TP3_CW_ATTR(S, W)                                                                                    \
  if ((e = cudaFuncSetAttribute(k_couple_warp<S, W, kCoupleThreads>,                                         \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, cs)) != cudaSuccess ||          \
      (e = cudaFuncSetAttribute(k_couple_warp<S, W, kCoupleThreadsSmall>,                                    \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, cs)) != cudaSuccess)            \
    return e;
  TP3_CW_ATTR(4, true) TP3_CW_ATTR(8, true) TP3_CW_ATTR(10, true) TP3_CW_ATTR(12, true) TP3_CW_ATTR(16, true)
  TP3_CW_ATTR(4, false) TP3_CW_ATTR(8, false) TP3_CW_ATTR(10, false) TP3_CW_ATTR(12, false)
  TP3_CW_ATTR(16, false)
#undef TP3_CW_ATTR
  return cudaSuccess;
}

cudaError_t launch_gather_sym(const DevTables& t, const TcTables& tc, int n, const double2* coeff, CoeffLayout lay,
                              float2* cc, int* sym, cudaStream_t s, const RagInfo* rag) {
  k_gather_sym<<<n, 256, 0, s>>>(t.K, t.nc, lay.stride, lay.map, tc.cm, tc.cmir, coeff, cc, sym, tc.cl, rag, tc.err);
  return cudaGetLastError();
}

cudaError_t launch_couple_pair(const DevTables& t, const TcTables& tc, int n, const float2* cc, const int* sym,
                               void* Thi, void* Tlo, bool tf32, float* T32, cudaStream_t s, const RagInfo* rag) {
  if (tc.use_fold >= 0 && tc.fold[tc.use_fold].ok)
    return launch_couple_fold(t, tc, tc.fold[tc.use_fold], n, cc, sym, Thi, Tlo, tf32, T32, s, rag);
  dim3 grid(tc.n_pb, n);
  const bool w2 = tc.use_warp2 && tc.warp2_ok;
  if ((tc.use_warp && tc.warp_ok) || w2) {
    const size_t smw = w2 ? tc.couple_smem_w2 : tc.couple_smem_w;
    const bool wsw = w2 ? tc.w_smem_w2 : tc.w_smem_w;
#define TP3_CW_LAUNCH(S, W)                                                                                       \
  if (w2)                                                                                                         \
    k_couple_warp<S, W, kCoupleThreadsSmall><<<grid, kCoupleThreadsSmall, smw, s>>>(                              \
        cc, t.K, t.nc, tc.ncp, tc.coff, tc.pbs, tc.eofs, tc.wtab, tc.SDp, tc.SDhp, tc.wsmem, t.klp, tc.KP, sym, Thi, \
        Tlo, tf32, T32, t.n_ltp, rag);                                                                            \
  else                                                                                                            \
    k_couple_warp<S, W, kCoupleThreads><<<grid, kCoupleThreads, smw, s>>>(                                        \
        cc, t.K, t.nc, tc.ncp, tc.coff, tc.pbs, tc.eofs, tc.wtab, tc.SDp, tc.SDhp, tc.wsmem, t.klp, tc.KP, sym, Thi, \
        Tlo, tf32, T32, t.n_ltp, rag)
    if (wsw) {
      if (tc.maxs <= 4) TP3_CW_LAUNCH(4, true);
      else if (tc.maxs <= 8) TP3_CW_LAUNCH(8, true);
      else if (tc.maxs <= 10) TP3_CW_LAUNCH(10, true);
      else if (tc.maxs <= 12) TP3_CW_LAUNCH(12, true);
      else TP3_CW_LAUNCH(16, true);
    } else {
      if (tc.maxs <= 4) TP3_CW_LAUNCH(4, false);
      else if (tc.maxs <= 8) TP3_CW_LAUNCH(8, false);
      else if (tc.maxs <= 10) TP3_CW_LAUNCH(10, false);
      else if (tc.maxs <= 12) TP3_CW_LAUNCH(12, false);
      else TP3_CW_LAUNCH(16, false);
    }
#undef TP3_CW_LAUNCH
    return cudaGetLastError();
  }
  const bool sm = tc.use_small && tc.small_ok;
  const size_t smem = sm ? tc.couple_smem_s : tc.couple_smem;
  const bool wsm = sm ? tc.w_smem_s : tc.w_smem;
  const int2* ch = sm ? tc.chunks_s : tc.chunks;
  const int2* chs = sm ? tc.chunks_sym_s : tc.chunks_sym;
  const int nch = sm ? tc.nchunks_s : tc.nchunks, nchs = sm ? tc.nchunks_sym_s : tc.nchunks_sym;
  const int pm = sm ? tc.pmax_s : tc.pmax, pms = sm ? tc.pmax_sym_s : tc.pmax_sym;
#define TP3_CP_LAUNCH(S, W, TH)                                                                            \
  k_couple_pair<S, W, TH><<<grid, TH, smem, s>>>(                                                          \
      cc, t.K, t.nc, tc.ncp, tc.coff, tc.pbs, tc.eofs, tc.wtab, ch, nch, pm, tc.SDp, chs, nchs, pms, tc.SDhp, \
      tc.wsmem, t.klp, tc.KP, sym, Thi, Tlo, tf32, T32, t.n_ltp, rag)
#define TP3_CP_PICK(TH)                                        \
  if (wsm) {                                                   \
    if (tc.maxs <= 4) TP3_CP_LAUNCH(4, true, TH);              \
    else if (tc.maxs <= 8) TP3_CP_LAUNCH(8, true, TH);         \
    else if (tc.maxs <= 10) TP3_CP_LAUNCH(10, true, TH);       \
    else if (tc.maxs <= 12) TP3_CP_LAUNCH(12, true, TH);       \
    else TP3_CP_LAUNCH(16, true, TH);                          \
  } else {                                                     \
    if (tc.maxs <= 4) TP3_CP_LAUNCH(4, false, TH);             \
    else if (tc.maxs <= 8) TP3_CP_LAUNCH(8, false, TH);        \
    else if (tc.maxs <= 10) TP3_CP_LAUNCH(10, false, TH);      \
    else if (tc.maxs <= 12) TP3_CP_LAUNCH(12, false, TH);      \
    else TP3_CP_LAUNCH(16, false, TH);                         \
  }
  if (sm) {
    TP3_CP_PICK(kCoupleThreads / 2)
  } else {
    TP3_CP_PICK(kCoupleThreads)
  }
#undef TP3_CP_PICK
#undef TP3_CP_LAUNCH
  return cudaGetLastError();
}

cudaError_t launch_angular_tc(const DevTables& t, const TcTables& tc, const TcMaps& maps, int n, const float* qt,
                              const double* Qs, double* Eslab, float* c3out, int* err, bool tf32, cudaStream_t s,
                              const RagInfo* rag) {
  // more than two grid halves do not fit one CTA's TMEM: the persistent kernel walks them
  if (tc.nhalf > 2)
    return c3out ? launch_angular_persistent(t, tc, maps, n, qt, nullptr, err, tf32, s, rag, c3out)
                 : cudaErrorInvalidValue;
  dim3 grid(t.klp / kBM, n);
  const size_t smem = tc_smem_bytes();
  const bool amn = t_order_major(tc, tf32);
#define TP3_ANG(ST, TF, MN, AH, AL)                                                                            \
  k_angular_tc<ST, TF, MN><<<grid, kThreads, smem, s>>>(AH, AL, maps.b_hi, maps.b_lo, t.klp, tc.KP, t.Gu,        \
                                                         tc.nhalf, t.klength, qt, Qs, t.tf, t.mult, Eslab, c3out, \
                                                         t.u_to_g, t.N, err, rag)
  if (c3out) {
    if (tf32) TP3_ANG(true, true, false, maps.a_hi, maps.a_lo);
    else if (amn) TP3_ANG(true, false, true, maps.a_hi_mn, maps.a_lo_mn);
    else TP3_ANG(true, false, false, maps.a_hi, maps.a_lo);
  } else {
    if (tf32) TP3_ANG(false, true, false, maps.a_hi, maps.a_lo);
    else if (amn) TP3_ANG(false, false, true, maps.a_hi_mn, maps.a_lo_mn);
    else TP3_ANG(false, false, false, maps.a_hi, maps.a_lo);
  }
#undef TP3_ANG
  return cudaGetLastError();
}

cudaError_t launch_finalize_slabs(int n, int klength, const double* Eslab, double* E, cudaStream_t s,
                                  const RagInfo* rag) {
  k_finalize_slabs<<<n, 256, 0, s>>>(Eslab, klength, E, rag);
  return cudaGetLastError();
}

cudaError_t launch_angular_persistent(const DevTables& t, const TcTables& tc, const TcMaps& maps, int n,
                                      const float* qt, float* part, int* err, bool tf32, cudaStream_t s,
                                      const RagInfo* rag, float* c3out) {
  const int nunits = n * (t.klp / kBM) * tc.nhalf;
  const int ctas = std::max(1, std::min(nunits, tc.nsm));
  const size_t smem = tc_smem_bytes();
  const bool amn = t_order_major(tc, tf32);
#define TP3_ANGP(ST, TF, MN, AH, AL)                                                                          \
  k_angular_tp<ST, TF, MN><<<ctas, kThreads, smem, s>>>(AH, AL, maps.b_hi, maps.b_lo, t.klp, tc.KP, t.Gu, tc.nhalf, \
                                                        nunits, qt, part, err, rag, t.klength, c3out, t.u_to_g, t.N,  \
                                                        t.mult)
  if (c3out) {
    if (tf32) TP3_ANGP(true, true, false, maps.a_hi, maps.a_lo);
    else if (amn) TP3_ANGP(true, false, true, maps.a_hi_mn, maps.a_lo_mn);
    else TP3_ANGP(true, false, false, maps.a_hi, maps.a_lo);
  } else {
    if (tf32) TP3_ANGP(false, true, false, maps.a_hi, maps.a_lo);
    else if (amn) TP3_ANGP(false, false, true, maps.a_hi_mn, maps.a_lo_mn);
    else TP3_ANGP(false, false, false, maps.a_hi, maps.a_lo);
  }
#undef TP3_ANGP
  return cudaGetLastError();
}

cudaError_t launch_finalize_parts(const DevTables& t, const TcTables& tc, int n, const float* part, const double* Qs,
                                  double* Eslab, double* E, cudaStream_t s, const RagInfo* rag) {
  k_slab_terms<<<dim3((t.klength + 255) / 256, n), 256, 0, s>>>(part, t.klp, t.klength, tc.nhalf, Qs, t.tf, t.mult,
                                                                 Eslab, rag);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_finalize_slabs<<<n, 256, 0, s>>>(Eslab, t.klength, E, rag);
  return cudaGetLastError();
}

}  // namespace tp3
