// Stage (a) coupling, folded-row form: the reference's triple products
//   T[(k1,k2,k3)][(l1,l2,l3)] = sum_j w_j Re(c_k1[l1,m1] c_k2[l2,m2] c_k3[l3,m3])
// (src/correlations.jl:157-176; src/cuda_kernel.cu:31-37), pair-factorised as
//   D[k1,k2][l3][m3] = sum_m1 w(l1 m1 l2 m2 l3 m3) c_k1[l1,m1] c_k2[l2,m2],  m2 = -m3 - m1
//   T[(k1,k2,k3)][lt] = Re sum_m3 D[k1,k2][l3][m3] c_k3[l3,m3]
// and laid out so that every warp instruction does full-width work.
//
// One CTA = one (l1, l2) pair block of one proposal.  Its warps take work units from a
// shared counter; a unit is a folded pair of k1 rows, k1 = j and k1 = K-1-j, whose
// (j + 1) + (K - j) = K + 1 shell pairs fill the warp's lanes (27 of 32 at K = 26).
//   Phase 1: the warp walks pairs of m3 and, inside them, m1; every lane owns one shell
//     pair and accumulates its D for both m3 and all the block's l3 at once (one complex
//     product per m1 and m3, reused by every l3).  All lanes read the same 3j values (a
//     16-byte broadcast holds two orders of both m3), the same two k1 rows of c_k1 and
//     consecutive c_k2 entries (no bank conflicts); 3j columns of orders l3 < |m3| (zero)
//     are not stored, so they are never multiplied.
//   Phase 2: lanes own 4 x 4 tiles (4 shells k2 x 4 shells k3 <= k2) of one l3 and
//     contract D with the staged c_k3 over m3; both operands come as 16-byte loads.
// Both phases synchronise only the warp.  D lives in a per-warp shared-memory buffer of
// `drows` rows (one row per (l3, m3), one slot per shell pair); a block whose D would not
// fit is processed in chunks of l3 (each chunk recomputes the shell products).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tp3.h"
#include "internal.h"
#include "tables.h"

namespace tp3 {
namespace {

__device__ __forceinline__ void fold_store_split(void* hi, void* lo, size_t i, float v, bool tf32) {
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

// Asynchronous global -> shared copies (cp.async): every copy of a staging step is in
// flight at once and one wait covers them.  live = false writes zeros (no bytes read).
__device__ __forceinline__ void fold_cp8(void* dst, const void* src, bool live) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(__cvta_generic_to_global(src)), "r"(live ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void fold_cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(__cvta_generic_to_global(src))
               : "memory");
}
__device__ __forceinline__ void fold_cp_wait() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// D row of order s inside a chunk starting at s_lo: rows of the orders before s,
// (l3 + 1) per order for real functions (m3 = 0..l3), (2 l3 + 1) otherwise.
__device__ __forceinline__ int fold_drow(int s, int s_lo, int l3min, bool sym) {
  const int d = s - s_lo;
  return sym ? d * (l3min + 1) + d * (s + s_lo - 1) : d * (2 * l3min + 1) + 2 * d * (s + s_lo - 1);
}

// Phase-1 inner loop for one m3 pair: n1 values of m1, NE 3j columns (even count).
// c1 / c2 point at this lane's shells in rows m1lo and m2(m1lo) of the first m3; the
// second m3's c_k2 row is dps away; rows are ps apart.  w holds (w_a, w_b) per column.
// Accumulators are packed over the m3 pair -- R[j] = (Re D_a, Re D_b), I[j] = (Im D_a,
// Im D_b) of column j -- so each (w_a, w_b) half of a 16-byte load feeds one packed FMA
// (fma.rn.f32x2: both lanes rounded as two fmaf, the same values as scalar FMAs).
template <int NE>
__device__ __forceinline__ void fold_p1(const float2* __restrict__ c1, const float2* __restrict__ c2, int dps, int ps,
                                        int n1, const float* __restrict__ w, int rs2, float2* R, float2* I) {
#pragma unroll
  for (int j = 0; j < NE; ++j) { R[j] = make_float2(0.f, 0.f); I[j] = make_float2(0.f, 0.f); }
#pragma unroll 2
  for (int i = 0; i < n1; ++i) {
    const float2 a = c1[i * ps];
    const float2 b0 = c2[-i * ps];
    const float2 b1 = c2[-i * ps + dps];
    const float2 xr = make_float2(fmaf(a.x, b0.x, -a.y * b0.y), fmaf(a.x, b1.x, -a.y * b1.y));
    const float2 xi = make_float2(fmaf(a.x, b0.y, a.y * b0.x), fmaf(a.x, b1.y, a.y * b1.x));
    const float4* wr = reinterpret_cast<const float4*>(w + i * rs2);
#pragma unroll
    for (int j2 = 0; j2 < NE / 2; ++j2) {
      const float4 wv = wr[j2];  // (w_a, w_b) of columns 2 j2 and 2 j2 + 1
      const float2 w0 = make_float2(wv.x, wv.y), w1 = make_float2(wv.z, wv.w);
      R[2 * j2] = __ffma2_rn(w0, xr, R[2 * j2]);
      I[2 * j2] = __ffma2_rn(w0, xi, I[2 * j2]);
      R[2 * j2 + 1] = __ffma2_rn(w1, xr, R[2 * j2 + 1]);
      I[2 * j2 + 1] = __ffma2_rn(w1, xi, I[2 * j2 + 1]);
    }
  }
}

template <int NE>
__device__ __forceinline__ void fold_p1_store(const float2* c1, const float2* c2, int dps, int ps, int n1,
                                              const float* w, int rs2, bool valid, int a, int s0a, int s0b,
                                              int s_hi, int s_lo, int l3min, int m3a, int m3b, bool sym, float2* Dw,
                                              int slot, int drows, int* err) {
  float2 R[NE], I[NE];
  fold_p1<NE>(c1, c2, dps, ps, n1, w, rs2, R, I);
  if (!valid) return;
#pragma unroll
  for (int j = 0; j < NE; ++j) {
    const int s = a + j;
    if (s >= s_lo && s < s_hi) {
      const int l3 = l3min + 2 * s;
      const int r = fold_drow(s, s_lo, l3min, sym);
      // real functions: T = 2 sum_{m3 >= 0} Re(D c) with the m3 = 0 term halved here;
      // D is stored conjugated, (Re D, -Im D), for the packed phase-2 products
      const float h = (sym && m3a == 0) ? 0.5f : 1.f;
      const int ra = r + (sym ? m3a : m3a + l3), rb = r + (sym ? m3b : m3b + l3);
      if (s >= s0a && TP3_DCHECK(ra >= 0 && ra < drows && slot < ps, err))
        Dw[ra * ps + slot] = make_float2(h * R[j].x, -(h * I[j].x));
      if (s >= s0b && TP3_DCHECK(rb >= 0 && rb < drows && slot < ps, err))
        Dw[rb * ps + slot] = make_float2(R[j].y, -I[j].y);
    }
  }
}

// Phase-2 tile: acc[i][j] = Re sum_r D[row r][pair slot + i] cT[row r][shell + j] over the
// cnt rows of one order (dp, cp at the order's first row; rows are rstride float4 apart).
// D is stored conjugated, so (Re D, -Im D) * (Re c, Im c) lane by lane is a pair whose sum
// is Re(D c): one packed FMA per (i, j) and row, the two lanes summed at the end.
__device__ __forceinline__ void fold_tile(const float4* __restrict__ dp, const float4* __restrict__ cp, int rstride,
                                          int cnt, float (&acc)[4][4]) {
  float2 a2[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) a2[i][j] = make_float2(0.f, 0.f);
#pragma unroll 2
  for (int r = 0; r < cnt; ++r) {
    const float4 d01 = dp[r * rstride], d23 = dp[r * rstride + 1];
    const float4 c01 = cp[r * rstride], c23 = cp[r * rstride + 1];
    const float2 x[4] = {make_float2(d01.x, d01.y), make_float2(d01.z, d01.w), make_float2(d23.x, d23.y),
                         make_float2(d23.z, d23.w)};
    const float2 y[4] = {make_float2(c01.x, c01.y), make_float2(c01.z, c01.w), make_float2(c23.x, c23.y),
                         make_float2(c23.z, c23.w)};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) a2[i][j] = __ffma2_rn(x[i], y[j], a2[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = a2[i][j].x + a2[i][j].y;
}

// Synchronise the G warps that share a unit: the warp itself (G = 1) or a named barrier
// (id 1 + group) over the group's 32 G threads.
template <int G>
__device__ __forceinline__ void fold_gsync(int group) {
  if (G == 1)
    __syncwarp();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(1 + group), "r"(32 * G) : "memory");
}

// Tile (q2, q3) of a unit's tile index t (tiles of one k1 row: q2 = 0.., q3 <= q2).
__device__ __forceinline__ void fold_tile_of(int t, int& q2, int& q3) {
  q2 = 0;
  while ((q2 + 1) * (q2 + 2) / 2 <= t) ++q2;
  q3 = t - q2 * (q2 + 1) / 2;
}

// grid: (n_pb, n); block NW * 32; dynamic shared memory FoldVariant::smem.
// T layout: ltmaj = false: [prop][ki][lt] (row stride KP); ltmaj = true (BF16 only):
// [prop][lt][ki] (row stride klp), written through a per-warp staging row of `stage`
// floats so that each order's values of the unit's shell triples leave as contiguous runs.
// MAXNE: the widest phase-1 column run compiled in (10 covers L <= 18); registers are sized
// for it, so the narrower instance fits 13 warps without spilling.  G: warps per unit.
// With G = 2 the two warps of a group share one D buffer and one staging row: phase 1
// splits the unit's m3 pairs between them (disjoint D rows), phase 2 its tiles and T runs,
// with a named barrier between the steps; units go to groups in a fixed order.  That keeps
// the D depth (hence l3 chunks) of NW / G buffers with NW warps hiding latency.
template <int NW, int MAXNE, int G>
__global__ void __launch_bounds__(NW * 32, 1) k_couple_fold(
    const float2* __restrict__ cc, int K, int nc, const int* __restrict__ coff, const FoldBlock* __restrict__ blks,
    const FoldRow* __restrict__ rows, const float* __restrict__ wtab, const int2* __restrict__ chunks, int ps,
    int drows, int wmax, int cmax, int stage, int klp, int KP, const int* __restrict__ symflags,
    void* __restrict__ Thi, void* __restrict__ Tlo, bool tf32out, bool ltmaj, float* __restrict__ T32, int ldT32,
    const RagInfo* __restrict__ rag, int* __restrict__ err) {
  extern __shared__ __align__(16) float smf[];
  __shared__ int s_next[kFoldMaxChunks];
  __shared__ FoldRow s_rows[kFoldMaxRows];
  // per-CTA constants, read once from global memory
  __shared__ FoldBlock s_fb;
  __shared__ int s_misc[4];  // sym, Kp, skip (absent orders of a ragged proposal), klen
  __shared__ int s_coff[kFoldMaxRows];
  __shared__ int2 s_chunks[kFoldMaxChunks];
  const int prop = blockIdx.y;
  if (threadIdx.x == 0) {
    const FoldBlock b = blks[blockIdx.x];
    s_fb = b;
    int Kq = K, skip = 0, klen = 0;
    if (rag) {
      const RagInfo ri = rag[prop];
      Kq = ri.K;
      klen = ri.klen;
      skip = (b.l1 > ri.L || b.l2 > ri.L) ? 1 : 0;
    }
    const int sy = symflags[prop] != 0;
    s_misc[0] = sy;
    s_misc[1] = Kq;
    s_misc[2] = skip;
    s_misc[3] = klen;
    const int nch = sy ? b.nch_sym : b.nch_gen, ch0 = sy ? b.ch_sym0 : b.ch_gen0;
    for (int c = 0; c < nch; ++c) s_chunks[c] = chunks[ch0 + c];
  }
  __syncthreads();
  const FoldBlock fb = s_fb;
  const int Kp = s_misc[1];
  if (s_misc[2]) {
    // absent orders: the block's l-triples are zero for this proposal's scored rows
    const int klen = s_misc[3];
    for (int i = threadIdx.x; i < klen * fb.nl3; i += blockDim.x) {
      const int ki = i / fb.nl3, sj = i - ki * fb.nl3;
      if (ltmaj) {
        const int li = i % klen, lj = i / klen;  // consecutive threads: consecutive shell triples
        fold_store_split(Thi, Tlo, ((size_t)prop * KP + fb.lt_base + lj) * klp + li, 0.f, false);
      } else {
        fold_store_split(Thi, Tlo, ((size_t)prop * klp + ki) * KP + fb.lt_base + sj, 0.f, tf32out);
      }
      if (T32) T32[((size_t)prop * klp + ki) * ldT32 + fb.lt_base + sj] = 0.f;
    }
    return;
  }
  const bool sym = s_misc[0] != 0;
  const int l1 = fb.l1, l2 = fb.l2, l3min = fb.l3min, M = fb.M;
  // shared memory: C1 [2 l1 + 1][ps], C2 [2 l2 + 3][ps] (rows m2 = -l2 - 1 .. l2 + 1;
  // shell index fastest), the block's 3j rows, cT [drows][ps] (the chunk's c_k3 rows,
  // shell index fastest), D [NW][drows][ps]
  float2* C1 = reinterpret_cast<float2*>(smf);
  float2* C2 = C1 + (size_t)cmax * ps;
  float* W = reinterpret_cast<float*>(C2 + (size_t)(cmax + 2) * ps);
  float2* cT = reinterpret_cast<float2*>(W + wmax);
  float2* Dall = cT + (size_t)drows * ps;
  constexpr int NG = NW / G;  // unit groups, each with a D buffer and a staging row
  float* Stage = reinterpret_cast<float*>(Dall + (size_t)NG * drows * ps);  // [NG][stage]
  const float2* src = cc + (size_t)prop * K * nc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    const int nl = (max(max(l1, l2), M) >> 1) + 1;  // even orders used by this block
    if (threadIdx.x < nl) s_coff[threadIdx.x] = coff[threadIdx.x];
  }
  __syncthreads();
  const int o1 = s_coff[l1 >> 1], o2 = s_coff[l2 >> 1];
  // staging: one warp per coefficient row, one lane per shell (the loads of a thread are
  // independent, so they overlap)
  {
    const int n1r = 2 * l1 + 1, n2r = 2 * l2 + 1;
    for (int k0 = 0; k0 < ps; k0 += 32) {
      const int k = k0 + lane;
      const bool live = k < Kp;
      const float2* sk = src + (size_t)(live ? k : 0) * nc;
      for (int m = warp; m < n1r; m += NW)
        if (TP3_DCHECK(m < cmax && o1 + m < nc, err)) fold_cp8(&C1[m * ps + k], sk + o1 + m, live);
      // C2 has a zero row at each end: the union m1 range of an m3 pair reaches one row
      // past either end, where the pair's 3j value is zero
      for (int m = warp; m < n2r + 2; m += NW)
        if (TP3_DCHECK(m < cmax + 2 && o2 + n2r - 1 < nc, err))
          fold_cp8(&C2[m * ps + k], sk + o2 + (m >= 1 && m <= n2r ? m - 1 : 0), live && m >= 1 && m <= n2r);
    }
    int wn = (sym ? fb.wsym : fb.wall) / 4;
    if (!TP3_DCHECK(4 * wn <= wmax, err)) wn = 0;
    const float4* w4 = reinterpret_cast<const float4*>(wtab + fb.w0);
    float4* s4 = reinterpret_cast<float4*>(W);
    for (int i = threadIdx.x; i < wn; i += NW * 32) fold_cp16(&s4[i], &w4[i]);
    const int nr = sym ? fb.npair_sym : fb.npair_all;
    for (int i = threadIdx.x; i < nr; i += NW * 32)
      if (TP3_DCHECK(i < kFoldMaxRows, err)) s_rows[i] = rows[fb.row0 + i];
    fold_cp_wait();
  }
  const int nch = sym ? fb.nch_sym : fb.nch_gen;
  if (threadIdx.x < kFoldMaxChunks) s_next[threadIdx.x] = 0;

  const int group = warp / G, sub = warp - group * G;
  float2* Dw = Dall + (size_t)group * drows * ps;
  float* Ts = Stage + (size_t)group * stage;
  const size_t tbase = (size_t)prop * klp * KP;
  void* ThiP = tf32out ? (void*)((float*)Thi + tbase) : (void*)((__nv_bfloat16*)Thi + tbase);
  void* TloP = tf32out ? (void*)((float*)Tlo + tbase) : (void*)((__nv_bfloat16*)Tlo + tbase);
  float* T32P = T32 ? T32 + (size_t)prop * klp * ldT32 : nullptr;
  const int nunits = (Kp + 1) >> 1;
  const int npairs = sym ? fb.npair_sym : fb.npair_all;

  for (int ch = 0; ch < nch; ++ch) {
    const int2 chk = s_chunks[ch];
    const int s_lo = chk.x, s_hi = chk.y;
    const int l3top = l3min + 2 * (s_hi - 1);
    __syncthreads();  // the previous chunk's cT reads are done; C1 / C2 / W are staged
    // cT rows of this chunk: c_k3[l3][m3] (m3 >= 0 for real functions)
    {
      int r0 = 0;
      for (int s = s_lo; s < s_hi; ++s) {
        const int l3 = l3min + 2 * s;
        const int cnt = sym ? l3 + 1 : 2 * l3 + 1;
        const int o3 = s_coff[l3 >> 1] + (sym ? l3 : 0);  // compact index of row r = 0
        for (int k0 = 0; k0 < ps; k0 += 32) {
          const int k = k0 + lane;
          const bool live = k < Kp;
          const float2* sk = src + (size_t)(live ? k : 0) * nc + o3;
          for (int r = warp; r < cnt; r += NW)
            if (TP3_DCHECK(r0 + r < drows && o3 + r < nc, err)) fold_cp8(&cT[(r0 + r) * ps + k], sk + r, live);
        }
        r0 += cnt;
      }
      fold_cp_wait();
    }
    __syncthreads();
    for (int gu = group;; gu += NG) {
      int u = 0;
      if (G == 1) {
        if (lane == 0) u = atomicAdd(&s_next[ch], 1);
        u = __shfl_sync(0xffffffffu, u, 0);
      } else {
        u = gu;
      }
      if (u >= nunits) break;
      const int k1a = u, k1b = Kp - 1 - u;
      const bool two = k1b != k1a;
      const int off2 = (u + 2) & ~1;  // slot of (k1b, 0): even, so shell quads are 16-byte aligned
      const int nslots = two ? off2 + k1b + 1 : u + 1;
      // ---------------- phase 1: D of the unit's shell pairs ----------------
      for (int slot0 = 0; slot0 < nslots; slot0 += 32) {
        const int slot = slot0 + lane;
        int k1 = k1a, k2 = 0;
        bool valid = false;
        if (slot <= u) { k2 = slot; valid = true; }
        else if (two && slot >= off2 && slot - off2 <= k1b) { k1 = k1b; k2 = slot - off2; valid = true; }
        const int mtop = min(M, l3top);
        for (int pi = sub; pi < npairs; pi += G) {
          const FoldRow fr = s_rows[pi];
          if ((fr.m3a < 0 ? -fr.m3a : fr.m3a) > mtop) continue;
          const int m3a = fr.m3a, m3b = m3a >= 0 ? m3a + 1 : m3a - 1;
          const int a = max(fr.c0, s_lo & ~1);  // even: 16-byte aligned 3j column pairs
          const int b = min(fr.c0 + fr.rs, (s_hi + 1) & ~1);
          const int ne = b - a;
          if (ne <= 0) continue;
          const float2* c1 = C1 + (fr.m1lo + l1) * ps + k1;
          const float2* c2 = C2 + (-m3a - fr.m1lo + l2 + 1) * ps + k2;
          const int dps = m3a >= 0 ? -ps : ps;
          const float* w = W + fr.wofs + 2 * (a - fr.c0);
#ifdef TP3_DEBUG
          {  // the m1 loop's first and last rows of c_k1, c_k2 (both m3) and 3j values
            const int r1 = fr.m1lo + l1, r2 = -m3a - fr.m1lo + l2 + 1, d = dps / ps;
            const int r2z = r2 - (fr.n1 - 1);
            const bool ok = r1 >= 0 && r1 + fr.n1 - 1 <= 2 * l1 && r2 < cmax + 2 && r2z >= 0 && r2 + d < cmax + 2 &&
                            r2z + d >= 0 && k1 < ps && k2 < ps && ne <= 16 &&
                            fr.wofs + 2 * (a - fr.c0) + 2 * fr.rs * (fr.n1 - 1) + 2 * ne <= (sym ? fb.wsym : fb.wall);
            if (!TP3_DCHECK(ok, err)) continue;
          }
#endif
#define TP3_FOLD_P1(NE)                                                                                  \
  case NE:                                                                                               \
    fold_p1_store<NE>(c1, c2, dps, ps, fr.n1, w, 2 * fr.rs, valid, a, fr.s0a, fr.s0b, s_hi, s_lo, l3min, \
                      m3a, m3b, sym, Dw, slot, drows, err);                                              \
    break;
          if (ne <= 10) {
            switch (ne) {
              TP3_FOLD_P1(2) TP3_FOLD_P1(4) TP3_FOLD_P1(6) TP3_FOLD_P1(8) TP3_FOLD_P1(10)
              default: break;
            }
          } else if constexpr (MAXNE > 10) {
            switch (ne) {
              TP3_FOLD_P1(12) TP3_FOLD_P1(14) TP3_FOLD_P1(16)
              default: break;
            }
          }
#undef TP3_FOLD_P1
        }
      }
      fold_gsync<G>(group);
      // ---------------- phase 2: T of the unit's shell triples ----------------
      const int qa = (k1a >> 2) + 1, ta = qa * (qa + 1) / 2;
      const int qb = (k1b >> 2) + 1, tb = two ? qb * (qb + 1) / 2 : 0;
      const int nt = ta + tb;
      const int nitems = (s_hi - s_lo) * nt;
      const float scale = sym ? 2.f : 1.f;
      const int rstride = ps / 2;  // float4 per row
      if (ltmaj) {
        // order by order: tiles -> staging row (the unit's shell triples, k1a's then
        // k1b's) -> contiguous runs of T[lt][ki]
        const int na = (k1a + 1) * (k1a + 2) / 2, nb = two ? (k1b + 1) * (k1b + 2) / 2 : 0;
        const int t3a = k1a * (k1a + 1) * (k1a + 2) / 6, t3b = k1b * (k1b + 1) * (k1b + 2) / 6;
        for (int s = s_hi - 1; s >= s_lo; --s) {
          const int l3 = l3min + 2 * s;
          const int cnt = sym ? l3 + 1 : 2 * l3 + 1;
          const int r0 = fold_drow(s, s_lo, l3min, sym);
          const int lt = fb.lt_base + s;
          for (int tile = lane + 32 * sub; tile < nt; tile += 32 * G) {
            int t = tile, k1 = k1a, pbase = 0, lbase = 0;
            if (t >= ta) { t -= ta; k1 = k1b; pbase = off2; lbase = na; }
            int q2, q3;
            fold_tile_of(t, q2, q3);
            if (!TP3_DCHECK(r0 + cnt <= drows && pbase + 4 * q2 + 3 < ps && 4 * q3 + 3 < ps, err)) continue;
            float acc[4][4];
            fold_tile(reinterpret_cast<const float4*>(Dw + r0 * ps + pbase + 4 * q2),
                      reinterpret_cast<const float4*>(cT + r0 * ps + 4 * q3), rstride, cnt, acc);
            const int t3 = k1 * (k1 + 1) * (k1 + 2) / 6;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const int k2 = 4 * q2 + i;
              if (k2 > k1) continue;
              const int loc0 = k2 * (k2 + 1) / 2 + 4 * q3;
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                if (4 * q3 + j <= k2 && TP3_DCHECK(lbase + loc0 + j < stage, err)) {
                  const float v = scale * acc[i][j];
                  Ts[lbase + loc0 + j] = v;
                  if (T32P) T32P[(size_t)(t3 + loc0 + j) * ldT32 + lt] = v;
                }
              }
            }
          }
          fold_gsync<G>(group);
          __nv_bfloat16* hrow = reinterpret_cast<__nv_bfloat16*>(Thi) + ((size_t)prop * KP + lt) * klp;
          __nv_bfloat16* lrow = reinterpret_cast<__nv_bfloat16*>(Tlo) + ((size_t)prop * KP + lt) * klp;
          for (int idx = lane + 32 * sub; idx < na + nb; idx += 32 * G) {
            const int ki = idx < na ? t3a + idx : t3b + (idx - na);
            if (!TP3_DCHECK(ki < klp && lt < KP && idx < stage, err)) continue;
            const float v = Ts[idx];
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            hrow[ki] = h;
            lrow[ki] = __float2bfloat16_rn(v - __bfloat162float(h));
          }
          fold_gsync<G>(group);
        }
      } else {
        for (int base = 32 * sub; base < nitems; base += 32 * G) {
          const int it = base + lane;
          if (it >= nitems) break;
          const int sidx = it / nt;
          const int tile = it - sidx * nt;
          const int s = s_hi - 1 - sidx;  // largest l3 first
          int t = tile, k1 = k1a, pbase = 0;
          if (t >= ta) { t -= ta; k1 = k1b; pbase = off2; }
          int q2, q3;
          fold_tile_of(t, q2, q3);
          const int l3 = l3min + 2 * s;
          const int cnt = sym ? l3 + 1 : 2 * l3 + 1;
          const int r0 = fold_drow(s, s_lo, l3min, sym);
          if (!TP3_DCHECK(r0 + cnt <= drows && pbase + 4 * q2 + 3 < ps && 4 * q3 + 3 < ps, err)) continue;
          float acc[4][4];
          fold_tile(reinterpret_cast<const float4*>(Dw + r0 * ps + pbase + 4 * q2),
                    reinterpret_cast<const float4*>(cT + r0 * ps + 4 * q3), rstride, cnt, acc);
          const int lt = fb.lt_base + s;
          const int t3 = k1 * (k1 + 1) * (k1 + 2) / 6;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int k2 = 4 * q2 + i;
            if (k2 > k1) continue;
            const int row0 = t3 + k2 * (k2 + 1) / 2 + 4 * q3;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              if (4 * q3 + j <= k2 && TP3_DCHECK(row0 + j < klp && lt < KP, err)) {
                const float v = scale * acc[i][j];
                fold_store_split(ThiP, TloP, (size_t)(row0 + j) * KP + lt, v, tf32out);
                if (T32P) T32P[(size_t)(row0 + j) * ldT32 + lt] = v;
              }
            }
          }
        }
      }
      fold_gsync<G>(group);  // the group's D and staging row are free for its next unit
    }
  }
}

}  // namespace

// ---- host side ----------------------------------------------------------------

std::string build_fold_tables(const std::vector<PairBlock>& pbs, int drows, std::vector<FoldBlock>& blks,
                              std::vector<FoldRow>& rows, std::vector<float>& w, std::vector<int2>& chunks,
                              int& wmax, int& cmax) {
  blks.clear();
  rows.clear();
  w.clear();
  chunks.clear();
  wmax = 0;
  cmax = 0;
  for (const PairBlock& pb : pbs) {
    FoldBlock fb{};
    fb.l1 = pb.l1; fb.l2 = pb.l2; fb.l3min = pb.l3min; fb.nl3 = pb.nl3; fb.M = pb.M; fb.lt_base = pb.lt_base;
    if (pb.M + 1 > kFoldMaxRows) return "fold tables: more m3 pairs than the kernel stages";
    fb.row0 = (int)rows.size();
    fb.w0 = (int)w.size();
    const int nl3e = (pb.nl3 + 1) & ~1;
    auto s0_of = [&](int m3) {
      const int am = m3 < 0 ? -m3 : m3;
      return am > pb.M ? pb.nl3 : std::max(0, (am - pb.l3min + 1) / 2);
    };
    auto m1lo_of = [&](int m3) { return std::max(-pb.l1, -pb.l2 - m3); };
    auto m1hi_of = [&](int m3) { return std::min(pb.l1, pb.l2 - m3); };
    int run = 0;
    // pairs (0,1), (2,3), ... (the real-function prefix), then (-1,-2), (-3,-4), ...
    for (int pass = 0; pass < 2; ++pass) {
      for (int m3a = pass == 0 ? 0 : -1; pass == 0 ? m3a <= pb.M : m3a >= -pb.M; m3a += pass == 0 ? 2 : -2) {
        const int m3b = pass == 0 ? m3a + 1 : m3a - 1;
        const bool hasb = (m3b < 0 ? -m3b : m3b) <= pb.M;
        FoldRow fr{};
        fr.m3a = m3a;
        int lo = m1lo_of(m3a), hi = m1hi_of(m3a);
        if (hi < lo) return "fold tables: empty m1 range";
        if (hasb && m1hi_of(m3b) >= m1lo_of(m3b)) {
          lo = std::min(lo, m1lo_of(m3b));
          hi = std::max(hi, m1hi_of(m3b));
        }
        fr.m1lo = lo;
        fr.n1 = hi - lo + 1;
        fr.s0a = s0_of(m3a);
        fr.s0b = hasb ? s0_of(m3b) : pb.nl3;
        if (fr.s0a >= pb.nl3) return "fold tables: no order l3 >= |m3|";
        fr.c0 = fr.s0a & ~1;
        fr.rs = nl3e - fr.c0;
        fr.wofs = run;
        for (int i = 0; i < fr.n1; ++i) {
          const int m1 = fr.m1lo + i;
          for (int c = 0; c < fr.rs; ++c) {
            const int s = fr.c0 + c;
            const int l3 = pb.l3min + 2 * s;
            for (int q = 0; q < 2; ++q) {
              const int m3 = q == 0 ? m3a : m3b;
              const int s0 = q == 0 ? fr.s0a : fr.s0b;
              const bool in = (q == 0 || hasb) && s >= s0 && s < pb.nl3 && m1 >= m1lo_of(m3) && m1 <= m1hi_of(m3);
              w.push_back(in ? (float)tp3::wigner3j(pb.l1, pb.l2, l3, m1, -m3 - m1, m3) : 0.f);
            }
          }
          run += 2 * fr.rs;
        }
        rows.push_back(fr);
      }
      if (pass == 0) {
        while (run % 4) { w.push_back(0.f); ++run; }
        fb.wsym = run;
        fb.npair_sym = (int)rows.size() - fb.row0;
      }
    }
    fb.npair_all = (int)rows.size() - fb.row0;
    while (run % 4) { w.push_back(0.f); ++run; }
    fb.wall = run;
    wmax = std::max(wmax, run);
    cmax = std::max(cmax, std::max(2 * pb.l1 + 1, 2 * pb.l2 + 1));
    // chunks of consecutive l3 orders whose D rows fit drows.  Each chunk forms its shell
    // products again for every m3 row up to its highest order, so the split is chosen to
    // minimise the estimated phase-1 instructions -- per m3-pair row reaching the chunk,
    // n1 (11 + 2.5 ne): the product and load overhead of an m1 step plus its column loads
    // and packed FMAs -- over at most kFoldMaxChunks chunks (dynamic programming over
    // chunk ends; nl3 <= 16).
    for (int pass = 0; pass < 2; ++pass) {
      const bool sym = pass == 0;
      const int r_begin = fb.row0, r_end = fb.row0 + (sym ? fb.npair_sym : fb.npair_all);
      auto drows_of = [&](int s_lo, int s_hi) {
        int r = 0;
        for (int s = s_lo; s < s_hi; ++s) {
          const int l3 = pb.l3min + 2 * s;
          r += sym ? l3 + 1 : 2 * l3 + 1;
        }
        return r;
      };
      auto cost = [&](int s_lo, int s_hi) {
        const int l3top = pb.l3min + 2 * (s_hi - 1);
        double c = 0.0;
        for (int ri = r_begin; ri < r_end; ++ri) {
          const FoldRow& fr = rows[ri];
          if ((fr.m3a < 0 ? -fr.m3a : fr.m3a) > std::min(pb.M, l3top)) continue;
          const int a = std::max(fr.c0, s_lo & ~1), b = std::min(fr.c0 + fr.rs, (s_hi + 1) & ~1);
          if (b > a) c += fr.n1 * (11.0 + 2.5 * (b - a));
        }
        return c;
      };
      const int nl = pb.nl3;
      const double inf = 1e300;
      // best[n][e]: cheapest split of orders [0, e) into n chunks; from[n][e]: its last start
      std::vector<std::vector<double>> best(kFoldMaxChunks + 1, std::vector<double>(nl + 1, inf));
      std::vector<std::vector<int>> from(kFoldMaxChunks + 1, std::vector<int>(nl + 1, -1));
      best[0][0] = 0.0;
      for (int n = 1; n <= kFoldMaxChunks; ++n)
        for (int e = 1; e <= nl; ++e)
          for (int st = 0; st < e; ++st) {
            if (best[n - 1][st] >= inf || drows_of(st, e) > drows) continue;
            const double v = best[n - 1][st] + cost(st, e);
            if (v < best[n][e]) { best[n][e] = v; from[n][e] = st; }
          }
      int nbest = -1;
      for (int n = 1; n <= kFoldMaxChunks; ++n)
        if (best[n][nl] < inf && (nbest < 0 || best[n][nl] < best[nbest][nl])) nbest = n;
      if (nbest < 0) {
        for (int s3 = 0; s3 < nl; ++s3)
          if (drows_of(s3, s3 + 1) > drows) return "fold tables: one order of D exceeds the per-warp buffer";
        return "fold tables: too many l3 chunks";
      }
      std::vector<int2> split;
      for (int n = nbest, e = nl; n > 0; --n) {
        const int st = from[n][e];
        split.push_back(make_int2(st, e));
        e = st;
      }
      (sym ? fb.ch_sym0 : fb.ch_gen0) = (int)chunks.size();
      for (auto it = split.rbegin(); it != split.rend(); ++it) chunks.push_back(*it);
      (sym ? fb.nch_sym : fb.nch_gen) = nbest;
    }
    blks.push_back(fb);
  }
  return "";
}

size_t fold_smem_bytes(int ngroups, int ps, int drows, int wmax, int cmax, int stage) {
  return (size_t)(2 * cmax + 2) * ps * sizeof(float2) + (size_t)wmax * sizeof(float) +
         (size_t)(1 + ngroups) * drows * ps * sizeof(float2) + (size_t)ngroups * stage * sizeof(float);
}

cudaError_t fold_configure() {
  cudaError_t e;
  const int cs = kCoupleMaxDynSmem;
  const cudaFuncAttribute ds = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if ((e = cudaFuncSetAttribute(k_couple_fold<7, 10, 1>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<8, 10, 1>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<13, 10, 1>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<14, 10, 2>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<7, 16, 1>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<8, 16, 1>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<13, 16, 1>, ds, cs)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_couple_fold<14, 16, 2>, ds, cs)) != cudaSuccess)
    return e;
  return cudaSuccess;
}

cudaError_t launch_couple_fold(const DevTables& t, const TcTables& tc, const FoldVariant& fv, int n, const float2* cc,
                               const int* sym, void* Thi, void* Tlo, bool tf32, float* T32, cudaStream_t s,
                               const RagInfo* rag) {
  dim3 grid(tc.n_pb, n);
  const bool ltmaj = t_order_major(tc, tf32);
#define TP3_FOLD_LAUNCH(NW, MX, G)                                                                                \
  k_couple_fold<NW, MX, G><<<grid, NW * 32, fv.smem, s>>>(cc, t.K, t.nc, tc.coff, fv.blks, fv.rows, fv.w,          \
                                                          fv.chunks, fv.ps, fv.drows, fv.wmax, fv.cmax, fv.stage,   \
                                                          t.klp, tc.KP, sym, Thi, Tlo, tf32, ltmaj, T32, t.n_ltp,   \
                                                          rag, tc.err)
  const bool narrow = fv.maxne <= 10;
  switch (fv.nw * 4 + fv.grp) {
    case 7 * 4 + 1: if (narrow) TP3_FOLD_LAUNCH(7, 10, 1); else TP3_FOLD_LAUNCH(7, 16, 1); break;
    case 8 * 4 + 1: if (narrow) TP3_FOLD_LAUNCH(8, 10, 1); else TP3_FOLD_LAUNCH(8, 16, 1); break;
    case 13 * 4 + 1: if (narrow) TP3_FOLD_LAUNCH(13, 10, 1); else TP3_FOLD_LAUNCH(13, 16, 1); break;
    case 14 * 4 + 2: if (narrow) TP3_FOLD_LAUNCH(14, 10, 2); else TP3_FOLD_LAUNCH(14, 16, 2); break;
    default: return cudaErrorInvalidValue;
  }
#undef TP3_FOLD_LAUNCH
  return cudaGetLastError();
}

}  // namespace tp3
