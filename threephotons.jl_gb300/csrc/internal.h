// Internal declarations shared by the context code and the kernel files.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

namespace tp3 {

// TP3_DEBUG builds (TP3_DEBUG=1 python threephotons.jl_gb300/build.py --force) check the
// indices that the gather and folded-row coupling kernels compute before each shared- or
// global-memory access; a failed check sets TP3_ERR_BOUNDS in the context's error flag
// (reported by the next synchronising call) and skips the access.  Release builds
// compile the checks out.
#ifdef TP3_DEBUG
__device__ __forceinline__ bool tp3_dcheck(bool ok, int* err) {
  if (!ok && err) atomicExch(err, 10 /* TP3_ERR_BOUNDS */);
  return ok;
}
#define TP3_DCHECK(cond, err) tp3_dcheck((cond), (err))
#else
#define TP3_DCHECK(cond, err) true
#endif

// Device view of the per-context tables (all pointers are device memory).
struct DevTables {
  int K, nc, LMAX;
  int n_lt, n_ltp;      // l-triples, padded count (row stride of T and F)
  int klength, klp;     // shell triples, padded to the TC row tile
  int G, Gu, mult, N;
  const int* csean;     // [nc] compact -> seanindex0
  const int* cident;    // [nc] identity map (compact input)
  const float* w;       // [basislen]
  const uint32_t* idx;  // [basislen] i1 | i2 << 10 | i3 << 20
  const int2* lt;       // [n_lt] (jstart, jcount)
  const int4* kl;       // [klength] (k1, k2, k3, tf)
  const double* tf;     // [klength]
  const float* Ffull;   // [G][n_ltp]  fp32, full grid (plain path)
  const int* u_to_g;    // [Gu]
  // lambda != 0 (shell-dependent Legendre factors): Fourier-pair form of the angular stage
  int nq = 0, nqp = 0;       // (m2, m3) pairs up to sign, padded to 16 (0 at lambda = 0)
  const float* Ytab = nullptr;   // [K][nc] sphPlm(l, m, theta_k)
  const int* lt_of_j = nullptr;  // [basislen]
  const int* qstart = nullptr;   // [nq + 1] ranges of qlist
  const int* qlist = nullptr;    // [basislen] basis entries grouped by pair
  const int4* qent = nullptr;    // [basislen] in qlist order: packed indices, w (float bits), l-triple
  const float* Cq = nullptr;     // [G][nqp] cos(m2 alpha + m3 beta)
  const int* g_to_u;    // [G]
};

// Plain path launches (kernels_plain.cu).
// Input coefficient layouts of the gather kernels: per shell either the full
// seanindex-ordered LMAX^2 vector (map = csean, stride LMAX^2) or the compact even-l
// block (map = identity, stride nc).
struct CoeffLayout {
  const int* map;
  int stride;
};
cudaError_t launch_gather(const DevTables& t, int n, const double2* coeff, CoeffLayout lay, float2* cc,
                          cudaStream_t s);
cudaError_t launch_couple_direct(const DevTables& t, int n, const float2* cc, float* T, cudaStream_t s);
// Bayes partials: part[prop][cg][klength] (Sp, Sql); ncg column groups over the full grid.
cudaError_t launch_angular_plain(const DevTables& t, int n, const float* T, const float* q,
                                 double2* part, int ncg, float* c3out, cudaStream_t s);
cudaError_t launch_build_H(const DevTables& t, int n, const float* T, float* H, cudaStream_t s);
// lambda != 0 on the tensor-core path: H of a batch from FP32 T, written as split rows
// [n][klp][KP] (bf16 hi + lo, or tf32 hi + fp32 lo); pair columns past nq are zero.
size_t build_H_split_smem(const DevTables& t, int ppl);
cudaError_t launch_build_H_split(const DevTables& t, int KP, int n, const float* T32, void* Hhi, void* Hlo, bool tf32,
                                 cudaStream_t s);
cudaError_t launch_finalize(const DevTables& t, int n, const double2* part, int ncg,
                            const double* Qs, int mult, double* E, cudaStream_t s);

// One (l1, l2) block of the pair-factorised coupling.
struct PairBlock {
  int l1, l2, l3min, nl3;  // l3 = l3min + 2 s, s < nl3
  int M;                   // |m3| <= M
  int SD;                  // sum_s (2 l3_s + 1)
  int lt_base;             // l-triple index of (l1, l2, l3min); the block's l-triples are consecutive
  int wofs;                // offset of the block in wtab (16-byte aligned)
  int eofs;                // offset of the block's per-m3 table in eofs[]
  int nl3p;                // nl3 rounded up to 2 (row length of the 3j table: whole float2s)
  int wcount;              // floats in the block's 3j table (multiple of 4)
};

// Folded-row coupling (kernels_fold.cu): per pair block, the 3j rows of every m3
// with only the orders l3 >= |m3| stored, and the l3 chunks whose D rows fit one
// warp's buffer.
constexpr int kFoldMaxChunks = 8;
constexpr int kFoldMaxRows = 32;  // m3 pairs of one block, <= M + 1 (M <= 30)
struct FoldBlock {
  int l1, l2, l3min, nl3, M, lt_base;
  int row0;                  // first FoldRow of the block
  int w0;                    // float offset of the block's 3j rows (16-byte aligned)
  int wsym, wall;            // floats of the m3 >= 0 prefix and of all rows (multiples of 4)
  int npair_sym, npair_all;  // m3 pairs of the prefix and in all
  int ch_sym0, nch_sym;      // l3 chunks, real-function path (D rows of l3 + 1)
  int ch_gen0, nch_gen;      // l3 chunks, general path (D rows of 2 l3 + 1)
};
// Rows come in pairs of m3 (m3a and m3b = m3a + 1 for m3a >= 0, m3a - 1 below), so a
// lane forms two products per m1 from one c_k1 load; the pair's 3j values are stored
// interleaved per column, (w_a, w_b), over the union of the two m1 ranges (zero where
// a row's own range or order range does not reach; a partner beyond M is all zero).
struct FoldRow {
  int m3a;       // first m3 of the pair
  int m1lo, n1;  // m1 = m1lo .. m1lo + n1 - 1 (union of the pair's ranges)
  int s0a, s0b;  // first order index with l3 >= |m3| for each m3 (nl3 for an absent partner)
  int c0, rs;    // first stored column (even) and columns per m1 (even)
  int wofs;      // float offset of the pair's rows in the block's table (multiple of 4)
};
// One tiling of the folded-row coupling: nw warps per CTA, drows D rows per warp, ps
// shell-pair slots per D row (>= K + 5, multiple of 32).
struct FoldVariant {
  bool ok = false;
  int nw = 0, drows = 0, ps = 0, wmax = 0, cmax = 0;
  int stage = 0;  // floats of a warp's staging row (1 + K(K+1)/2 shell triples, rounded to 4)
  int maxne = 0;  // widest phase-1 column run of any block (even l3 count, rounded up to even)
  int grp = 1;    // warps per unit (each group of grp warps shares one D buffer)
  size_t smem = 0;
  const FoldBlock* blks = nullptr;
  const FoldRow* rows = nullptr;
  const float* w = nullptr;
  const int2* chunks = nullptr;
};

// Device tables of the tensor-core path.
struct TcTables {
  // folded-row coupling tilings: [0] 8 warps, [1] 7 warps, [2] 13 warps (smaller D
  // buffers, more l3 chunks), [3] 14 warps in pairs sharing 7 D buffers; one CTA per SM
  FoldVariant fold[4];
  int use_fold = -1;
  int* err = nullptr;  // the context's device error flag (index checks of TP3_DEBUG builds)
  int n_pb = 0, maxs = 0, SDmax = 0;
  int ncp = 0, SDp = 0, pmax = 0, nchunks = 0, wsmem = 0;  // coupling kernel shared-memory layout
  bool w_smem = false;
  size_t couple_smem = 0;
  const int2* chunks = nullptr;  // (k1 high, k1 low) runs of shells, pairs per run <= pmax
  const int2* chunks_sym = nullptr;  // same for the real-function path (rows of SDhp)
  int nchunks_sym = 0, pmax_sym = 0, SDhp = 0;
  // second tiling of the one-kernel coupling: 256 threads and at most kCoupleSmallSmem
  // bytes of shared memory per CTA, so two CTAs share an SM (one computes while the
  // other waits at its chunk barrier)
  bool small_ok = false;
  bool use_small = false;
  bool w_smem_s = false;
  size_t couple_smem_s = 0;
  const int2* chunks_s = nullptr;
  const int2* chunks_sym_s = nullptr;
  int nchunks_s = 0, nchunks_sym_s = 0, pmax_s = 0, pmax_sym_s = 0;
  // warp-local one-kernel coupling (k_couple_warp): per-warp D buffers of 4 shell pairs
  bool warp_ok = false;
  bool use_warp = false;
  bool w_smem_w = false;
  size_t couple_smem_w = 0;
  // the warp-local coupling at 256 threads, two CTAs per SM
  bool warp2_ok = false, use_warp2 = false, w_smem_w2 = false;
  size_t couple_smem_w2 = 0;
  // split coupling (kernels_couple.cu)
  bool split = false;            // use the two-kernel coupling
  bool split_ok = false;         // the two-kernel coupling fits this shape
  bool fused_ok = false;         // the one-kernel coupling fits this shape
  const long long* doff = nullptr;  // [n_pb] offset of each pair block's D rows in one proposal's D
  long long dstride = 0;         // float2 per proposal of D
  int dsub = 1;                  // proposals per (D, T) kernel pair, sized so D stays in L2
  const int4* units_sym = nullptr;  // (pair block, m3 lo, m3 hi) work units, real-function path
  const int4* units_gen = nullptr;  // same for the general path
  int n_units_sym = 0, n_units_gen = 0;
  int dmax = 0;                  // largest l1 (or l2) of any block
  int unit_wmax = 0;             // largest 3j row range of any unit (floats)
  const int* cm = nullptr;       // [nc] m of each compact coefficient
  const int* cl = nullptr;       // [nc] l of each compact coefficient
  const int* cmir = nullptr;     // [nc] compact index of (l, -m)
  int KP = 0;              // K extent of the angular GEMM: l-triples (lambda = 0) or Fourier
                           // pairs (lambda != 0), padded to 32; also the row stride of T hi / lo
  int NP = 0, nhalf = 0;   // unique grid points padded to 256 * nhalf
  int nsm = 0;             // SMs of the context's device (persistent angular grid)
  bool hform = false;      // lambda != 0: the angular A operand is H (Fourier pairs), B the cosine table
  bool persist = true;     // angular stage: persistent kernel (true) or one CTA per tile
  const int* coff = nullptr;
  const PairBlock* pbs = nullptr;
  const int* eofs = nullptr;
  const float* wtab = nullptr;
  const __nv_bfloat16* Fhi = nullptr;  // [NP][KP]
  const __nv_bfloat16* Flo = nullptr;
  const float* Fhi32 = nullptr;        // [NP][KP] TF32 hi (fp32 with the low 13 bits clear)
  const float* Flo32 = nullptr;        // [NP][KP] fp32 remainder
};

// Per-proposal limits of a ragged batch (chains of different L and K scored in one
// launch on the context's largest shape): orders above L and shells from K on are
// treated as absent, only the first klen = K(K+1)(K+2)/6 shell triples are scored,
// against histogram number hist of the context's histogram set.
struct RagInfo {
  int L, K, klen, hist;
};

struct TcMaps {
  CUtensorMap a_hi, a_lo, b_hi, b_lo;
  CUtensorMap a_hi_mn, a_lo_mn;  // BF16 T operand in the order-major layout [lt][ki]
};

size_t tc_smem_bytes();
// Dynamic shared memory the coupling kernel may request (the opt-in maximum of
// 227 KB minus its static counters and slack).
constexpr int kCoupleMaxDynSmem = 227 * 1024 - 2048;
constexpr int kCoupleSmallSmem = 110 * 1024;
cudaError_t tc_configure();
cudaError_t launch_gather_sym(const DevTables& t, const TcTables& tc, int n, const double2* coeff, CoeffLayout lay,
                              float2* cc, int* sym, cudaStream_t s, const RagInfo* rag = nullptr);
cudaError_t launch_couple_pair(const DevTables& t, const TcTables& tc, int n, const float2* cc, const int* sym,
                               void* Thi, void* Tlo, bool tf32, float* T32, cudaStream_t s,
                               const RagInfo* rag = nullptr);
// qt / Qs: one histogram, or (rag) the histogram set with strides klp * Gu and klength.
cudaError_t launch_angular_tc(const DevTables& t, const TcTables& tc, const TcMaps& maps, int n, const float* qt,
                              const double* Qs, double* Eslab, float* c3out, int* err, bool tf32, cudaStream_t s,
                              const RagInfo* rag = nullptr);
cudaError_t launch_finalize_slabs(int n, int klength, const double* Eslab, double* E, cudaStream_t s,
                                  const RagInfo* rag = nullptr);
// Persistent angular stage: compensated partial sums into part ([n][klp][4 nhalf] floats),
// or (c3out) c3 rows [n][klength][2N^2];
// launch_finalize_parts turns them into slab terms (Eslab [n][klength]) and sums those
// per proposal in a fixed order.
cudaError_t launch_angular_persistent(const DevTables& t, const TcTables& tc, const TcMaps& maps, int n,
                                      const float* qt, float* part, int* err, bool tf32, cudaStream_t s,
                                      const RagInfo* rag = nullptr, float* c3out = nullptr);
cudaError_t launch_finalize_parts(const DevTables& t, const TcTables& tc, int n, const float* part, const double* Qs,
                                  double* Eslab, double* E, cudaStream_t s, const RagInfo* rag = nullptr);
size_t couple_split_smem_d(const DevTables& t, const TcTables& tc);
size_t couple_split_smem_t(const DevTables& t, const TcTables& tc);
cudaError_t couple_split_configure(const DevTables& t, const TcTables& tc);
std::string build_fold_tables(const std::vector<PairBlock>& pbs, int drows, std::vector<FoldBlock>& blks,
                              std::vector<FoldRow>& rows, std::vector<float>& w, std::vector<int2>& chunks,
                              int& wmax, int& cmax);
// ngroups: D buffers and staging rows (warps per CTA / warps per unit)
size_t fold_smem_bytes(int ngroups, int ps, int drows, int wmax, int cmax, int stage);
// Layout of the T operand: the folded-row coupling in BF16 mode writes it order-major,
// [lt][ki] (shell triples contiguous), read by the angular kernel as an MN-major operand;
// every other coupling form and the TF32 mode use [ki][lt].
inline bool t_order_major(const TcTables& tc, bool tf32) {
  return !tf32 && !tc.hform && tc.use_fold >= 0 && tc.fold[tc.use_fold].ok;
}
cudaError_t fold_configure();
cudaError_t launch_couple_fold(const DevTables& t, const TcTables& tc, const FoldVariant& fv, int n, const float2* cc,
                               const int* sym, void* Thi, void* Tlo, bool tf32, float* T32, cudaStream_t s,
                               const RagInfo* rag = nullptr);
cudaError_t launch_couple_split(const DevTables& t, const TcTables& tc, int n, const float2* cc, const int* sym,
                                float2* Dg, void* Thi, void* Tlo, bool tf32, float* T32, cudaStream_t s);

int plain_ncg(const DevTables& t);
// Detail text returned by tp3_last_error(NULL) on this thread.
void set_thread_error(const std::string& msg);
// Per-device kernel attributes of the plain path (call with the device current).
cudaError_t plain_configure();
constexpr int kPlainMaxSmem = 200 * 1024;

}  // namespace tp3
