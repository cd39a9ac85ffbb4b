// Context and C ABI of libtp3 (declared in include/tp3.h).
//
// A context owns every device buffer of one (L, LMAX, N, K, lambda) basis: the
// tables built once from tables.cpp, the normalised histogram, and scratch sized
// for the largest batch seen (or reserved).  Nothing is allocated per call once
// the scratch fits; no call falls back to the CPU.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <tuple>
#include <vector>

#include "ctx_internal.h"

using tp3::Basis;
using tp3::DevTables;
using tp3::PairBlock;
using tp3::TcMaps;
using tp3::TcTables;

namespace {
thread_local std::string g_create_error;

// Autotuned evaluation variant (mode, coupling form, angular schedule) per shape,
// shared by every context of the process; TP3_MODE_AUTO uses it when present.
struct TuneEntry {
  int mode = -1;
  int split = 0;
  bool persist = true;
};
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int, double, double>, TuneEntry> g_tuned;

std::tuple<int, int, int, int, double, double> tune_key(const tp3::Basis& b) {
  return std::make_tuple(b.L, b.LMAX, b.N, b.K, b.lambda, b.dq);
}

}  // namespace

void tp3::set_thread_error(const std::string& msg) { g_create_error = msg; }

namespace {

bool is_tc(int mode) { return mode == TP3_MODE_TC_BF16X3 || mode == TP3_MODE_TC_TF32X3; }

int fail(tp3_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg; else g_create_error = msg;
  return code;
}

int cuda_fail(tp3_ctx* c, cudaError_t e, const char* where) {
  return fail(c, TP3_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <class T>
cudaError_t upload(tp3_ctx* c, const std::vector<T>& h, const T** out) {
  void* p = nullptr;
  size_t bytes = std::max<size_t>(h.size() * sizeof(T), 16);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return e;
  c->allocs.push_back(p);
  if (!h.empty()) e = cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  *out = (const T*)p;
  return e;
}

// ---- tensor-core path tables -------------------------------------------------
std::string build_tc_tables(const Basis& b, std::vector<PairBlock>& pbs, std::vector<int>& eofs,
                            std::vector<float>& wtab, int& maxs, int& SDmax) {
  std::map<std::tuple<int, int, int>, int> ltidx;
  for (int t = 0; t < b.n_lt(); ++t) ltidx[{b.lt_l1[t], b.lt_l2[t], b.lt_l3[t]}] = t;
  struct Item { PairBlock pb; double work; std::vector<int> e; std::vector<float> w; };
  std::vector<Item> items;
  maxs = 0;
  SDmax = 0;
  for (int l1 = 0; l1 <= b.L; l1 += 2)
    for (int l2 = 0; l2 <= b.L; l2 += 2) {
      const int l3min = std::abs(l1 - l2), l3max = std::min(l1 + l2, b.L - (b.L & 1));
      if (l3min > l3max) continue;
      Item it{};
      PairBlock& pb = it.pb;
      pb.l1 = l1; pb.l2 = l2; pb.l3min = l3min; pb.nl3 = (l3max - l3min) / 2 + 1; pb.M = l3max;
      pb.SD = 0;
      for (int s = 0; s < pb.nl3; ++s) {
        const int l3 = l3min + 2 * s;
        auto f = ltidx.find({l1, l2, l3});
        if (f == ltidx.end()) return "pair block l-triple missing from the basis";
        if (s == 0) pb.lt_base = f->second;
        else if (f->second != pb.lt_base + s) return "pair block l-triples are not consecutive";
        pb.SD += 2 * l3 + 1;
      }
      pb.nl3p = (pb.nl3 + 1) / 2 * 2;
      int run = 0;
      for (int e = 0; e <= 2 * pb.M; ++e) {
        const int m3 = e - pb.M;
        it.e.push_back(run);
        const int m1lo = std::max(-l1, -l2 - m3), m1hi = std::min(l1, l2 - m3);
        for (int m1 = m1lo; m1 <= m1hi; ++m1) {
          const int m2 = -m3 - m1;
          for (int s = 0; s < pb.nl3p; ++s) {
            const int l3 = l3min + 2 * s;
            it.w.push_back(s < pb.nl3 && std::abs(m3) <= l3 ? (float)tp3::wigner3j(l1, l2, l3, m1, m2, m3) : 0.f);
          }
          run += pb.nl3p;
        }
      }
      while (run % 4) { it.w.push_back(0.f); ++run; }  // block length: whole float4s
      pb.wcount = run;
      it.work = (double)run;
      maxs = std::max(maxs, pb.nl3);
      SDmax = std::max(SDmax, pb.SD);
      items.push_back(std::move(it));
    }
  std::sort(items.begin(), items.end(), [](const Item& a, const Item& c) { return a.work > c.work; });
  for (auto& it : items) {
    it.pb.wofs = (int)wtab.size();  // multiple of 4: every block starts on a 16-byte boundary
    it.pb.eofs = (int)eofs.size();
    wtab.insert(wtab.end(), it.w.begin(), it.w.end());
    eofs.insert(eofs.end(), it.e.begin(), it.e.end());
    pbs.push_back(it.pb);
  }
  return "";
}

// 2-D tensor map over a [rows][inner] K-major operand; the box is one 64-byte row of K
// (32 bf16 or 16 tf32 elements) by box_rows rows, 64-byte swizzle.
cudaError_t encode_2d(tp3_ctx* c, CUtensorMap* m, void* ptr, uint64_t inner, uint64_t rows, uint32_t box_rows,
                      bool f32) {
  const uint64_t esz = f32 ? 4 : 2;
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {inner * esz};
  cuuint32_t box[2] = {(cuuint32_t)(64 / esz), box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = c->encode(m, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims,
                         strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// 2-D tensor map over the BF16 T operand in the order-major layout [rows][inner] (inner =
// shell triples): boxes of 64 shell triples (128 bytes) by 32 orders, 128-byte swizzle.
cudaError_t encode_2d_mn(tp3_ctx* c, CUtensorMap* m, void* ptr, uint64_t inner, uint64_t rows) {
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {inner * 2};
  cuuint32_t box[2] = {64, 32};
  cuuint32_t es[2] = {1, 1};
  CUresult r = c->encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

std::string setup_tc(tp3_ctx* c) {
  const Basis& b = c->b;
  DevTables& t = c->t;
  TcTables& tc = c->tc;
  // lambda = 0: F on the 4:1-folded grid; lambda != 0: the cosine table of the Fourier
  // pairs on the full grid (the persistent angular kernel walks any number of halves)
  tc.hform = b.lambda != 0.0;
  if (!tc.hform && b.mult != 4) return "needs even N (grid fold)";
  if (!tc.hform && b.Gu > 512) return "more than 512 unique grid points (N > 32)";
  if (tc.hform && (b.Gu > 8192 || c->qpairs.empty())) return "lambda != 0: more than 8192 grid points";
  if (tc.hform && tp3::build_H_split_smem(c->t, 1) > (size_t)tp3::kPlainMaxSmem)
    return "lambda != 0: the l-triples of a shell triple exceed the H kernel's shared memory";
  std::vector<PairBlock> pbs;
  std::vector<int> eofs;
  std::vector<float> wtab;
  int maxs = 0, SDmax = 0;
  std::string m = build_tc_tables(b, pbs, eofs, wtab, maxs, SDmax);
  if (!m.empty()) return m;
  if (maxs > 16) return "more than 16 l3 values per pair block (L > 30)";
  for (const auto& pb : pbs)
    if (pb.wofs % 4 != 0 || pb.wcount % 4 != 0 || pb.nl3p % 2 != 0) return "3j block alignment invariant violated";
  for (int v : eofs)
    if (v % 2 != 0) return "3j row alignment invariant violated";
  tc.n_pb = (int)pbs.size();
  tc.maxs = maxs;
  if (cudaDeviceGetAttribute(&tc.nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || tc.nsm < 1)
    return "SM count query failed";
  tc.SDmax = SDmax;
  // coupling kernel shared memory: coefficients [K][ncp], 3j block, D [pmax][SDp]
  tc.ncp = b.nc | 1;
  tc.SDp = SDmax | 1;
  int wmax = 0;
  for (const auto& pb : pbs) wmax = std::max(wmax, pb.wcount);
  tc.wsmem = wmax;
  const size_t limit = tp3::kCoupleMaxDynSmem;
  // coefficient block rounded up to 16 bytes so the 3j block (float4 copies) stays aligned
  const size_t base = ((size_t)b.K * tc.ncp * sizeof(float2) + 15) / 16 * 16;
  // D is double-buffered: two chunks of up to pmax shell pairs
  int pmax = std::max(b.K, 128);
  tc.w_smem = true;
  auto need = [&](int pm, bool ws) {
    return base + (ws ? (size_t)wmax * 4 : 0) + 2 * (size_t)pm * tc.SDp * sizeof(float2);
  };
  while (need(pmax, true) > limit && pmax > b.K) --pmax;
  if (need(pmax, true) > limit) { tc.w_smem = false; pmax = std::max(b.K, 128); }
  while (need(pmax, false) > limit && pmax > b.K) --pmax;
  // the fused coupling needs one k1's pairs per chunk in shared memory; when it does not
  // fit (large K x L) only the split coupling (D through global memory) is used
  tc.fused_ok = need(pmax, tc.w_smem) <= limit;
  if (!tc.fused_ok) pmax = b.K;
  tc.pmax = pmax;
  tc.couple_smem = need(pmax, tc.w_smem);
  // real-function path: D rows hold m3 = 0..l3 only, so the same bytes hold more pairs
  int SDh = 0;
  for (const auto& pb : pbs) {
    int h = 0;
    for (int s3 = 0; s3 < pb.nl3; ++s3) h += pb.l3min + 2 * s3 + 1;
    SDh = std::max(SDh, h);
  }
  tc.SDhp = SDh | 1;
  tc.pmax_sym = (int)((2 * (size_t)pmax * tc.SDp) / (2 * (size_t)tc.SDhp));
  // chunks of whole k1 values, largest shells first, at most pmax shell pairs each
  auto make_chunks = [&](int pm) {
    std::vector<int2> ch;
    for (int k1 = b.K - 1; k1 >= 0;) {
      int hi = k1, cnt = 0;
      while (k1 >= 0 && cnt + k1 + 1 <= pm) { cnt += k1 + 1; --k1; }
      ch.push_back(make_int2(hi, k1 + 1));
    }
    return ch;
  };
  std::vector<int2> chunks = make_chunks(pmax), chunks_sym = make_chunks(tc.pmax_sym);
  tc.nchunks = (int)chunks.size();
  tc.nchunks_sym = (int)chunks_sym.size();
  if (tc.nchunks_sym > 64 || tc.nchunks > 64) tc.fused_ok = false;
  // the small tiling (256 threads, two CTAs per SM)
  const size_t limit_s = tp3::kCoupleSmallSmem;
  int pmax_s = std::max(b.K, 128);
  tc.w_smem_s = true;
  while (need(pmax_s, true) > limit_s && pmax_s > b.K) --pmax_s;
  if (need(pmax_s, true) > limit_s) { tc.w_smem_s = false; pmax_s = std::max(b.K, 128); }
  while (need(pmax_s, false) > limit_s && pmax_s > b.K) --pmax_s;
  tc.small_ok = need(pmax_s, tc.w_smem_s) <= limit_s;
  tc.pmax_s = pmax_s;
  tc.couple_smem_s = need(pmax_s, tc.w_smem_s);
  tc.pmax_sym_s = (int)((2 * (size_t)pmax_s * tc.SDp) / (2 * (size_t)tc.SDhp));
  std::vector<int2> chunks_s = make_chunks(pmax_s), chunks_sym_s = make_chunks(tc.pmax_sym_s);
  tc.nchunks_s = (int)chunks_s.size();
  tc.nchunks_sym_s = (int)chunks_sym_s.size();
  if (tc.nchunks_s > 64 || tc.nchunks_sym_s > 64) tc.small_ok = false;
  // the warp-local coupling: 16 warps x 4 shell pairs of D (general rows, SDp)
  {
    const size_t dw = (size_t)16 * 4 * tc.SDp * sizeof(float2);
    tc.w_smem_w = base + (size_t)wmax * 4 + dw <= limit;
    tc.couple_smem_w = base + (tc.w_smem_w ? (size_t)wmax * 4 : 0) + dw;
    tc.warp_ok = tc.couple_smem_w <= limit && b.K <= 64;
    // 256 threads: two CTAs per SM when the layout fits 110 KB, else one CTA per SM
    // with up to the full dynamic shared memory (large K and L, where 16 warps' D does not fit)
    const size_t dw2 = (size_t)8 * 4 * tc.SDp * sizeof(float2);
    const size_t lim2 = base + dw2 <= limit_s ? limit_s : limit;
    tc.w_smem_w2 = base + (size_t)wmax * 4 + dw2 <= lim2;
    tc.couple_smem_w2 = base + (tc.w_smem_w2 ? (size_t)wmax * 4 : 0) + dw2;
    tc.warp2_ok = tc.couple_smem_w2 <= lim2 && b.K <= 64;
  }
  // split coupling: D offsets, L2-sized sub-batches, balanced (pair block, m3 range) units
  const int npairs = b.K * (b.K + 1) / 2;
  std::vector<long long> doff(pbs.size());
  long long dst = 0;
  tc.dmax = 0;
  for (size_t i = 0; i < pbs.size(); ++i) {
    doff[i] = dst;
    dst += (long long)npairs * pbs[i].SD;
    tc.dmax = std::max(tc.dmax, std::max(pbs[i].l1, pbs[i].l2));
  }
  tc.dstride = dst;
  tc.dsub = (int)std::max<long long>(1, (72LL << 20) / (dst * (long long)sizeof(float2)));
  auto m3work = [&](const PairBlock& pb, int m3) {
    const int n = std::min(pb.l1, pb.l2 - m3) - std::max(-pb.l1, -pb.l2 - m3) + 1;
    return (double)std::max(n, 0) * (4 + 2 * pb.nl3p);
  };
  double target = 0;
  for (const auto& pb : pbs)
    for (int m3 = 0; m3 <= pb.M; ++m3) target = std::max(target, m3work(pb, m3));
  struct U { int4 u; double w; };
  std::vector<U> us, ug;
  auto cut = [&](std::vector<U>& out, int pbi, int from, int to, int step) {  // m3 = from .. to by step
    const PairBlock& pb = pbs[pbi];
    int lo = from;
    double w = 0;
    for (int m3 = from;; m3 += step) {
      w += m3work(pb, m3);
      const bool last = m3 == to;
      if (w >= target || last) {
        const int a = std::min(lo, m3), z = std::max(lo, m3);
        out.push_back({make_int4(pbi, a, z, 0), w});
        lo = m3 + step;
        w = 0;
      }
      if (last) break;
    }
  };
  for (int i = 0; i < (int)pbs.size(); ++i) {
    cut(us, i, 0, pbs[i].M, 1);
    cut(ug, i, 0, pbs[i].M, 1);
    if (pbs[i].M > 0) cut(ug, i, -1, -pbs[i].M, -1);
  }
  auto heavy_first = [](const U& a, const U& c) { return a.w > c.w; };
  std::sort(us.begin(), us.end(), heavy_first);
  std::sort(ug.begin(), ug.end(), heavy_first);
  std::vector<int4> units_sym, units_gen;
  tc.unit_wmax = 0;
  for (const auto* lst : {&us, &ug})
    for (const auto& x : *lst) {
      const PairBlock& pb = pbs[x.u.x];
      if (x.u.y < 0 && x.u.z > 0) return "work unit straddles m3 = 0";
      const int wb = eofs[pb.eofs + x.u.y + pb.M];
      const int we = (x.u.z + pb.M + 1 <= 2 * pb.M) ? eofs[pb.eofs + x.u.z + pb.M + 1] : pb.wcount;
      tc.unit_wmax = std::max(tc.unit_wmax, we - wb);
    }
  for (const auto& x : us) units_sym.push_back(x.u);
  for (const auto& x : ug) units_gen.push_back(x.u);
  // every (pair block, m3) is covered exactly once: m3 >= 0 by the real-function units,
  // -M..M by the general ones
  for (int pass = 0; pass < 2; ++pass) {
    const auto& lst = pass == 0 ? units_sym : units_gen;
    for (int i = 0; i < (int)pbs.size(); ++i) {
      std::vector<int> cover(2 * pbs[i].M + 1, 0);
      for (const auto& u : lst)
        if (u.x == i)
          for (int m3 = u.y; m3 <= u.z; ++m3) cover[m3 + pbs[i].M]++;
      for (int m3 = -pbs[i].M; m3 <= pbs[i].M; ++m3)
        if (cover[m3 + pbs[i].M] != ((pass == 0 && m3 < 0) ? 0 : 1)) return "coupling work units do not cover m3";
    }
  }
  tc.n_units_sym = (int)units_sym.size();
  tc.n_units_gen = (int)units_gen.size();
  std::vector<int> cmir(b.nc);
  for (int i = 0; i < b.nc; ++i) cmir[i] = b.coff[b.c_l[i] / 2] + b.c_l[i] - b.c_m[i];
  const int kcols = tc.hform ? (int)c->qpairs.size() : b.n_lt();  // K extent before padding
  tc.KP = (std::max(kcols, b.n_lt()) + 31) / 32 * 32;
  tc.nhalf = (b.Gu + 255) / 256;
  tc.NP = 256 * tc.nhalf;
  // B operand on the unique grid points, split into bf16 hi + lo and into tf32 hi + fp32
  // lo: F[u][lt] (lambda = 0) or cos(m2 alpha + m3 beta) of each Fourier pair (lambda != 0)
  std::vector<double> F;
  if (tc.hform) {
    F.assign((size_t)b.Gu * kcols, 0.0);
    for (int u = 0; u < b.Gu; ++u) {
      const int g = b.u_to_g[u], a = g % b.N, bb = g / b.N;
      const double al = (a + 0.5) * M_PI / b.N, be = (bb + 0.5) * M_PI / b.N;
      for (int q = 0; q < kcols; ++q)
        F[(size_t)u * kcols + q] = std::cos(c->qpairs[q].first * al + c->qpairs[q].second * be);
    }
  } else {
    tp3::build_F(b, F);
  }
  std::vector<__nv_bfloat16> Fhi((size_t)tc.NP * tc.KP, __float2bfloat16(0.f)), Flo(Fhi);
  std::vector<float> Fhi32((size_t)tc.NP * tc.KP, 0.f), Flo32(Fhi32);
  for (int u = 0; u < b.Gu; ++u)
    for (int l = 0; l < kcols; ++l) {
      const double v64 = F[(size_t)u * kcols + l];
      const float v = (float)v64;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      Fhi[(size_t)u * tc.KP + l] = hi;
      Flo[(size_t)u * tc.KP + l] = __float2bfloat16_rn(v - __bfloat162float(hi));
      // tf32: round the fp32 value to 10 explicit mantissa bits (nearest, ties away from zero)
      uint32_t bits;
      std::memcpy(&bits, &v, 4);
      bits = (bits + 0x1000u) & ~0x1FFFu;
      float h32;
      std::memcpy(&h32, &bits, 4);
      Fhi32[(size_t)u * tc.KP + l] = h32;
      Flo32[(size_t)u * tc.KP + l] = (float)(v64 - (double)h32);
    }
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return "cuTensorMapEncodeTiled unavailable";
  c->encode = (tp3::EncodeTiledFn)fn;
  cudaError_t e;
  if ((e = upload(c, b.coff, &tc.coff)) != cudaSuccess || (e = upload(c, pbs, &tc.pbs)) != cudaSuccess ||
      (e = upload(c, eofs, &tc.eofs)) != cudaSuccess || (e = upload(c, wtab, &tc.wtab)) != cudaSuccess ||
      (e = upload(c, chunks, &tc.chunks)) != cudaSuccess || (e = upload(c, chunks_sym, &tc.chunks_sym)) != cudaSuccess ||
      (e = upload(c, chunks_s, &tc.chunks_s)) != cudaSuccess ||
      (e = upload(c, chunks_sym_s, &tc.chunks_sym_s)) != cudaSuccess || (e = upload(c, b.c_m, &tc.cm)) != cudaSuccess ||
      (e = upload(c, b.c_l, &tc.cl)) != cudaSuccess ||
      (e = upload(c, cmir, &tc.cmir)) != cudaSuccess || (e = upload(c, doff, &tc.doff)) != cudaSuccess ||
      (e = upload(c, units_sym, &tc.units_sym)) != cudaSuccess ||
      (e = upload(c, units_gen, &tc.units_gen)) != cudaSuccess ||
      (e = upload(c, Fhi, &tc.Fhi)) != cudaSuccess || (e = upload(c, Flo, &tc.Flo)) != cudaSuccess ||
      (e = upload(c, Fhi32, &tc.Fhi32)) != cudaSuccess || (e = upload(c, Flo32, &tc.Flo32)) != cudaSuccess ||
      (e = tp3::tc_configure()) != cudaSuccess)
    return std::string("tensor-core table upload: ") + cudaGetErrorString(e);
  // folded-row coupling: three tilings in up to 225 KB, one CTA per SM (8 warps; 7 warps,
  // which take a K = 26 proposal's 13 folded units in two rounds with one warp idle; 13
  // warps, one round, with smaller D buffers), each with the largest D buffer that fits
  if ((e = tp3::fold_configure()) != cudaSuccess) return std::string("fold coupling: ") + cudaGetErrorString(e);
  {
    int rows_gen = 0;  // D rows of the largest block, general path (all l3 in one chunk)
    for (const auto& pb : pbs) {
      int r = 0;
      for (int s3 = 0; s3 < pb.nl3; ++s3) r += 2 * (pb.l3min + 2 * s3) + 1;
      rows_gen = std::max(rows_gen, r);
    }
    const int ps = (b.K + 5 + 31) / 32 * 32;
    // tilings: warps per CTA and warps per unit (the D buffers are nw / grp)
    const struct { int nw, grp; size_t budget; } fvs[4] = {{8, 1, (size_t)tp3::kCoupleMaxDynSmem},
                                                           {7, 1, (size_t)tp3::kCoupleMaxDynSmem},
                                                           {13, 1, (size_t)tp3::kCoupleMaxDynSmem},
                                                           {14, 2, (size_t)tp3::kCoupleMaxDynSmem}};
    for (int v = 0; v < 4; ++v) {
      tp3::FoldVariant& fv = tc.fold[v];
      std::vector<tp3::FoldBlock> fbl;
      std::vector<tp3::FoldRow> frows;
      std::vector<float> fw;
      std::vector<int2> fch;
      int wmx = 0, cmx = 0;
      if (!tp3::build_fold_tables(pbs, rows_gen, fbl, frows, fw, fch, wmx, cmx).empty()) continue;
      const int stage = (1 + b.K * (b.K + 1) / 2 + 3) / 4 * 4;
      const int ngroups = fvs[v].nw / fvs[v].grp;
      const size_t fixed = tp3::fold_smem_bytes(ngroups, ps, 0, wmx, cmx, stage);
      const size_t per_row = (size_t)(1 + ngroups) * ps * sizeof(float2);
      if (fixed + per_row > fvs[v].budget) continue;
      const int drows = (int)std::min<size_t>((size_t)rows_gen, (fvs[v].budget - fixed) / per_row);
      if (!tp3::build_fold_tables(pbs, drows, fbl, frows, fw, fch, wmx, cmx).empty()) continue;
      if ((e = upload(c, fbl, &fv.blks)) != cudaSuccess || (e = upload(c, frows, &fv.rows)) != cudaSuccess ||
          (e = upload(c, fw, &fv.w)) != cudaSuccess || (e = upload(c, fch, &fv.chunks)) != cudaSuccess)
        return std::string("fold coupling tables: ") + cudaGetErrorString(e);
      fv.nw = fvs[v].nw;
      fv.grp = fvs[v].grp;
      fv.drows = drows;
      fv.ps = ps;
      fv.wmax = wmx;
      fv.cmax = cmx;
      fv.stage = stage;
      fv.maxne = 0;
      for (const auto& pb : pbs) fv.maxne = std::max(fv.maxne, (pb.nl3 + 1) & ~1);
      fv.smem = tp3::fold_smem_bytes(ngroups, ps, drows, wmx, cmx, stage);
      fv.ok = fv.smem <= fvs[v].budget;
    }
  }
  // the split coupling is kept for the autotuner and for shapes the fused kernel cannot hold
  tc.split_ok = tp3::couple_split_smem_d(t, tc) <= (size_t)tp3::kCoupleMaxDynSmem &&
             tp3::couple_split_smem_t(t, tc) <= (size_t)tp3::kCoupleMaxDynSmem &&
             tp3::couple_split_configure(t, tc) == cudaSuccess;
  cudaGetLastError();
  if ((e = encode_2d(c, &c->maps.b_hi, (void*)tc.Fhi, tc.KP, tc.NP, 256, false)) != cudaSuccess ||
      (e = encode_2d(c, &c->maps.b_lo, (void*)tc.Flo, tc.KP, tc.NP, 256, false)) != cudaSuccess ||
      (e = encode_2d(c, &c->maps32.b_hi, (void*)tc.Fhi32, tc.KP, tc.NP, 256, true)) != cudaSuccess ||
      (e = encode_2d(c, &c->maps32.b_lo, (void*)tc.Flo32, tc.KP, tc.NP, 256, true)) != cudaSuccess)
    return "tensor map encoding of F failed";
  cudaGetLastError();
  if (!tc.fused_ok && !tc.split_ok) return "coupling tile exceeds shared memory";
  tc.split = !tc.fused_ok;
  (void)t;
  return "";
}

// ---- scratch ------------------------------------------------------------------
void free_scratch(tp3_ctx* c) {
  cudaFree(c->d_coeff); cudaFree(c->d_cc); cudaFree(c->d_T); cudaFree(c->d_part); cudaFree(c->d_E);
  cudaFree(c->d_Thi); cudaFree(c->d_Tlo); cudaFree(c->d_Eslab); cudaFree(c->d_sym); cudaFree(c->d_D);
  cudaFree(c->d_H);
  c->d_D = nullptr;
  c->d_H = nullptr;
  cudaFreeHost(c->h_coeff); cudaFreeHost(c->h_E);
  c->d_sym = nullptr;
  c->d_coeff = nullptr; c->d_cc = nullptr; c->d_T = nullptr; c->d_part = nullptr; c->d_E = nullptr;
  c->d_Thi = nullptr; c->d_Tlo = nullptr; c->d_Eslab = nullptr;
  c->h_coeff = nullptr; c->h_E = nullptr;
  c->cap = 0;
}

int ensure_cap(tp3_ctx* c, int n) {
  const bool need4 = c->mode == TP3_MODE_TC_TF32X3 && c->t_elem != 4;
  if (n <= c->cap && !need4) return TP3_OK;
  if (n < c->cap) n = c->cap;
  free_scratch(c);
  const auto& t = c->t;
  const int ncg = tp3::plain_ncg(t);
  const size_t ncoef = (size_t)t.LMAX * t.LMAX;
  cudaError_t e;
  const size_t tbytes = (size_t)n * t.klp * t.n_ltp * sizeof(float);
  // T operands: 2 bytes per element (bf16), 4 once the tf32 mode has been selected
  const int elem = (c->mode == TP3_MODE_TC_TF32X3 || c->t_elem == 4) ? 4 : 2;
  const size_t tcb = c->tc_ok ? (size_t)n * t.klp * c->tc.KP * elem : 0;
  if ((e = cudaMalloc(&c->d_coeff, (size_t)n * t.K * ncoef * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_cc, (size_t)n * t.K * t.nc * sizeof(float2))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_T, tbytes)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_part, (size_t)n * ncg * t.klength * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_E, (size_t)n * sizeof(double))) != cudaSuccess ||
      (c->tc_ok && (e = cudaMalloc(&c->d_Thi, tcb)) != cudaSuccess) ||
      (c->tc_ok && (e = cudaMalloc(&c->d_Tlo, tcb)) != cudaSuccess) ||
      // per-slab terms [n][klength], then (persistent schedule) 4 partial sums per grid half
      // and shell triple [n][klp][nhalf][4] floats
      (c->tc_ok && (e = cudaMalloc(&c->d_Eslab, ((size_t)n * (t.klength + 2 * (size_t)c->tc.nhalf * t.klp) + 1) *
                                                    sizeof(double))) != cudaSuccess) ||
      (e = cudaMalloc(&c->d_sym, (size_t)n * sizeof(int))) != cudaSuccess ||
      (t.nqp > 0 && (e = cudaMalloc(&c->d_H, (size_t)n * t.klp * t.nqp * sizeof(float))) != cudaSuccess) ||
      (c->tc_ok && c->tc.split_ok &&
       (e = cudaMalloc(&c->d_D, (size_t)c->tc.dsub * c->tc.dstride * sizeof(float2))) != cudaSuccess) ||
      (e = cudaMallocHost(&c->h_coeff, (size_t)n * t.K * ncoef * 2 * sizeof(double))) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_E, (size_t)n * sizeof(double))) != cudaSuccess) {
    free_scratch(c);
    cudaGetLastError();
    return fail(c, TP3_ERR_ALLOC, std::string("scratch allocation: ") + cudaGetErrorString(e));
  }
  // padding rows/columns of the coupling outputs stay zero for the lifetime of the buffers
  if ((e = cudaMemset(c->d_T, 0, tbytes)) != cudaSuccess) return cuda_fail(c, e, "cudaMemset T");
  if (t.nqp > 0 && (e = cudaMemset(c->d_H, 0, (size_t)n * t.klp * t.nqp * sizeof(float))) != cudaSuccess)
    return cuda_fail(c, e, "cudaMemset H");
  if (c->tc_ok) {
    if ((e = cudaMemset(c->d_Thi, 0, tcb)) != cudaSuccess || (e = cudaMemset(c->d_Tlo, 0, tcb)) != cudaSuccess)
      return cuda_fail(c, e, "cudaMemset T hi/lo");
    if ((e = encode_2d(c, &c->maps.a_hi, c->d_Thi, c->tc.KP, (uint64_t)n * t.klp, 128, false)) != cudaSuccess ||
        (e = encode_2d(c, &c->maps.a_lo, c->d_Tlo, c->tc.KP, (uint64_t)n * t.klp, 128, false)) != cudaSuccess ||
        (e = encode_2d_mn(c, &c->maps.a_hi_mn, c->d_Thi, t.klp, (uint64_t)n * c->tc.KP)) != cudaSuccess ||
        (e = encode_2d_mn(c, &c->maps.a_lo_mn, c->d_Tlo, t.klp, (uint64_t)n * c->tc.KP)) != cudaSuccess ||
        (elem == 4 &&
         ((e = encode_2d(c, &c->maps32.a_hi, c->d_Thi, c->tc.KP, (uint64_t)n * t.klp, 128, true)) != cudaSuccess ||
          (e = encode_2d(c, &c->maps32.a_lo, c->d_Tlo, c->tc.KP, (uint64_t)n * t.klp, 128, true)) != cudaSuccess)))
      return fail(c, TP3_ERR_CUDA, "tensor map encoding of T failed");
  }
  c->cap = n;
  c->t_elem = elem;
  ++c->scratch_gen;
  return TP3_OK;
}

int prof_begin_in(tp3_ctx* c, std::vector<cudaEvent_t>& ev, size_t& used, cudaEvent_t* a, cudaEvent_t* b) {
  if (!c->prof) return 0;
  if (used + 2 > ev.size()) {
    cudaEvent_t e1, e2;
    if (cudaEventCreate(&e1) != cudaSuccess || cudaEventCreate(&e2) != cudaSuccess) return 0;
    ev.push_back(e1);
    ev.push_back(e2);
  }
  *a = ev[used];
  *b = ev[used + 1];
  used += 2;
  cudaEventRecord(*a, c->stream);
  return 1;
}

int prof_begin(tp3_ctx* c, cudaEvent_t* a, cudaEvent_t* b) { return prof_begin_in(c, c->ev, c->ev_used, a, b); }

// Gather + coupling stage for n proposals whose FP64 coefficients are in d_coeff.
int run_coupling(tp3_ctx* c, int n, const double2* d_coeff, bool want_T32, bool compact = false,
                 const tp3::RagInfo* rag = nullptr) {
  const auto& t = c->t;
  cudaError_t e;
  const tp3::CoeffLayout lay = compact ? tp3::CoeffLayout{t.cident, t.nc} : tp3::CoeffLayout{t.csean, t.LMAX * t.LMAX};
  if (is_tc(c->mode)) {
    // lambda != 0: the coupling also writes FP32 T, from which H (the angular operand) is built
    if (c->tc.hform) want_T32 = true;
    if ((e = tp3::launch_gather_sym(t, c->tc, n, d_coeff, lay, c->d_cc, c->d_sym, c->stream, rag)) != cudaSuccess)
      return cuda_fail(c, e, "gather_sym");
    cudaEvent_t ca, cb;
    const int pc = prof_begin_in(c, c->ev_c, c->ev_c_used, &ca, &cb);
    if (rag)  // ragged batches use the one-kernel coupling (it skips absent blocks and shells)
      e = tp3::launch_couple_pair(t, c->tc, n, c->d_cc, c->d_sym, c->d_Thi, c->d_Tlo, c->mode == TP3_MODE_TC_TF32X3,
                                  want_T32 ? c->d_T : nullptr, c->stream, rag);
    else if (c->tc.split)
      e = tp3::launch_couple_split(t, c->tc, n, c->d_cc, c->d_sym, c->d_D, c->d_Thi, c->d_Tlo,
                                   c->mode == TP3_MODE_TC_TF32X3, want_T32 ? c->d_T : nullptr, c->stream);
    else
      e = tp3::launch_couple_pair(t, c->tc, n, c->d_cc, c->d_sym, c->d_Thi, c->d_Tlo, c->mode == TP3_MODE_TC_TF32X3,
                                  want_T32 ? c->d_T : nullptr, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "coupling");
    if (c->tc.hform && (e = tp3::launch_build_H_split(t, c->tc.KP, n, c->d_T, c->d_Thi, c->d_Tlo,
                                                      c->mode == TP3_MODE_TC_TF32X3, c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "build_H_split");
    if (pc) cudaEventRecord(cb, c->stream);
  } else {
    if ((e = tp3::launch_gather(t, n, d_coeff, lay, c->d_cc, c->stream)) != cudaSuccess) return cuda_fail(c, e, "gather");
    if ((e = tp3::launch_couple_direct(t, n, c->d_cc, c->d_T, c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "couple_direct");
    if (t.nqp > 0 && (e = tp3::launch_build_H(t, n, c->d_T, c->d_H, c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "build_H");
  }
  return TP3_OK;
}

// operand of the plain angular kernel: T (lambda = 0) or H (lambda != 0)
const float* plain_A(tp3_ctx* c) { return c->t.nqp > 0 ? c->d_H : c->d_T; }

// Score n proposals whose FP64 coefficients are already in d_coeff (device).
int run_energy(tp3_ctx* c, int n, const double2* d_coeff, double* d_E, bool compact = false,
               const tp3::RagInfo* rag = nullptr) {
  const auto& t = c->t;
  cudaError_t e;
  if (rag) {
    if (c->nhist == 0) return fail(c, TP3_ERR_NO_HISTOGRAM, "tp3_set_histograms has not been called");
    if (!is_tc(c->mode) || (!c->tc.fused_ok && c->tc.use_fold < 0) || c->tc.hform)
      return fail(c, TP3_ERR_UNSUPPORTED,
                  "ragged batches need a tensor-core mode with the one-kernel coupling at lambda = 0");
  } else if (!c->has_hist) {
    return fail(c, TP3_ERR_NO_HISTOGRAM, "tp3_set_histogram has not been called");
  }
  if (int r = run_coupling(c, n, d_coeff, false, compact, rag)) return r;
  cudaEvent_t a, b;
  int pr = prof_begin(c, &a, &b);
  if (is_tc(c->mode)) {
    const bool tf = c->mode == TP3_MODE_TC_TF32X3;
    const float* qt = rag ? c->d_qt_set : c->d_qt;
    const double* Qf = rag ? c->d_Qf_set : c->d_Qfold;
    if (c->tc.persist || c->tc.nhalf > 2) {
      // the partial sums start 16-byte aligned after the slab terms (float4 reads)
      float* part = reinterpret_cast<float*>(c->d_Eslab + (((size_t)c->cap * t.klength + 1) & ~(size_t)1));
      if ((e = tp3::launch_angular_persistent(t, c->tc, tf ? c->maps32 : c->maps, n, qt, part, c->d_err, tf, c->stream,
                                              rag)) != cudaSuccess)
        return cuda_fail(c, e, "angular_persistent");
      if (pr) cudaEventRecord(b, c->stream);
      if ((e = tp3::launch_finalize_parts(t, c->tc, n, part, Qf, c->d_Eslab, d_E, c->stream, rag)) != cudaSuccess)
        return cuda_fail(c, e, "finalize_parts");
    } else {
      if ((e = tp3::launch_angular_tc(t, c->tc, tf ? c->maps32 : c->maps, n, qt, Qf, c->d_Eslab, nullptr, c->d_err,
                                      tf, c->stream, rag)) != cudaSuccess)
        return cuda_fail(c, e, "angular_tc");
      if (pr) cudaEventRecord(b, c->stream);
      if ((e = tp3::launch_finalize_slabs(n, t.klength, c->d_Eslab, d_E, c->stream, rag)) != cudaSuccess)
        return cuda_fail(c, e, "finalize_slabs");
    }
  } else {
    const int ncg = tp3::plain_ncg(t);
    if ((e = tp3::launch_angular_plain(t, n, plain_A(c), c->d_qfull, c->d_part, ncg, nullptr, c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "angular_plain");
    if (pr) cudaEventRecord(b, c->stream);
    if ((e = tp3::launch_finalize(t, n, c->d_part, ncg, c->d_Qfull, 1, d_E, c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "finalize");
  }
  return TP3_OK;
}

// After a synchronising call: report a device-side timeout, if any.
int check_device_error(tp3_ctx* c) {
  cudaError_t e = cudaMemcpy(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(c, e, "error flag read");
  if (*c->h_err != 0) {
    const int code = *c->h_err;
    cudaMemset(c->d_err, 0, sizeof(int));
    return fail(c, code, code == TP3_ERR_TIMEOUT ? "a bounded device wait ran out; results of this call are invalid"
                         : code == TP3_ERR_BOUNDS
                             ? "a device index check of the TP3_DEBUG build failed (the access was skipped); results "
                               "of this call are invalid"
                             : "a device-side argument check failed (ragged limits out of range); "
                               "results of this call are invalid");
  }
  return TP3_OK;
}

int check_ctx(tp3_ctx* c) {
  if (!c) return TP3_ERR_ARG;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  return TP3_OK;
}

// Coupling form of the tensor-core path: 0 one-kernel, 1 split, 2 one-kernel small
// tiling, 3 warp-local (512 threads), 4 warp-local (256 threads, two CTAs per SM); a
// form this shape cannot run falls back to one that it can.
void apply_coupling(tp3_ctx* c, int form) {
  TcTables& tc = c->tc;
  tc.use_fold = (form == 5 && tc.fold[0].ok) ? 0 : (form == 6 && tc.fold[1].ok) ? 1
                 : (form == 7 && tc.fold[2].ok) ? 2 : (form == 8 && tc.fold[3].ok) ? 3 : -1;
  tc.use_small = form == 2 && tc.small_ok;
  tc.use_warp = form == 3 && tc.warp_ok;
  tc.use_warp2 = form == 4 && tc.warp2_ok;
  tc.split = (form == 1 && tc.split_ok) || (!tc.fused_ok && !tc.use_warp && !tc.use_warp2 && tc.use_fold < 0);
  if (tc.split) tc.use_small = tc.use_warp = tc.use_warp2 = false, tc.use_fold = -1;
}

// Folded, slab-normalised histogram of Kh shells (slabs with k1 < Kh; the rest zero)
// in the tensor-core epilogue layout qt [klp/128][Gu][128] and the folded slab sums Qf.
const char* fold_histogram(const Basis& b, const DevTables& t, const double* c3ref, int K3, int Kh, float* qt,
                           double* Qf) {
  const int G = b.G;
  const int klen = Kh * (Kh + 1) * (Kh + 2) / 6;
  std::vector<double> fold(b.Gu);
  std::fill(qt, qt + (size_t)t.klp * b.Gu, 0.f);
  for (int ki = 0; ki < b.klength; ++ki) {
    Qf[ki] = 0.0;
    if (ki >= klen) continue;
    const size_t off = (size_t)G * ((size_t)b.k3s[ki] + (size_t)K3 * ((size_t)b.k2s[ki] + (size_t)K3 * b.k1s[ki]));
    const double* s = c3ref + off;
    double l1 = 0.0;
    for (int g = 0; g < G; ++g) {
      if (!std::isfinite(s[g])) return "histogram holds NaN or Inf";
      l1 += std::fabs(s[g]);
    }
    if (!(l1 > 0.0)) return "histogram slab with zero L1 norm";
    std::fill(fold.begin(), fold.end(), 0.0);
    for (int g = 0; g < G; ++g) fold[b.g_to_u[g]] += s[g] / l1;
    const int tile = ki / 128, r = ki % 128;
    double qf = 0.0;
    for (int u = 0; u < b.Gu; ++u) {
      const float vf = (float)fold[u];
      qt[((size_t)tile * b.Gu + u) * 128 + r] = vf;
      qf += (double)vf;
    }
    Qf[ki] = qf;
  }
  return nullptr;
}

// (L, K, hist) triples -> RagInfo, clamped into range; a bad triple sets *err.
__global__ void k_rag_info(const int* __restrict__ lkh, int n, int Lmax, int Kmax, int nhist,
                           const int* __restrict__ histK, tp3::RagInfo* __restrict__ out, int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int L = lkh[3 * i], K = lkh[3 * i + 1], h = lkh[3 * i + 2];
  bool bad = false;
  if (h < 0 || h >= nhist) { bad = true; h = 0; }
  if (L < 0 || L > Lmax) { bad = true; L = L < 0 ? 0 : Lmax; }
  if (K < 1 || K > histK[h]) { bad = true; K = K < 1 ? 1 : histK[h]; }
  if (K > Kmax) K = Kmax;
  if (bad) atomicExch(err, TP3_ERR_ARG);
  tp3::RagInfo r;
  r.L = L; r.K = K; r.klen = K * (K + 1) * (K + 2) / 6; r.hist = h;
  out[i] = r;
}

// The coefficients the kernels use (even l <= L of every shell), read in place from the
// caller's [n][K][LMAX^2] buffer -- host memory the device reaches through the host page
// tables -- into the compact device layout [n][K][nc]; one thread per value, so every
// read of a batch is in flight at once.
__global__ void k_stage_coeff(const double2* __restrict__ src, int64_t total, int nc, int ncoef,
                              const int* __restrict__ csean, double2* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % nc);
    dst[i] = src[(i / nc) * ncoef + csean[c]];
  }
}

}  // namespace

int tp3::ctx_fail(tp3_ctx* c, int code, const std::string& msg) { return fail(c, code, msg); }
int tp3::ctx_cuda_fail(tp3_ctx* c, cudaError_t e, const char* where) { return cuda_fail(c, e, where); }
int tp3::ctx_check(tp3_ctx* c) { return check_ctx(c); }
int tp3::ctx_ensure_cap(tp3_ctx* c, int n) { return ensure_cap(c, n); }
int tp3::ctx_run_energy(tp3_ctx* c, int n, const double2* d_coeff, double* d_E, const tp3::RagInfo* rag) {
  return run_energy(c, n, d_coeff, d_E, false, rag);
}
int tp3::ctx_check_device_error(tp3_ctx* c) { return check_device_error(c); }
int tp3::ctx_make_rag(tp3_ctx* c, int n, const int* d_lkh, tp3::RagInfo* out) {
  if (c->nhist == 0) return fail(c, TP3_ERR_NO_HISTOGRAM, "tp3_set_histograms has not been called");
  k_rag_info<<<(n + 127) / 128, 128, 0, c->stream>>>(d_lkh, n, c->b.L, c->b.K, c->nhist, c->d_hist_K, out, c->d_err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "ragged limits");
  return TP3_OK;
}

extern "C" {

const char* tp3_status_string(int s) {
  switch (s) {
    case TP3_OK: return "ok";
    case TP3_ERR_ARG: return "bad argument or shape";
    case TP3_ERR_TABLE: return "table construction failed";
    case TP3_ERR_CUDA: return "CUDA runtime error";
    case TP3_ERR_NO_DEVICE: return "no usable CUDA device";
    case TP3_ERR_NO_HISTOGRAM: return "no histogram set";
    case TP3_ERR_BAD_HISTOGRAM: return "histogram has NaN/Inf or an all-zero slab";
    case TP3_ERR_TIMEOUT: return "device wait timed out";
    case TP3_ERR_UNSUPPORTED: return "unsupported mode or shape";
    case TP3_ERR_ALLOC: return "allocation failed";
    case TP3_ERR_BOUNDS: return "device index check failed (TP3_DEBUG build)";
    default: return "unknown status";
  }
}

const char* tp3_last_error(const tp3_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int tp3_version(void) { return (1 << 16) | 1; }

double tp3_wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  return tp3::wigner3j(j1, j2, j3, m1, m2, m3);
}

double tp3_sphPlm(int l, int m, double theta) { return tp3::sphPlm_x(l, m, std::cos(theta)); }

int tp3_basis_info(int L, int LMAX, int N, int K, double lambda, double dq, int64_t* info) {
  if (!info) return TP3_ERR_ARG;
  Basis b;
  std::string m = tp3::build_basis(b, L, LMAX, N, K, lambda, dq);
  if (!m.empty()) { g_create_error = m; return TP3_ERR_ARG; }
  tp3::fold_grid(b, true);
  info[0] = b.basislen(); info[1] = b.n_lt(); info[2] = b.klength; info[3] = b.G;
  info[4] = b.Gu; info[5] = b.mult; info[6] = b.nc;
  int64_t nnz0 = 0;  // entries whose Legendre product is non-zero at theta = pi/2
  for (int j = 0; j < b.basislen(); ++j)
    nnz0 += ((b.l1[j] + b.m1[j]) % 2 == 0 && (b.l2[j] + b.m2[j]) % 2 == 0 && (b.l3[j] + b.m3[j]) % 2 == 0);
  info[7] = nnz0;
  return TP3_OK;
}

int tp3_ctx_create(int L, int LMAX, int N, int K, double lambda, double dq, tp3_ctx** out) {
  if (!out) return fail(nullptr, TP3_ERR_ARG, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(nullptr, TP3_ERR_NO_DEVICE, "no CUDA device visible");
  }
  tp3_ctx* c = new tp3_ctx();
  cudaGetDevice(&c->device);
  {  // kernels may read pageable host buffers in place only where the device says so
    int pa = 0, pt = 0;
    cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, c->device);
    cudaDeviceGetAttribute(&pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, c->device);
    cudaGetLastError();
    c->pageable_ok = pa == 1 && pt == 1;
    c->host_direct = c->pageable_ok;
  }
  std::string m = tp3::build_basis(c->b, L, LMAX, N, K, lambda, dq);
  if (!m.empty()) { delete c; return fail(nullptr, TP3_ERR_ARG, m); }
  Basis& b = c->b;
  if (std::fabs((double)K * lambda * dq / (4.0 * M_PI)) > 1.0) {
    delete c;
    return fail(nullptr, TP3_ERR_ARG, "K * lambda * dq / (4 pi) exceeds 1: theta_k = acos(k lambda dq / 4pi) undefined");
  }
  if (b.nc > 1024) { delete c; return fail(nullptr, TP3_ERR_UNSUPPORTED, "L too large: more than 1024 coefficients per shell"); }
  if ((size_t)b.K * b.nc * sizeof(float2) > (size_t)tp3::kPlainMaxSmem ||
      (lambda != 0.0 && ((size_t)b.K * b.nc + 32 * ((size_t)(b.n_lt() + 63) / 64 * 64 + 1)) * sizeof(float) >
                            (size_t)tp3::kPlainMaxSmem)) {
    delete c;
    return fail(nullptr, TP3_ERR_UNSUPPORTED, "K x coefficients per shell exceed the coupling kernel's shared memory");
  }
  tp3::fold_grid(b, true);
  // host-side invariants of every table before upload
  for (int t = 0; t < b.n_lt(); ++t) {
    if (b.lt_jstart[t] < 0 || b.lt_jstart[t] + b.lt_jcount[t] > b.basislen()) {
      delete c;
      return fail(nullptr, TP3_ERR_TABLE, "l-triple range outside the basis");
    }
  }
  for (int j = 0; j < b.basislen(); ++j)
    if (b.i1[j] >= b.nc || b.i2[j] >= b.nc || b.i3[j] >= b.nc || b.i1[j] < 0 || b.i2[j] < 0 || b.i3[j] < 0) {
      delete c;
      return fail(nullptr, TP3_ERR_TABLE, "coefficient index outside the compact layout");
    }
  for (int i = 0; i < b.nc; ++i)
    if (b.c_sean[i] < 0 || b.c_sean[i] >= LMAX * LMAX) {
      delete c;
      return fail(nullptr, TP3_ERR_TABLE, "seanindex outside LMAX^2");
    }

  DevTables& t = c->t;
  t.K = K; t.nc = b.nc; t.LMAX = LMAX; t.N = N;
  t.n_lt = b.n_lt();
  t.n_ltp = (t.n_lt + 63) / 64 * 64;
  t.klength = b.klength;
  t.klp = (t.klength + 127) / 128 * 128;
  t.G = b.G; t.Gu = b.Gu; t.mult = b.mult;

  std::vector<float> w32(b.basislen());
  std::vector<uint32_t> idx(b.basislen());
  for (int j = 0; j < b.basislen(); ++j) {
    w32[j] = (float)b.w[j];
    idx[j] = (uint32_t)b.i1[j] | ((uint32_t)b.i2[j] << 10) | ((uint32_t)b.i3[j] << 20);
  }
  std::vector<int2> lt(t.n_lt);
  for (int i = 0; i < t.n_lt; ++i) lt[i] = make_int2(b.lt_jstart[i], b.lt_jcount[i]);
  std::vector<int4> kl(b.klength);
  for (int i = 0; i < b.klength; ++i) kl[i] = make_int4(b.k1s[i], b.k2s[i], b.k3s[i], (int)b.tf[i]);
  // F on the full grid (plain path, lambda = 0)
  std::vector<float> Ffull;
  // lambda != 0: sphPlm(l, m, theta_k) per shell, basis entries grouped by (m2, m3) up to sign,
  // and the cosine table of those pairs on the full grid
  std::vector<float> Ytab, Cq;
  std::vector<int> lt_of_j, qstart, qlist;
  std::vector<int4> qent;  // per entry in pair order: packed shell-coefficient indices, w bits, l-triple
  if (lambda == 0.0) {
    Basis bf = b;
    tp3::fold_grid(bf, false);
    std::vector<double> F64;
    tp3::build_F(bf, F64);
    Ffull.assign((size_t)t.G * t.n_ltp, 0.f);
    for (int g = 0; g < t.G; ++g)
      for (int l = 0; l < t.n_lt; ++l) Ffull[(size_t)g * t.n_ltp + l] = (float)F64[(size_t)g * t.n_lt + l];
  } else {
    Ytab.resize((size_t)K * b.nc);
    for (int k = 0; k < K; ++k) {
      const double x = std::cos(std::acos((k + 1) * lambda * dq / (4.0 * M_PI)));  // as the reference: cos(qlist[k])
      for (int cix = 0; cix < b.nc; ++cix) Ytab[(size_t)k * b.nc + cix] = (float)tp3::sphPlm_x(b.c_l[cix], b.c_m[cix], x);
    }
    lt_of_j.resize(b.basislen());
    for (int tt = 0; tt < b.n_lt(); ++tt)
      for (int jj = 0; jj < b.lt_jcount[tt]; ++jj) lt_of_j[b.lt_jstart[tt] + jj] = tt;
    std::map<std::pair<int, int>, int> qid;
    std::vector<std::pair<int, int>> qs;
    std::vector<int> q_of_j(b.basislen());
    for (int j = 0; j < b.basislen(); ++j) {
      int m2 = b.m2[j], m3 = b.m3[j];
      if (m2 < 0 || (m2 == 0 && m3 < 0)) { m2 = -m2; m3 = -m3; }
      auto f = qid.find({m2, m3});
      if (f == qid.end()) { f = qid.emplace(std::make_pair(m2, m3), (int)qs.size()).first; qs.push_back({m2, m3}); }
      q_of_j[j] = f->second;
    }
    t.nq = (int)qs.size();
    t.nqp = (t.nq + 15) / 16 * 16;
    c->qpairs = qs;
    qstart.assign(t.nq + 1, 0);
    for (int j = 0; j < b.basislen(); ++j) qstart[q_of_j[j] + 1]++;
    for (int q = 0; q < t.nq; ++q) qstart[q + 1] += qstart[q];
    qlist.resize(b.basislen());
    std::vector<int> fillp(qstart.begin(), qstart.end() - 1);
    for (int j = 0; j < b.basislen(); ++j) qlist[fillp[q_of_j[j]]++] = j;
    qent.resize(b.basislen());
    for (int e = 0; e < b.basislen(); ++e) {
      const int j = qlist[e];
      int wb;
      std::memcpy(&wb, &w32[j], 4);
      qent[e] = make_int4((int)idx[j], wb, lt_of_j[j], 0);
    }
    Cq.assign((size_t)t.G * t.nqp, 0.f);
    for (int g = 0; g < t.G; ++g) {
      const int a = g % N, bb = g / N;
      const double al = (a + 0.5) * M_PI / N, be = (bb + 0.5) * M_PI / N;
      for (int q = 0; q < t.nq; ++q) Cq[(size_t)g * t.nqp + q] = (float)std::cos(qs[q].first * al + qs[q].second * be);
    }
  }

  cudaError_t e;
  // a blocking stream: ordered with the legacy default stream, so device buffers that a
  // caller fills there (e.g. PyTorch's default stream) are complete before the context's
  // kernels read them, and results are complete before later default-stream work
  if ((e = cudaStreamCreate(&c->own)) != cudaSuccess) {
    std::string msg = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    delete c;
    return fail(nullptr, TP3_ERR_CUDA, msg);
  }
  c->stream = c->own;
  std::vector<int> ident(b.nc);
  for (int i = 0; i < b.nc; ++i) ident[i] = i;
  if ((e = upload(c, b.c_sean, &t.csean)) != cudaSuccess || (e = upload(c, ident, &t.cident)) != cudaSuccess ||
      (e = upload(c, w32, &t.w)) != cudaSuccess ||
      (e = upload(c, idx, &t.idx)) != cudaSuccess || (e = upload(c, lt, &t.lt)) != cudaSuccess ||
      (e = upload(c, kl, &t.kl)) != cudaSuccess || (e = upload(c, b.tf, &t.tf)) != cudaSuccess ||
      (e = upload(c, Ffull, &t.Ffull)) != cudaSuccess || (e = upload(c, b.u_to_g, &t.u_to_g)) != cudaSuccess ||
      (e = upload(c, b.g_to_u, &t.g_to_u)) != cudaSuccess || (e = tp3::plain_configure()) != cudaSuccess ||
      (e = upload(c, Ytab, &t.Ytab)) != cudaSuccess || (e = upload(c, lt_of_j, &t.lt_of_j)) != cudaSuccess ||
      (e = upload(c, qstart, &t.qstart)) != cudaSuccess || (e = upload(c, qlist, &t.qlist)) != cudaSuccess ||
      (e = upload(c, qent, &t.qent)) != cudaSuccess ||
      (e = upload(c, Cq, &t.Cq)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_err, sizeof(int))) != cudaSuccess || (e = cudaMemset(c->d_err, 0, sizeof(int))) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_err, sizeof(int))) != cudaSuccess) {
    std::string msg = std::string("table upload: ") + cudaGetErrorString(e);
    tp3_ctx_destroy(c);
    return fail(nullptr, TP3_ERR_CUDA, msg);
  }
  c->tc.err = c->d_err;  // device error flag of the TP3_DEBUG index checks
  c->tc_why = setup_tc(c);
  c->tc_ok = c->tc_why.empty();
  cudaGetLastError();
  c->mode = c->tc_ok ? TP3_MODE_TC_BF16X3 : TP3_MODE_PLAIN_FP32;
  *out = c;
  return TP3_OK;
}

void tp3_ctx_destroy(tp3_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_scratch(c);
  for (void* p : c->allocs) cudaFree(p);
  cudaFree(c->d_qfull); cudaFree(c->d_Qfull); cudaFree(c->d_qt); cudaFree(c->d_Qfold); cudaFree(c->d_c3);
  cudaFree(c->d_qt_set); cudaFree(c->d_Qf_set); cudaFree(c->d_rag);
  cudaFree(c->d_err);
  cudaFreeHost(c->h_err);
  for (auto ev : c->ev) cudaEventDestroy(ev);
  for (auto ev : c->ev_c) cudaEventDestroy(ev);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

int tp3_set_stream(tp3_ctx* c, void* s) {
  if (int r = check_ctx(c)) return r;
  c->stream = s ? (cudaStream_t)s : c->own;
  return TP3_OK;
}

int tp3_set_mode(tp3_ctx* c, int mode) {
  if (int r = check_ctx(c)) return r;
  if (mode == TP3_MODE_AUTO) {
    TuneEntry te;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tuned.find(tune_key(c->b));
      if (it != g_tuned.end()) te = it->second;
    }
    if (te.mode >= 0 && (te.mode == TP3_MODE_PLAIN_FP32 || c->tc_ok)) {
      c->mode = te.mode;
      if (c->tc_ok) {
        apply_coupling(c, te.split);
        c->tc.persist = te.persist;
      }
      return TP3_OK;
    }
    mode = c->tc_ok ? TP3_MODE_TC_BF16X3 : TP3_MODE_PLAIN_FP32;
  }
  if (is_tc(mode) && !c->tc_ok) return fail(c, TP3_ERR_UNSUPPORTED, "tensor-core mode unavailable: " + c->tc_why);
  if (mode != TP3_MODE_PLAIN_FP32 && !is_tc(mode)) return fail(c, TP3_ERR_ARG, "unknown mode");
  c->mode = mode;
  return TP3_OK;
}

int tp3_autotune(tp3_ctx* c, int n, double* report, int* nreport) {
  if (int r = check_ctx(c)) return r;
  if (n < 1) return fail(c, TP3_ERR_ARG, "n must be >= 1");
  if (!c->has_hist) return fail(c, TP3_ERR_NO_HISTOGRAM, "autotune scores proposals: set a histogram first");
  const Basis& b = c->b;
  // variants: the plain path, and each tensor-core mode with each coupling form it can run
  // coupling forms: 0 one-kernel (512 threads, one CTA per SM), 1 two-kernel split,
  // 2 one-kernel small tiling (256 threads, two CTAs per SM)
  struct Var {
    int mode, form;
    bool persist;
  };
  std::vector<Var> vars = {{TP3_MODE_PLAIN_FP32, 0, true}};
  if (c->tc_ok)
    for (int m : {TP3_MODE_TC_BF16X3, TP3_MODE_TC_TF32X3}) {
      if (c->tc.fused_ok) vars.push_back({m, 0, true});
      if (c->tc.small_ok) vars.push_back({m, 2, true});
      if (c->tc.warp_ok) vars.push_back({m, 3, true});
      if (c->tc.warp2_ok) vars.push_back({m, 4, true});
      if (c->tc.split_ok) vars.push_back({m, 1, true});
      if (c->tc.fold[0].ok) vars.push_back({m, 5, true});
      if (c->tc.fold[1].ok) vars.push_back({m, 6, true});
      if (c->tc.fold[2].ok) vars.push_back({m, 7, true});
      if (c->tc.fold[3].ok) vars.push_back({m, 8, true});
    }
  // synthetic real-function coefficients (c[l,-m] = (-1)^m conj c[l,m]), n sets
  const size_t nco = (size_t)b.K * b.LMAX * b.LMAX;
  std::vector<double> h(2 * nco * n, 0.0);
  std::mt19937_64 rng(12345);
  std::normal_distribution<double> nd(0.0, 1.0);
  for (int p = 0; p < n; ++p)
    for (int k = 0; k < b.K; ++k)
      for (int l = 0; l < b.LMAX; ++l)
        for (int m = 0; m <= l; ++m) {
          double* a = &h[2 * ((size_t)p * nco + (size_t)k * b.LMAX * b.LMAX + tp3::seanindex0(l, m, b.LMAX))];
          const double sc = 1.0 / (1.0 + l + 0.2 * k);
          a[0] = nd(rng) * sc;
          a[1] = m == 0 ? 0.0 : nd(rng) * sc;
          if (m > 0) {
            double* bb = &h[2 * ((size_t)p * nco + (size_t)k * b.LMAX * b.LMAX + tp3::seanindex0(l, -m, b.LMAX))];
            const double sg = (m & 1) ? -1.0 : 1.0;
            bb[0] = sg * a[0];
            bb[1] = -sg * a[1];
          }
        }
  double2* d_c = nullptr;
  double* d_e = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&d_c, nco * n * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&d_e, n * sizeof(double))) != cudaSuccess || (e = cudaEventCreate(&e0)) != cudaSuccess ||
      (e = cudaEventCreate(&e1)) != cudaSuccess ||
      (e = cudaMemcpy(d_c, h.data(), nco * n * sizeof(double2), cudaMemcpyHostToDevice)) != cudaSuccess) {
    cudaFree(d_c); cudaFree(d_e);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return cuda_fail(c, e, "autotune setup");
  }
  const int mode0 = c->mode;
  const bool split0 = c->tc_ok ? c->tc.split : false;
  const bool small0 = c->tc_ok ? c->tc.use_small : false;
  const bool warp0 = c->tc_ok ? c->tc.use_warp : false;
  const bool warp20 = c->tc_ok ? c->tc.use_warp2 : false;
  const int fold0 = c->tc_ok ? c->tc.use_fold : -1;
  const bool persist0 = c->tc_ok ? c->tc.persist : true;
  const bool prof0 = c->prof;
  c->prof = false;
  int best = -1, rc = TP3_OK;
  double best_ms = 0.0;
  std::vector<double> ms;
  // ms per proposal of one variant (best of 3 after a warm-up), or a negative status
  auto time_var = [&](const Var& va, double& out) -> int {
    c->mode = va.mode;
    if (c->tc_ok) {
      apply_coupling(c, va.form);
      c->tc.persist = va.persist;
    }
    int r;
    if ((r = ensure_cap(c, n)) != TP3_OK) return r;
    if ((r = run_energy(c, n, d_c, d_e)) != TP3_OK) return r;  // warm-up
    double mn = 1e300;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, c->stream);
      if ((r = run_energy(c, n, d_c, d_e)) != TP3_OK) return r;
      cudaEventRecord(e1, c->stream);
      if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return cuda_fail(c, e, "autotune timing");
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      mn = std::min(mn, (double)t);
    }
    if ((r = check_device_error(c)) != TP3_OK) return r;
    out = mn / n;
    return TP3_OK;
  };
  // pass 1: every (mode, coupling form) with the persistent angular schedule
  for (size_t v = 0; v < vars.size() && rc == TP3_OK; ++v) {
    double t = -1.0;
    if ((rc = time_var(vars[v], t)) != TP3_OK) break;
    ms.push_back(t);
    if (best < 0 || t < best_ms) { best = (int)v; best_ms = t; }
  }
  // pass 2: the winner, if it is a tensor-core variant, with one CTA per angular tile
  if (rc == TP3_OK && best >= 0 && vars[best].mode != TP3_MODE_PLAIN_FP32 && c->tc.nhalf <= 2) {
    const Var alt{vars[best].mode, vars[best].form, false};
    double t = -1.0;
    if ((rc = time_var(alt, t)) == TP3_OK) {
      vars.push_back(alt);
      ms.push_back(t);
      if (t < best_ms) { best = (int)vars.size() - 1; best_ms = t; }
    }
  }
  cudaFree(d_c); cudaFree(d_e);
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  c->prof = prof0;
  if (rc != TP3_OK || best < 0) {
    c->mode = mode0;
    if (c->tc_ok) {
      c->tc.split = split0; c->tc.use_small = small0; c->tc.use_warp = warp0;
      c->tc.use_warp2 = warp20; c->tc.use_fold = fold0; c->tc.persist = persist0;
    }
    return rc != TP3_OK ? rc : fail(c, TP3_ERR_UNSUPPORTED, "no variant ran");
  }
  c->mode = vars[best].mode;
  if (c->tc_ok) {
    apply_coupling(c, vars[best].mode == TP3_MODE_PLAIN_FP32 ? 0 : vars[best].form);
    c->tc.persist = vars[best].persist;
  }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    TuneEntry te;
    te.mode = vars[best].mode;
    te.split = vars[best].form;
    te.persist = vars[best].persist;
    g_tuned[tune_key(b)] = te;
  }
  if (nreport) {
    const int cap = *nreport;
    int k = 0;
    for (size_t v = 0; v < vars.size() && k < cap; ++v, ++k) {
      if (report) {
        report[4 * k] = vars[v].mode;
        report[4 * k + 1] = vars[v].form;
        report[4 * k + 2] = vars[v].persist ? 1.0 : 0.0;
        report[4 * k + 3] = ms[v];
      }
    }
    *nreport = (int)vars.size();
  }
  return TP3_OK;
}

int tp3_set_coupling(tp3_ctx* c, int form) {
  if (int r = check_ctx(c)) return r;
  if (!c->tc_ok) return fail(c, TP3_ERR_UNSUPPORTED, "tensor-core path unavailable: " + c->tc_why);
  const bool ok = (form == 0 && c->tc.fused_ok) || (form == 1 && c->tc.split_ok) || (form == 2 && c->tc.small_ok) ||
                  (form == 3 && c->tc.warp_ok) || (form == 4 && c->tc.warp2_ok) || (form == 5 && c->tc.fold[0].ok) ||
                  (form == 6 && c->tc.fold[1].ok) || (form == 7 && c->tc.fold[2].ok) ||
                  (form == 8 && c->tc.fold[3].ok);
  if (!ok) return fail(c, form < 0 || form > 8 ? TP3_ERR_ARG : TP3_ERR_UNSUPPORTED, "coupling form not available");
  apply_coupling(c, form);
  return TP3_OK;
}

int tp3_set_angular(tp3_ctx* c, int schedule) {
  if (int r = check_ctx(c)) return r;
  if (schedule != TP3_ANGULAR_TILE && schedule != TP3_ANGULAR_PERSISTENT)
    return fail(c, TP3_ERR_ARG, "unknown angular schedule");
  if (!c->tc_ok) return fail(c, TP3_ERR_UNSUPPORTED, "tensor-core path unavailable: " + c->tc_why);
  if (schedule == TP3_ANGULAR_TILE && c->tc.nhalf > 2)
    return fail(c, TP3_ERR_UNSUPPORTED, "the per-tile angular schedule holds at most 512 grid points in TMEM");
  c->tc.persist = schedule == TP3_ANGULAR_PERSISTENT;
  return TP3_OK;
}

int tp3_get_mode(const tp3_ctx* c, int* mode) {
  if (!c || !mode) return TP3_ERR_ARG;
  *mode = c->mode;
  return TP3_OK;
}

int tp3_reserve(tp3_ctx* c, int n) {
  if (int r = check_ctx(c)) return r;
  if (n < 1) return fail(c, TP3_ERR_ARG, "n must be >= 1");
  return ensure_cap(c, n);
}

int tp3_set_histogram(tp3_ctx* c, const double* c3ref, int K3) {
  if (int r = check_ctx(c)) return r;
  if (!c3ref) return fail(c, TP3_ERR_ARG, "c3ref is NULL");
  const Basis& b = c->b;
  const DevTables& t = c->t;
  if (K3 < b.K) return fail(c, TP3_ERR_ARG, "histogram has fewer shells (K3) than the basis (K)");
  const int G = b.G;
  std::vector<float> q((size_t)b.klength * G);
  std::vector<double> Qs(b.klength), Qf(b.klength);
  std::vector<float> qt((size_t)t.klp * b.Gu, 0.f);  // [klp/128][Gu][128]
  std::vector<double> fold(b.Gu);
  for (int ki = 0; ki < b.klength; ++ki) {
    const size_t off = (size_t)G * ((size_t)b.k3s[ki] + (size_t)K3 * ((size_t)b.k2s[ki] + (size_t)K3 * b.k1s[ki]));
    const double* s = c3ref + off;
    double l1 = 0.0;
    for (int g = 0; g < G; ++g) {
      if (!std::isfinite(s[g])) return fail(c, TP3_ERR_BAD_HISTOGRAM, "histogram holds NaN or Inf");
      l1 += std::fabs(s[g]);
    }
    if (!(l1 > 0.0)) return fail(c, TP3_ERR_BAD_HISTOGRAM, "histogram slab with zero L1 norm");
    double qs = 0.0;
    std::fill(fold.begin(), fold.end(), 0.0);
    for (int g = 0; g < G; ++g) {
      const double v = s[g] / l1;
      const float vf = (float)v;
      q[(size_t)ki * G + g] = vf;
      qs += (double)vf;
      fold[b.g_to_u[g]] += v;
    }
    Qs[ki] = qs;
    double qf = 0.0;
    const int tile = ki / 128, r = ki % 128;
    for (int u = 0; u < b.Gu; ++u) {
      const float vf = (float)fold[u];
      qt[((size_t)tile * b.Gu + u) * 128 + r] = vf;
      qf += (double)vf;
    }
    Qf[ki] = qf;
  }
  cudaError_t e;
  if (!c->d_qfull) {
    if ((e = cudaMalloc(&c->d_qfull, q.size() * sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_Qfull, Qs.size() * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_qt, qt.size() * sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_Qfold, Qf.size() * sizeof(double))) != cudaSuccess)
      return cuda_fail(c, e, "cudaMalloc histogram");
  }
  if ((e = cudaMemcpyAsync(c->d_qfull, q.data(), q.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(c->d_Qfull, Qs.data(), Qs.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(c->d_qt, qt.data(), qt.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(c->d_Qfold, Qf.data(), Qf.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "histogram upload");
  c->has_hist = true;
  return TP3_OK;
}

int tp3_set_histograms(tp3_ctx* c, int nhist, const double* const* c3refs, const int* K3s, const int* Ks) {
  if (int r = check_ctx(c)) return r;
  if (nhist < 1 || !c3refs || !K3s || !Ks) return fail(c, TP3_ERR_ARG, "bad histogram set");
  const Basis& b = c->b;
  const DevTables& t = c->t;
  const size_t per = (size_t)t.klp * b.Gu;
  std::vector<float> qt(per * nhist);
  std::vector<double> Qf((size_t)b.klength * nhist);
  std::vector<int> hk(nhist);
  for (int h = 0; h < nhist; ++h) {
    if (!c3refs[h]) return fail(c, TP3_ERR_ARG, "histogram pointer is NULL");
    if (Ks[h] < 1 || Ks[h] > b.K || K3s[h] < Ks[h])
      return fail(c, TP3_ERR_ARG, "each histogram needs 1 <= K <= the basis K and K3 >= K");
    if (const char* m = fold_histogram(b, t, c3refs[h], K3s[h], Ks[h], qt.data() + per * h, Qf.data() + (size_t)b.klength * h))
      return fail(c, TP3_ERR_BAD_HISTOGRAM, m);
    hk[h] = Ks[h];
  }
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "histogram set sync");
  cudaFree(c->d_qt_set); cudaFree(c->d_Qf_set);
  c->d_qt_set = nullptr; c->d_Qf_set = nullptr; c->nhist = 0;
  int* d_hk = nullptr;
  if ((e = cudaMalloc(&c->d_qt_set, qt.size() * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_Qf_set, Qf.size() * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&d_hk, hk.size() * sizeof(int))) != cudaSuccess)
    return cuda_fail(c, e, "cudaMalloc histogram set");
  c->allocs.push_back(d_hk);
  if ((e = cudaMemcpy(c->d_qt_set, qt.data(), qt.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_Qf_set, Qf.data(), Qf.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(d_hk, hk.data(), hk.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(c, e, "histogram set upload");
  c->hist_K = hk;
  c->d_hist_K = d_hk;
  c->nhist = nhist;
  return TP3_OK;
}

int tp3_ragged_limits_device(tp3_ctx* c, int n, const int* d_lkh) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !d_lkh) return fail(c, TP3_ERR_ARG, "bad ragged limits");
  if (c->nhist == 0) return fail(c, TP3_ERR_NO_HISTOGRAM, "tp3_set_histograms has not been called");
  cudaError_t e;
  if (n > c->rag_cap) {
    cudaFree(c->d_rag);
    c->d_rag = nullptr;
    c->rag_cap = 0;
    if ((e = cudaMalloc(&c->d_rag, (size_t)n * sizeof(tp3::RagInfo))) != cudaSuccess)
      return cuda_fail(c, e, "cudaMalloc ragged limits");
    c->rag_cap = n;
    c->scratch_gen++;
  }
  k_rag_info<<<(n + 127) / 128, 128, 0, c->stream>>>(d_lkh, n, c->b.L, c->b.K, c->nhist, c->d_hist_K, c->d_rag,
                                                      c->d_err);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, e, "ragged limits");
  return TP3_OK;
}

int tp3_energy_batch_ragged_device(tp3_ctx* c, int n, const void* d_coeffs, const int* d_lkh, void* d_E) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !d_coeffs || !d_E) return fail(c, TP3_ERR_ARG, "bad batch arguments");
  if (int r = ensure_cap(c, n)) return r;
  if (int r = tp3_ragged_limits_device(c, n, d_lkh)) return r;
  return run_energy(c, n, (const double2*)d_coeffs, (double*)d_E, false, c->d_rag);
}

int tp3_c3(tp3_ctx* c, const double* coeff, float* out) {
  if (int r = check_ctx(c)) return r;
  if (!coeff || !out) return fail(c, TP3_ERR_ARG, "NULL pointer");
  if (int r = ensure_cap(c, 1)) return r;
  const auto& t = c->t;
  const size_t nco = (size_t)t.K * t.LMAX * t.LMAX;
  cudaError_t e;
  if (!c->d_c3 && (e = cudaMalloc(&c->d_c3, (size_t)t.klength * t.G * sizeof(float))) != cudaSuccess)
    return cuda_fail(c, e, "cudaMalloc c3");
  std::memcpy(c->h_coeff, coeff, nco * 2 * sizeof(double));
  if ((e = cudaMemcpyAsync(c->d_coeff, c->h_coeff, nco * sizeof(double2), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "H2D coeff");
  if (int r = run_coupling(c, 1, c->d_coeff, false)) return r;
  if (is_tc(c->mode))
    e = tp3::launch_angular_tc(t, c->tc, c->mode == TP3_MODE_TC_TF32X3 ? c->maps32 : c->maps, 1, nullptr, nullptr,
                               nullptr, c->d_c3, c->d_err, c->mode == TP3_MODE_TC_TF32X3, c->stream);
  else
    e = tp3::launch_angular_plain(t, 1, plain_A(c), nullptr, nullptr, tp3::plain_ncg(t), c->d_c3, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "angular store");
  // device layout [ki][g] is the column-major G x klength layout of the reference
  if ((e = cudaMemcpyAsync(out, c->d_c3, (size_t)t.klength * t.G * sizeof(float), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "D2H c3");
  return check_device_error(c);
}

int tp3_c3_batch_device(tp3_ctx* c, int n, const void* d_coeffs, void* d_c3) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !d_coeffs || !d_c3) return fail(c, TP3_ERR_ARG, "bad batch arguments");
  if (int r = ensure_cap(c, n)) return r;
  const auto& t = c->t;
  cudaError_t e;
  if (int r = run_coupling(c, n, (const double2*)d_coeffs, false)) return r;
  if (is_tc(c->mode))
    e = tp3::launch_angular_tc(t, c->tc, c->mode == TP3_MODE_TC_TF32X3 ? c->maps32 : c->maps, n, nullptr, nullptr,
                               nullptr, (float*)d_c3, c->d_err, c->mode == TP3_MODE_TC_TF32X3, c->stream);
  else
    e = tp3::launch_angular_plain(t, n, plain_A(c), nullptr, nullptr, tp3::plain_ncg(t), (float*)d_c3, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "angular store");
  return TP3_OK;
}

int tp3_triple_products(tp3_ctx* c, const double* coeff, float* out) {
  if (int r = check_ctx(c)) return r;
  if (!coeff || !out) return fail(c, TP3_ERR_ARG, "NULL pointer");
  if (int r = ensure_cap(c, 1)) return r;
  const auto& t = c->t;
  const size_t nco = (size_t)t.K * t.LMAX * t.LMAX;
  cudaError_t e;
  std::memcpy(c->h_coeff, coeff, nco * 2 * sizeof(double));
  if ((e = cudaMemcpyAsync(c->d_coeff, c->h_coeff, nco * sizeof(double2), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "H2D coeff");
  if (int r = run_coupling(c, 1, c->d_coeff, true)) return r;
  if ((e = cudaMemcpy2DAsync(out, t.n_lt * sizeof(float), c->d_T, t.n_ltp * sizeof(float), t.n_lt * sizeof(float),
                             t.klength, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "D2H T");
  return TP3_OK;
}

int tp3_energy_batch(tp3_ctx* c, int n, const double* coeffs, double* E) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !coeffs || !E) return fail(c, TP3_ERR_ARG, "bad batch arguments");
  if (int r = ensure_cap(c, n)) return r;
  const auto& t = c->t;
  const Basis& b = c->b;
  const size_t ncoef = (size_t)t.LMAX * t.LMAX;
  // Only the even-l <= L block of each shell reaches the kernels: pack it on the host
  // (3.3x fewer bytes at L=18, LMAX=25) with all host threads, then one copy and one
  // launch sequence for the whole batch; very large batches go in chunks so that packing
  // chunk i+1 overlaps the copy and kernels of chunk i.
  const int nchunk = n >= 1024 ? 4 : 1;
  const int per = (n + nchunk - 1) / nchunk;
  const double2* src = (const double2*)coeffs;
  double2* pin = (double2*)c->h_coeff;
  double2* dev = c->d_coeff;
  cudaError_t e;
  if (c->host_direct) {
    // the device reads the caller's buffer in place: no host packing and no staging copy
    const int64_t total = (int64_t)n * t.K * t.nc;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 65535);
    k_stage_coeff<<<blocks, 256, 0, c->stream>>>(src, total, t.nc, (int)ncoef, t.csean, dev);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, e, "stage coefficients");
    if (int r = run_energy(c, n, dev, c->d_E, true)) return r;
  }
  for (int p0 = 0; p0 < n && !c->host_direct; p0 += per) {
    const int m = std::min(per, n - p0);
    // host threads pack the proposals of a chunk (the previous chunk's kernels run meanwhile)
#pragma omp parallel for schedule(static) if (m >= 8)
    for (int p = p0; p < p0 + m; ++p)
      for (int k = 0; k < t.K; ++k) {
        const double2* s = src + ((size_t)p * t.K + k) * ncoef;
        double2* d = pin + ((size_t)p * t.K + k) * t.nc;
        for (int i = 0; i < t.nc; ++i) d[i] = s[b.c_sean[i]];
      }
    const size_t off = (size_t)p0 * t.K * t.nc;
    if ((e = cudaMemcpyAsync(dev + off, pin + off, (size_t)m * t.K * t.nc * sizeof(double2), cudaMemcpyHostToDevice,
                             c->stream)) != cudaSuccess)
      return cuda_fail(c, e, "H2D coeff");
    if (int r = run_energy(c, m, dev + off, c->d_E + p0, true)) return r;
  }
  if ((e = cudaMemcpyAsync(c->h_E, c->d_E, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "D2H energy");
  if (int r = check_device_error(c)) return r;
  std::memcpy(E, c->h_E, n * sizeof(double));
  return TP3_OK;
}

int tp3_energy(tp3_ctx* c, const double* coeff, double* E) { return tp3_energy_batch(c, 1, coeff, E); }

int tp3_set_host_input(tp3_ctx* c, int mode) {
  if (int r = check_ctx(c)) return r;
  if (mode != TP3_HOST_INPUT_STAGED && mode != TP3_HOST_INPUT_DIRECT) return fail(c, TP3_ERR_ARG, "unknown host input mode");
  if (mode == TP3_HOST_INPUT_DIRECT && !c->pageable_ok)
    return fail(c, TP3_ERR_UNSUPPORTED, "the device cannot read pageable host memory");
  c->host_direct = mode == TP3_HOST_INPUT_DIRECT;
  return TP3_OK;
}

int tp3_energy_batch_device(tp3_ctx* c, int n, const void* d_coeffs, void* d_E) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !d_coeffs || !d_E) return fail(c, TP3_ERR_ARG, "bad batch arguments");
  if (int r = ensure_cap(c, n)) return r;
  return run_energy(c, n, (const double2*)d_coeffs, (double*)d_E);
}

int tp3_sync(tp3_ctx* c) {
  if (int r = check_ctx(c)) return r;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "stream synchronize");
  return check_device_error(c);
}

int tp3_profile_enable(tp3_ctx* c, int on) {
  if (int r = check_ctx(c)) return r;
  c->prof = on != 0;
  c->ev_used = 0;
  c->ev_c_used = 0;
  return TP3_OK;
}

int tp3_profile_read_stage(tp3_ctx* c, int stage, int64_t* launches, double* total_ms) {
  if (int r = check_ctx(c)) return r;
  if (!launches || !total_ms) return fail(c, TP3_ERR_ARG, "NULL pointer");
  if (stage != 0 && stage != 1) return fail(c, TP3_ERR_ARG, "stage must be 0 (angular) or 1 (coupling)");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "profile sync");
  std::vector<cudaEvent_t>& ev = stage == 0 ? c->ev : c->ev_c;
  size_t& used = stage == 0 ? c->ev_used : c->ev_c_used;
  double ms = 0.0;
  for (size_t i = 0; i + 1 < used; i += 2) {
    float f = 0.f;
    if (cudaEventElapsedTime(&f, ev[i], ev[i + 1]) == cudaSuccess) ms += f;
  }
  *launches = (int64_t)(used / 2);
  *total_ms = ms;
  used = 0;
  return TP3_OK;
}

int tp3_profile_read(tp3_ctx* c, int64_t* launches, double* total_ms) {
  return tp3_profile_read_stage(c, 0, launches, total_ms);
}

}  // extern "C"
