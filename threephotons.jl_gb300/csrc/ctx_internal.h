// Definition of the library context, shared by the C ABI files (ctx.cu, chains.cu).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/tp3.h"
#include "internal.h"
#include "tables.h"

namespace tp3 {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
}  // namespace tp3


struct tp3_ctx {
  tp3::Basis b;
  tp3::DevTables t{};
  tp3::TcTables tc{};
  bool tc_ok = false;
  std::string tc_why;
  int device = 0;
  int mode = TP3_MODE_PLAIN_FP32;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<void*> allocs;  // table allocations, freed at destroy
  tp3::EncodeTiledFn encode = nullptr;
  tp3::TcMaps maps{};    // bf16 operands
  tp3::TcMaps maps32{};  // tf32 operands
  std::vector<std::pair<int, int>> qpairs;  // lambda != 0: the Fourier pairs (m2, m3) of H's columns

  // histogram
  bool has_hist = false;
  float* d_qfull = nullptr;    // [klength][G]
  double* d_Qfull = nullptr;   // [klength]
  float* d_qt = nullptr;       // [klp/128][Gu][128] folded, tiled for the TMEM epilogue
  double* d_Qfold = nullptr;   // [klength]

  // scratch (sized for cap proposals)
  int cap = 0;
  int scratch_gen = 0;         // incremented whenever the scratch below is reallocated
  int t_elem = 2;              // bytes per element of the T operand buffers (2 bf16, 4 tf32)
  double2* d_coeff = nullptr;  // [cap][K][LMAX^2]
  float2* d_cc = nullptr;      // [cap][K][nc]
  float* d_T = nullptr;        // [cap][klp][n_ltp]      plain path
  double2* d_part = nullptr;   // [cap][ncg][klength]    plain path
  __nv_bfloat16* d_Thi = nullptr;  // [cap][klp][KP]    tensor-core path
  __nv_bfloat16* d_Tlo = nullptr;
  double* d_Eslab = nullptr;   // [cap][klength]         tensor-core path
  double* d_E = nullptr;       // [cap]
  float* d_c3 = nullptr;       // [klength][G] (one proposal)
  int* d_err = nullptr;        // device error flag (timeouts)
  int* d_sym = nullptr;        // [cap] real-function symmetry flag per proposal
  float2* d_D = nullptr;       // [dsub][dstride] pair-coupled D of the split coupling
  float* d_H = nullptr;        // [cap][klp][nqp] Fourier-pair operand (lambda != 0)
  double* h_coeff = nullptr;   // pinned [cap][K][LMAX^2][2]
  double* h_E = nullptr;       // pinned [cap]
  int* h_err = nullptr;        // pinned

  // histogram set of ragged batches: [nhist][klp/128][Gu][128] and [nhist][klength]
  int nhist = 0;
  float* d_qt_set = nullptr;
  double* d_Qf_set = nullptr;
  std::vector<int> hist_K;          // shells of each histogram of the set
  int* d_hist_K = nullptr;
  tp3::RagInfo* d_rag = nullptr;    // [cap] per-proposal limits of the current ragged batch
  int rag_cap = 0;

  // Wigner-D tables: Delta^l = d^l(pi/2) row-major for l = 0..rot_lmax, at d_doff[l]
  int rot_lmax = -1;
  double* d_delta = nullptr;
  int* d_doff = nullptr;

  // profiling: event pairs around each launch of the angular + Bayes kernel (ev) and
  // of the coupling kernel of the tensor-core path (ev_c)
  bool prof = false;
  bool pageable_ok = false;    // the device reads pageable host memory through the host page tables
  bool host_direct = false;    // tp3_energy_batch reads the caller's buffer in place
  std::vector<cudaEvent_t> ev;  // pairs
  size_t ev_used = 0;
  std::vector<cudaEvent_t> ev_c;
  size_t ev_c_used = 0;
};


namespace tp3 {
// Helpers of ctx.cu used by the other C ABI files.
int ctx_fail(tp3_ctx* c, int code, const std::string& msg);
int ctx_cuda_fail(tp3_ctx* c, cudaError_t e, const char* where);
int ctx_check(tp3_ctx* c);
int ctx_ensure_cap(tp3_ctx* c, int n);
// Score n proposals whose FP64 seanindex-ordered coefficients are in device memory
// (rag: per-proposal limits of a ragged batch, device; null for the whole shape).
int ctx_run_energy(tp3_ctx* c, int n, const double2* d_coeff, double* d_E, const RagInfo* rag = nullptr);
int ctx_check_device_error(tp3_ctx* c);
// Per-proposal RagInfo from (L, K, histogram) triples (device), validated on the device.
int ctx_make_rag(tp3_ctx* c, int n, const int* d_lkh, RagInfo* out);
// Upload the Wigner-D tables for orders 0..lmax once (shellrot.cu).
int ctx_ensure_rot_tables(tp3_ctx* c, int lmax);
// Proposal network hooks (mlp.cu): its input buffer (rows of mlp_n_in_pad bf16),
// the raw [rows][kMlpOutPad] outputs of a forward pass over rows [0, R).
__nv_bfloat16* mlp_input(tp3_mlp* n);
int mlp_max_rows(const tp3_mlp* n);
int mlp_n_in_of(const tp3_mlp* n);
int mlp_forward_raw(tp3_mlp* n, int R, const float** out);
}  // namespace tp3
