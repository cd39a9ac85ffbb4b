// Context and C ABI of libtp3 (declared in include/tp3.h).
//
// A context owns every device buffer of one (L, LMAX, N, K, lambda) basis: the
// tables built once by tables.cpp, the normalised histogram, and scratch sized
// for the largest batch seen (or reserved).  Nothing is allocated per call once
// the scratch fits; no call falls back to the CPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tp3.h"
#include "internal.h"
#include "tables.h"

using tp3::Basis;
using tp3::DevTables;

namespace {

thread_local std::string g_create_error;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct tp3_ctx {
  Basis b;
  DevTables t{};
  int device = 0;
  int mode = TP3_MODE_PLAIN_FP32;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<void*> allocs;  // table allocations, freed at destroy

  // histogram
  bool has_hist = false;
  float* d_qfull = nullptr;    // [klength][G]
  double* d_Qfull = nullptr;   // [klength]

  // scratch (sized for cap proposals)
  int cap = 0;
  double2* d_coeff = nullptr;  // [cap][K][LMAX^2]
  float2* d_cc = nullptr;      // [cap][K][nc]
  float* d_T = nullptr;        // [cap][klp][n_ltp]
  double2* d_part = nullptr;   // [cap][ncg][klength]
  double* d_E = nullptr;       // [cap]
  float* d_c3 = nullptr;       // [klength][G] (one proposal)
  double* h_coeff = nullptr;   // pinned [cap][K][LMAX^2][2]
  double* h_E = nullptr;       // pinned [cap]

  // profiling of the angular + Bayes kernel
  bool prof = false;
  std::vector<cudaEvent_t> ev;  // pairs
  size_t ev_used = 0;
};

namespace {

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

void free_scratch(tp3_ctx* c) {
  cudaFree(c->d_coeff); cudaFree(c->d_cc); cudaFree(c->d_T); cudaFree(c->d_part); cudaFree(c->d_E);
  cudaFreeHost(c->h_coeff); cudaFreeHost(c->h_E);
  c->d_coeff = nullptr; c->d_cc = nullptr; c->d_T = nullptr; c->d_part = nullptr; c->d_E = nullptr;
  c->h_coeff = nullptr; c->h_E = nullptr;
  c->cap = 0;
}

int ensure_cap(tp3_ctx* c, int n) {
  if (n <= c->cap) return TP3_OK;
  free_scratch(c);
  const auto& t = c->t;
  const int ncg = tp3::plain_ncg(t);
  const size_t ncoef = (size_t)t.LMAX * t.LMAX;
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_coeff, (size_t)n * t.K * ncoef * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_cc, (size_t)n * t.K * t.nc * sizeof(float2))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_T, (size_t)n * t.klp * t.n_ltp * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_part, (size_t)n * ncg * t.klength * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_E, (size_t)n * sizeof(double))) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_coeff, (size_t)n * t.K * ncoef * 2 * sizeof(double))) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_E, (size_t)n * sizeof(double))) != cudaSuccess) {
    free_scratch(c);
    cudaGetLastError();
    return fail(c, TP3_ERR_ALLOC, std::string("scratch allocation: ") + cudaGetErrorString(e));
  }
  // padding rows/columns of T stay zero for the lifetime of the buffer
  if ((e = cudaMemset(c->d_T, 0, (size_t)n * t.klp * t.n_ltp * sizeof(float))) != cudaSuccess)
    return cuda_fail(c, e, "cudaMemset T");
  c->cap = n;
  return TP3_OK;
}

int prof_begin(tp3_ctx* c, cudaEvent_t* a, cudaEvent_t* b) {
  if (!c->prof) return 0;
  if (c->ev_used + 2 > c->ev.size()) {
    cudaEvent_t e1, e2;
    if (cudaEventCreate(&e1) != cudaSuccess || cudaEventCreate(&e2) != cudaSuccess) return 0;
    c->ev.push_back(e1);
    c->ev.push_back(e2);
  }
  *a = c->ev[c->ev_used];
  *b = c->ev[c->ev_used + 1];
  c->ev_used += 2;
  cudaEventRecord(*a, c->stream);
  return 1;
}

// Score n proposals whose FP64 coefficients are already in d_coeff (device).
int run_energy(tp3_ctx* c, int n, const double2* d_coeff, double* d_E) {
  const auto& t = c->t;
  cudaError_t e;
  if (!c->has_hist) return fail(c, TP3_ERR_NO_HISTOGRAM, "tp3_set_histogram has not been called");
  if ((e = tp3::launch_gather(t, n, d_coeff, c->d_cc, c->stream)) != cudaSuccess) return cuda_fail(c, e, "gather");
  if ((e = tp3::launch_couple_direct(t, n, c->d_cc, c->d_T, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "couple_direct");
  const int ncg = tp3::plain_ncg(t);
  cudaEvent_t a, b;
  int pr = prof_begin(c, &a, &b);
  if ((e = tp3::launch_angular_plain(t, n, c->d_T, c->d_qfull, c->d_part, ncg, nullptr, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "angular_plain");
  if (pr) cudaEventRecord(b, c->stream);
  if ((e = tp3::launch_finalize(t, n, c->d_part, ncg, c->d_Qfull, 1, d_E, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "finalize");
  return TP3_OK;
}

int check_ctx(tp3_ctx* c) {
  if (!c) return TP3_ERR_ARG;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  return TP3_OK;
}

}  // namespace

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
    default: return "unknown status";
  }
}

const char* tp3_last_error(const tp3_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int tp3_version(void) { return (1 << 16) | 0; }

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
  std::string m = tp3::build_basis(c->b, L, LMAX, N, K, lambda, dq);
  if (!m.empty()) { delete c; return fail(nullptr, TP3_ERR_ARG, m); }
  Basis& b = c->b;
  if (lambda != 0.0) {
    delete c;
    return fail(nullptr, TP3_ERR_UNSUPPORTED, "lambda != 0 (Ewald curvature) is not supported by this build");
  }
  if (b.nc > 1024) { delete c; return fail(nullptr, TP3_ERR_UNSUPPORTED, "L too large: more than 1024 coefficients per shell"); }
  if ((size_t)b.K * b.nc * sizeof(float2) > (size_t)tp3::kPlainMaxSmem) {
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
  // F on the full grid (plain path)
  Basis bf = b;
  tp3::fold_grid(bf, false);
  std::vector<double> F64;
  tp3::build_F(bf, F64);
  std::vector<float> Ffull((size_t)t.G * t.n_ltp, 0.f);
  for (int g = 0; g < t.G; ++g)
    for (int l = 0; l < t.n_lt; ++l) Ffull[(size_t)g * t.n_ltp + l] = (float)F64[(size_t)g * t.n_lt + l];

  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess) {
    std::string msg = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    delete c;
    return fail(nullptr, TP3_ERR_CUDA, msg);
  }
  c->stream = c->own;
  if ((e = upload(c, b.c_sean, &t.csean)) != cudaSuccess || (e = upload(c, w32, &t.w)) != cudaSuccess ||
      (e = upload(c, idx, &t.idx)) != cudaSuccess || (e = upload(c, lt, &t.lt)) != cudaSuccess ||
      (e = upload(c, kl, &t.kl)) != cudaSuccess || (e = upload(c, b.tf, &t.tf)) != cudaSuccess ||
      (e = upload(c, Ffull, &t.Ffull)) != cudaSuccess || (e = upload(c, b.u_to_g, &t.u_to_g)) != cudaSuccess ||
      (e = upload(c, b.g_to_u, &t.g_to_u)) != cudaSuccess || (e = tp3::plain_configure()) != cudaSuccess) {
    std::string msg = std::string("table upload: ") + cudaGetErrorString(e);
    tp3_ctx_destroy(c);
    return fail(nullptr, TP3_ERR_CUDA, msg);
  }
  *out = c;
  return TP3_OK;
}

void tp3_ctx_destroy(tp3_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_scratch(c);
  for (void* p : c->allocs) cudaFree(p);
  cudaFree(c->d_qfull); cudaFree(c->d_Qfull); cudaFree(c->d_c3);
  for (auto ev : c->ev) cudaEventDestroy(ev);
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
  if (mode == TP3_MODE_AUTO) mode = TP3_MODE_PLAIN_FP32;
  if (mode != TP3_MODE_PLAIN_FP32) return fail(c, TP3_ERR_UNSUPPORTED, "mode not available in this build");
  c->mode = mode;
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
  if (K3 < b.K) return fail(c, TP3_ERR_ARG, "histogram has fewer shells (K3) than the basis (K)");
  const int N = b.N, G = b.G;
  const size_t slab = (size_t)G;
  std::vector<float> q((size_t)b.klength * G);
  std::vector<double> Qs(b.klength);
  for (int ki = 0; ki < b.klength; ++ki) {
    const size_t off = slab * ((size_t)b.k3s[ki] + (size_t)K3 * ((size_t)b.k2s[ki] + (size_t)K3 * b.k1s[ki]));
    const double* s = c3ref + off;
    double l1 = 0.0;
    for (int g = 0; g < G; ++g) {
      if (!std::isfinite(s[g])) return fail(c, TP3_ERR_BAD_HISTOGRAM, "histogram holds NaN or Inf");
      l1 += std::fabs(s[g]);
    }
    if (!(l1 > 0.0)) return fail(c, TP3_ERR_BAD_HISTOGRAM, "histogram slab with zero L1 norm");
    double qs = 0.0;
    for (int g = 0; g < G; ++g) {
      float v = (float)(s[g] / l1);
      q[(size_t)ki * G + g] = v;
      qs += (double)v;
    }
    Qs[ki] = qs;
  }
  (void)N;
  cudaError_t e;
  if (!c->d_qfull) {
    if ((e = cudaMalloc(&c->d_qfull, q.size() * sizeof(float))) != cudaSuccess) return cuda_fail(c, e, "cudaMalloc q");
    if ((e = cudaMalloc(&c->d_Qfull, Qs.size() * sizeof(double))) != cudaSuccess) return cuda_fail(c, e, "cudaMalloc Qs");
  }
  if ((e = cudaMemcpyAsync(c->d_qfull, q.data(), q.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(c->d_Qfull, Qs.data(), Qs.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "histogram upload");
  c->has_hist = true;
  return TP3_OK;
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
  if ((e = tp3::launch_gather(t, 1, c->d_coeff, c->d_cc, c->stream)) != cudaSuccess) return cuda_fail(c, e, "gather");
  if ((e = tp3::launch_couple_direct(t, 1, c->d_cc, c->d_T, c->stream)) != cudaSuccess) return cuda_fail(c, e, "couple");
  if ((e = tp3::launch_angular_plain(t, 1, c->d_T, nullptr, nullptr, tp3::plain_ncg(t), c->d_c3, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "angular store");
  // device layout [ki][g] is the column-major G x klength layout of the reference
  if ((e = cudaMemcpyAsync(out, c->d_c3, (size_t)t.klength * t.G * sizeof(float), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "D2H c3");
  return TP3_OK;
}

int tp3_energy_batch(tp3_ctx* c, int n, const double* coeffs, double* E) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !coeffs || !E) return fail(c, TP3_ERR_ARG, "bad batch arguments");
  if (int r = ensure_cap(c, n)) return r;
  const auto& t = c->t;
  const size_t nco = (size_t)n * t.K * t.LMAX * t.LMAX;
  std::memcpy(c->h_coeff, coeffs, nco * 2 * sizeof(double));
  cudaError_t e;
  if ((e = cudaMemcpyAsync(c->d_coeff, c->h_coeff, nco * sizeof(double2), cudaMemcpyHostToDevice, c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "H2D coeff");
  if (int r = run_energy(c, n, c->d_coeff, c->d_E)) return r;
  if ((e = cudaMemcpyAsync(c->h_E, c->d_E, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return cuda_fail(c, e, "D2H energy");
  std::memcpy(E, c->h_E, n * sizeof(double));
  return TP3_OK;
}

int tp3_energy(tp3_ctx* c, const double* coeff, double* E) { return tp3_energy_batch(c, 1, coeff, E); }

int tp3_energy_batch_device(tp3_ctx* c, int n, const void* d_coeffs, void* d_E) {
  if (int r = check_ctx(c)) return r;
  if (n < 1 || !d_coeffs || !d_E) return fail(c, TP3_ERR_ARG, "bad batch arguments");
  if (int r = ensure_cap(c, n)) return r;
  return run_energy(c, n, (const double2*)d_coeffs, (double*)d_E);
}

int tp3_profile_enable(tp3_ctx* c, int on) {
  if (int r = check_ctx(c)) return r;
  c->prof = on != 0;
  c->ev_used = 0;
  return TP3_OK;
}

int tp3_profile_read(tp3_ctx* c, int64_t* launches, double* total_ms) {
  if (int r = check_ctx(c)) return r;
  if (!launches || !total_ms) return fail(c, TP3_ERR_ARG, "NULL pointer");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "profile sync");
  double ms = 0.0;
  for (size_t i = 0; i + 1 < c->ev_used; i += 2) {
    float f = 0.f;
    if (cudaEventElapsedTime(&f, c->ev[i], c->ev[i + 1]) == cudaSuccess) ms += f;
  }
  *launches = (int64_t)(c->ev_used / 2);
  *total_ms = ms;
  c->ev_used = 0;
  return TP3_OK;
}

}  // extern "C"
