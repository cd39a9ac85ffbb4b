// Internal declarations shared by the context code and the kernel files.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace tp3 {

// Device view of the per-context tables (all pointers are device memory).
struct DevTables {
  int K, nc, LMAX;
  int n_lt, n_ltp;      // l-triples, padded count (row stride of T and F)
  int klength, klp;     // shell triples, padded to the TC row tile
  int G, Gu, mult, N;
  const int* csean;     // [nc] compact -> seanindex0
  const float* w;       // [basislen]
  const uint32_t* idx;  // [basislen] i1 | i2 << 10 | i3 << 20
  const int2* lt;       // [n_lt] (jstart, jcount)
  const int4* kl;       // [klength] (k1, k2, k3, tf)
  const double* tf;     // [klength]
  const float* Ffull;   // [G][n_ltp]  fp32, full grid (plain path)
  const int* u_to_g;    // [Gu]
  const int* g_to_u;    // [G]
};

// Plain path launches (kernels_plain.cu).
cudaError_t launch_gather(const DevTables& t, int n, const double2* coeff, float2* cc, cudaStream_t s);
cudaError_t launch_couple_direct(const DevTables& t, int n, const float2* cc, float* T, cudaStream_t s);
// Bayes partials: part[prop][cg][klength] (Sp, Sql); ncg column groups over the full grid.
cudaError_t launch_angular_plain(const DevTables& t, int n, const float* T, const float* q,
                                 double2* part, int ncg, float* c3out, cudaStream_t s);
cudaError_t launch_finalize(const DevTables& t, int n, const double2* part, int ncg,
                            const double* Qs, int mult, double* E, cudaStream_t s);

int plain_ncg(const DevTables& t);
// Per-device kernel attributes of the plain path (call with the device current).
cudaError_t plain_configure();
constexpr int kPlainMaxSmem = 200 * 1024;

}  // namespace tp3
