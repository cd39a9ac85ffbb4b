// Wigner-D rotations of spherical-harmonic coefficients (src/spherical_harmonics.jl:572-603):
// the host matrix rotationMatrix(theta, phi, gamma, l) and the device rotation of every
// shell of many coefficient sets by its own SO(3) element.  Formulas: shellrot.cuh.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "ctx_internal.h"
#include "shellrot.cuh"

namespace {

// grid: n * K blocks (one shell of one coefficient set); block 32 * warps.
// Rotates orders l = lstart, lstart + lstep, ..., <= lend of shell (set, k) by
// exp([v]x), v = axis_angle[set][k][0..2]; every other coefficient is copied.
__global__ void __launch_bounds__(128) k_rotate_shells(const double2* in, double2* out,
                                                       const double* __restrict__ axis_angle, int K, int LMAX,
                                                       int lstart, int lstep, int lend,
                                                       const double* __restrict__ delta,
                                                       const int* __restrict__ doff) {
  __shared__ double2 xs[4][2 * tp3::kMaxRotL + 1], ys[4][2 * tp3::kMaxRotL + 1];
  __shared__ double euler[3];
  const int ncoef = LMAX * LMAX;
  const size_t base = (size_t)blockIdx.x * ncoef;
  const double2* c = in + base;
  double2* o = out + base;
  if (threadIdx.x == 0) {
    const double* v = axis_angle + (size_t)blockIdx.x * 3;
    tp3::axis_angle_euler(v[0], v[1], v[2], euler[0], euler[1], euler[2]);
  }
  if (c != o)
    for (int e = threadIdx.x; e < ncoef; e += blockDim.x) o[e] = c[e];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const double th = euler[0], ph = euler[1], ga = euler[2];
  // largest orders first so the warps finish together
  const int nord = (lend - lstart) / lstep + 1;
  for (int j = warp; j < nord; j += nw) {
    const int l = lend - ((lend - lstart) % lstep) - j * lstep;
    tp3::rotate_order_warp(c, o, l, LMAX, th, ph, ga, delta + doff[l], xs[warp], ys[warp], lane);
  }
}

}  // namespace

namespace tp3 {

int ctx_ensure_rot_tables(tp3_ctx* c, int lmax) {
  if (lmax <= c->rot_lmax) return TP3_OK;
  if (lmax > kMaxRotL) return ctx_fail(c, TP3_ERR_UNSUPPORTED, "rotations need l <= 62");
  std::vector<int> off(lmax + 2, 0);
  for (int l = 0; l <= lmax; ++l) off[l + 1] = off[l] + (2 * l + 1) * (2 * l + 1);
  std::vector<double> del(off[lmax + 1]);
  for (int l = 0; l <= lmax; ++l) {
    const int d = 2 * l + 1;
    for (int m = -l; m <= l; ++m)
      for (int k = -l; k <= l; ++k) del[off[l] + (m + l) * d + (k + l)] = wigner_d_half_pi(l, m, k);
  }
  double* dd = nullptr;
  int* doff = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&dd, del.size() * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&doff, (lmax + 1) * sizeof(int))) != cudaSuccess) {
    cudaFree(dd);
    return ctx_cuda_fail(c, e, "rotation tables");
  }
  c->allocs.push_back(dd);
  c->allocs.push_back(doff);
  if ((e = cudaMemcpy(dd, del.data(), del.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(doff, off.data(), (lmax + 1) * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
    return ctx_cuda_fail(c, e, "rotation tables upload");
  c->d_delta = dd;
  c->d_doff = doff;
  c->rot_lmax = lmax;
  return TP3_OK;
}

cudaError_t launch_rotate_shells(tp3_ctx* c, int n, const double2* in, double2* out, const double* axis_angle,
                                 int lstart, int lstep, int lend) {
  k_rotate_shells<<<n * c->b.K, 128, 0, c->stream>>>(in, out, axis_angle, c->b.K, c->b.LMAX, lstart, lstep, lend,
                                                     c->d_delta, c->d_doff);
  return cudaGetLastError();
}

}  // namespace tp3

extern "C" {

int tp3_wigner_D(int l, double theta, double phi, double gamma, double* out) {
  if (l < 0 || l > tp3::kMaxRotL || !out) return TP3_ERR_ARG;
  const int d = 2 * l + 1;
  std::vector<double> del((size_t)d * d);
  for (int m = -l; m <= l; ++m)
    for (int k = -l; k <= l; ++k) del[(size_t)(m + l) * d + (k + l)] = tp3::wigner_d_half_pi(l, m, k);
  for (int m = -l; m <= l; ++m) {
    for (int s = -l; s <= l; ++s) {
      // d_ms(theta) = i^(m-s) sum_k Delta[m][k] Delta[s][k] e^{ik theta}, which is real:
      // the sum of Delta[m][k] Delta[s][k] cos(k theta + (m - s) pi/2)
      long double acc = 0.0L;
      for (int k = -l; k <= l; ++k)
        acc += (long double)del[(size_t)(m + l) * d + (k + l)] * del[(size_t)(s + l) * d + (k + l)] *
               cosl((long double)k * theta + (long double)(m - s) * 1.5707963267948966192313216916397514L);
      const double dms = (double)acc;
      const double ang = -(double)s * gamma - (double)m * phi;
      double* o = out + 2 * ((size_t)(m + l) + (size_t)d * (s + l));  // column-major [m, s]
      o[0] = dms * std::cos(ang);
      o[1] = dms * std::sin(ang);
    }
  }
  return TP3_OK;
}

int tp3_rotate_shells_device(tp3_ctx* c, int n, const void* d_coeffs, const void* d_axis_angle, void* d_out) {
  if (int r = tp3::ctx_check(c)) return r;
  if (n < 1 || !d_coeffs || !d_axis_angle || !d_out) return tp3::ctx_fail(c, TP3_ERR_ARG, "bad rotation arguments");
  const int lend = c->b.LMAX - 1;
  if (int r = tp3::ctx_ensure_rot_tables(c, lend)) return r;
  cudaError_t e = tp3::launch_rotate_shells(c, n, (const double2*)d_coeffs, (double2*)d_out,
                                            (const double*)d_axis_angle, 0, 1, lend);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "rotate shells");
  return TP3_OK;
}

}  // extern "C"
