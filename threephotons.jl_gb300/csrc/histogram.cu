// Triplet histogram of photon pictures on the device: the all-to-all binning of
// histogramCorrelationsInPicture_alltoall (src/datagen.jl:228-277), the step before the
// hot path (it makes the c3ref histogram the energy is scored against).
//
// Per picture: photons with k = round(|p| / dq) in 1..K2 (round half to even, as
// Julia's round) are kept and sorted by |p| ascending; for every i, c1[k1] gets one
// count; for every j < i, alpha = angle_between(p_i, p_j) in [0, 2 pi) (the
// reference's utilities.jl:61-72, including its 0 for exactly perpendicular vectors),
// folded to [0, pi], gives the c2 bin ai; for every k < j with k1, k2, k3 <= K3,
// beta = angle_between(p_i, p_k), mirrored to 2 pi - beta when alpha > pi, gives the c3
// bin bi in 0..2N-1.  The reference adds the weights 1/k1, 1/(doubletFactor k1 k2) and
// 1/(tripletFactor k1 k2 k3) per entry; here every bin counts its entries exactly
// (64-bit integer atomics) and the weights, which depend only on the bin's shells,
// are applied once when the counts are read out.
//
// Arithmetic mirrors the reference's evaluation order (products and sums rounded
// separately, no fused multiply-add), so bins agree with an FP64 CPU evaluation.
//
// Pictures themselves come from k_sample_pictures, the role of pointsPerOrientation
// (src/datagen.jl:88-144) for an intensity given by its SH coefficients: per picture a
// Haar-random orientation R; incident photons p ~ N(0, sigma^2) on the detector
// (z = 0); each with |p| <= qcut is mapped to the Ewald sphere (detector_to_Ewald_sphere,
// src/datagen.jl:33-39), rotated, and kept with probability
//     I(R e(p)) / (I_max / g(0) g(R e(p))),  g = 3-D Gaussian of width sigma,
// i.e. photons are drawn proportionally to the intensity.  I(q) is the SH synthesis
// sum_lm c_lm(k) Y_lm on the shells, linear in |q| between shells.  Random numbers:
// Philox4x32-10 keyed by the seed, counter (picture, photon, purpose).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "ctx_internal.h"

namespace {

constexpr int kMaxPhotons = 1536;  // photons per picture after the k filter (43 KB of shared memory)
constexpr int kBinThreads = 256;
constexpr int kMaxIncident = 1 << 24;  // incident photons of one picture

__device__ inline double angle_between(double x1, double y1, double x2, double y2, double n1, double n2) {
  const double dot = __dadd_rn(__dmul_rn(x1, x2), __dmul_rn(y1, y2));
  double val = dot / __dmul_rn(n1, n2);
  val = fmin(fmax(val, -1.0), 1.0);
  if (fabs(val) > 0.0) {
    double a = acos(val);
    const double cz = __dsub_rn(__dmul_rn(x1, y2), __dmul_rn(y1, x2));
    if (cz > 0.0) a = 2.0 * 3.141592653589793 - a;
    return a;
  }
  return 0.0;
}

// grid: pictures; block kBinThreads.  photons [total][2] (x, y), offsets [n + 1].
__global__ void __launch_bounds__(kBinThreads) k_bin_pictures(const double2* __restrict__ photons,
                                                              const long long* __restrict__ offsets,
                                                              long long n_photons, double dq, int N,
                                                              int K2, int K3, unsigned long long* __restrict__ c1,
                                                              unsigned long long* __restrict__ c2,
                                                              unsigned long long* __restrict__ c3, int* __restrict__ err) {
  __shared__ double sx[kMaxPhotons], sy[kMaxPhotons], sn[kMaxPhotons];
  __shared__ int sk[kMaxPhotons];
  __shared__ int s_count;
  const long long o0 = offsets[blockIdx.x], o1 = offsets[blockIdx.x + 1];
  if (o0 < 0 || o1 < o0 || o1 > n_photons) {  // offsets outside the photon array: report, skip
    if (threadIdx.x == 0) atomicExch(err, TP3_ERR_ARG);
    return;
  }
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  // keep photons with 1 <= k <= K2
  for (long long p = o0 + threadIdx.x; p < o1; p += blockDim.x) {
    const double2 v = photons[p];
    const double n = sqrt(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)));
    const int k = (int)rint(n / dq);
    if (k >= 1 && k <= K2) {
      const int slot = atomicAdd(&s_count, 1);
      if (slot < kMaxPhotons) {
        sx[slot] = v.x; sy[slot] = v.y; sn[slot] = n; sk[slot] = k;
      }
    }
  }
  __syncthreads();
  const int l = s_count;
  if (l > kMaxPhotons) {
    if (threadIdx.x == 0) atomicExch(err, TP3_ERR_ARG);
    return;
  }
  if (l < 3) return;  // the reference skips pictures of fewer than three photons
  // sort by norm ascending: odd-even transposition over the l kept photons
  for (int pass = 0; pass < l; ++pass) {
    for (int i = 2 * threadIdx.x + (pass & 1); i + 1 < l; i += 2 * blockDim.x) {
      if (sn[i] > sn[i + 1]) {
        double t = sn[i]; sn[i] = sn[i + 1]; sn[i + 1] = t;
        t = sx[i]; sx[i] = sx[i + 1]; sx[i + 1] = t;
        t = sy[i]; sy[i] = sy[i + 1]; sy[i + 1] = t;
        const int tk = sk[i]; sk[i] = sk[i + 1]; sk[i + 1] = tk;
      }
    }
    __syncthreads();
  }
  const double da = 3.141592653589793 / N;
  for (int i = threadIdx.x; i < l; i += blockDim.x) atomicAdd(&c1[sk[i] - 1], 1ull);
  // pairs (i, j < i), then triplets (i, j, k < j)
  const long long npairs = (long long)l * (l - 1) / 2;
  for (long long P = threadIdx.x; P < npairs; P += blockDim.x) {
    int i = (int)((1.0 + sqrt(1.0 + 8.0 * (double)P)) * 0.5);
    while ((long long)i * (i - 1) / 2 > P) --i;
    while ((long long)(i + 1) * i / 2 <= P) ++i;
    const int j = (int)(P - (long long)i * (i - 1) / 2);
    const int k1 = sk[i], k2 = sk[j];
    const double alpha = angle_between(sx[i], sy[i], sx[j], sy[j], sn[i], sn[j]);
    const double alpha_s = alpha > 3.141592653589793 ? 2.0 * 3.141592653589793 - alpha : alpha;
    int ai = (int)floor(alpha_s / da) % N;
    if (ai < 0) ai += N;
    atomicAdd(&c2[(size_t)ai + (size_t)N * ((size_t)(k2 - 1) + (size_t)K2 * (k1 - 1))], 1ull);
    if (k1 > K3 || k2 > K3) continue;
    for (int k = 0; k < j; ++k) {
      const int k3 = sk[k];
      if (k3 > K3) continue;
      double beta = angle_between(sx[i], sy[i], sx[k], sy[k], sn[i], sn[k]);
      if (alpha > 3.141592653589793) beta = 2.0 * 3.141592653589793 - beta;
      int bi = (int)floor(beta / da) % (2 * N);
      if (bi < 0) bi += 2 * N;
      const size_t idx = (size_t)ai + (size_t)N * ((size_t)bi + (size_t)(2 * N) *
                                                   ((size_t)(k3 - 1) + (size_t)K3 * ((size_t)(k2 - 1) + (size_t)K3 * (k1 - 1))));
      atomicAdd(&c3[idx], 1ull);
    }
  }
}

__host__ __device__ inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ inline double u01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }

__device__ inline void normal4(uint64_t seed, uint32_t a, uint32_t b, uint32_t purpose, double z[4]) {
  uint32_t c[4] = {a, b, purpose, 0u};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  for (int h = 0; h < 2; ++h) {
    const double r = sqrt(-2.0 * log(u01(c[2 * h])));
    double sn, cs;
    sincos(6.283185307179586 * u01(c[2 * h + 1]), &sn, &cs);
    z[2 * h] = r * cs;
    z[2 * h + 1] = r * sn;
  }
}

// I(r) from SH coefficients coeff[KMAX][LMAX^2] (seanindex order) of shells q_k = k dq,
// k = 1..KMAX, linear in |r| between shells (below shell 1: shell 1; above KMAX: KMAX).
// Real function: I = sum_l sum_{m >= 0} (2 - delta_m0) Re(c_lm e^{i m phi}) P_lm(cos theta).
__device__ inline double intensity_at(const double2* __restrict__ coeff, int KMAX, int LMAX, double dq, double x,
                                      double y, double z) {
  const double q = sqrt(x * x + y * y + z * z);
  double t = q / dq;
  int k0 = (int)floor(t);
  double w = t - k0;
  if (k0 < 1) { k0 = 1; w = 0.0; }
  if (k0 >= KMAX) { k0 = KMAX; w = 0.0; }
  const int k1 = k0 < KMAX ? k0 + 1 : k0;
  const double ct = q > 0.0 ? z / q : 1.0;
  const double st = sqrt(fmax(0.0, (1.0 - ct) * (1.0 + ct)));
  const double ph = atan2(y, x);
  const double2* ca = coeff + (size_t)(k0 - 1) * LMAX * LMAX;
  const double2* cb = coeff + (size_t)(k1 - 1) * LMAX * LMAX;
  const int bigL = LMAX - 1;
  double acc = 0.0;
  double pmm = 0.28209479177387814;  // 1 / sqrt(4 pi)
  for (int m = 0; m < LMAX; ++m) {
    if (m > 0) pmm *= -st * sqrt((2.0 * m + 1.0) / (2.0 * m));
    double sn, cs;
    sincos((double)m * ph, &sn, &cs);
    const double fac = m == 0 ? 1.0 : 2.0;
    double p2 = 0.0, p1 = pmm;
    for (int l = m; l < LMAX; ++l) {
      double pl;
      if (l == m) pl = pmm;
      else if (l == m + 1) pl = ct * sqrt(2.0 * m + 3.0) * pmm;
      else pl = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m)) *
                (ct * p1 - sqrt((((double)l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * ((double)l - 1.0) * (l - 1.0) - 1.0)) * p2);
      if (l > m) { p2 = p1; p1 = pl; }
      const int idx = m * (bigL + 1) - (m * (m - 1)) / 2 + (l - m);
      const double2 a = ca[idx], b = cb[idx];
      const double re = (1.0 - w) * a.x + w * b.x, im = (1.0 - w) * a.y + w * b.y;
      acc += fac * (re * cs - im * sn) * pl;
    }
  }
  return acc;
}

// grid: pictures; block 256.  Accepted photons go to out[pic][0 .. counts[pic]) ((x, y)).
// incident_var > 0: the picture's incident photons are round(N(incident, incident_var))
// (>= 0, <= kMaxIncident) instead of `incident` (src/datagen.jl:93-97).  beamstop > 0:
// incident photons with |x| <= beamstop or |y| <= beamstop are dropped
// (src/datagen.jl:111-113).  stream selects independent photon draws for the same
// pictures (the same orientation R): 0 for the molecule, 1 for noise photons
// (src/datagen.jl:403-405 samples the noise with the molecule's rotation).
__global__ void __launch_bounds__(256) k_sample_pictures(const double2* __restrict__ coeff, int KMAX, int LMAX,
                                                         double dq, double qcut, double sigma, int incident,
                                                         int incident_var, double beamstop, int stream,
                                                         double lambda, double Imax, uint64_t seed, int max_out,
                                                         double2* __restrict__ out, int* __restrict__ counts,
                                                         long long pic0) {
  __shared__ double R[9];
  __shared__ int s_n, s_incident;
  const long long pic = pic0 + blockIdx.x;
  const uint32_t pur = 16u * (uint32_t)stream;  // purposes of this stream's photon draws
  if (threadIdx.x == 0) {
    // Haar rotation from a uniform unit quaternion
    double z[4];
    normal4(seed, (uint32_t)pic, 0xFFFFFFFFu, 7u, z);
    const double nq = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2] + z[3] * z[3]);
    const double a = z[0] / nq, b = z[1] / nq, c = z[2] / nq, d = z[3] / nq;
    R[0] = a * a + b * b - c * c - d * d; R[1] = 2 * (b * c - a * d);         R[2] = 2 * (b * d + a * c);
    R[3] = 2 * (b * c + a * d);         R[4] = a * a - b * b + c * c - d * d; R[5] = 2 * (c * d - a * b);
    R[6] = 2 * (b * d - a * c);         R[7] = 2 * (c * d + a * b);         R[8] = a * a - b * b - c * c + d * d;
    s_n = 0;
    int n = incident;
    if (incident_var > 0) {
      double zc[4];
      normal4(seed, (uint32_t)pic, 0xFFFFFFFEu, 10u + pur, zc);
      const double v = rint((double)incident + (double)incident_var * zc[0]);
      n = v < 0.0 ? 0 : (v > (double)kMaxIncident ? kMaxIncident : (int)v);
    }
    s_incident = n;
  }
  __syncthreads();
  const double inv2s2 = 0.5 / (sigma * sigma);
  const int n_inc = s_incident;
  for (int i = threadIdx.x; i < n_inc; i += blockDim.x) {
    double z[4];
    normal4(seed, (uint32_t)pic, (uint32_t)i, 8u + pur, z);
    const double px = sigma * z[0], py = sigma * z[1];
    if (beamstop > 0.0 && !(fabs(px) > beamstop && fabs(py) > beamstop)) continue;
    const double qn = sqrt(px * px + py * py);
    if (qn > qcut) continue;
    // detector_to_Ewald_sphere: theta = acos(q lambda / 4 pi), (sin(theta) p, cos(theta) q)
    const double th = acos(qn * lambda / (4.0 * 3.141592653589793));
    const double ex = sin(th) * px, ey = sin(th) * py, ez = cos(th) * qn;
    const double rx = R[0] * ex + R[1] * ey + R[2] * ez;
    const double ry = R[3] * ex + R[4] * ey + R[5] * ez;
    const double rz = R[6] * ex + R[7] * ey + R[8] * ez;
    const double I = intensity_at(coeff, KMAX, LMAX, dq, rx, ry, rz);
    const double r2 = rx * rx + ry * ry + rz * rz;
    const double ratio = I / Imax * exp(r2 * inv2s2);
    uint32_t c[4] = {(uint32_t)pic, (uint32_t)i, 9u + pur, 0u};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    if (u01(c[0]) < ratio) {
      const int slot = atomicAdd(&s_n, 1);
      if (slot < max_out) out[(size_t)blockIdx.x * max_out + slot] = make_double2(px, py);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = min(s_n, max_out);
}

// grid: ceil(n / 256); block 256.  Max of I over a shells x n_theta x n_phi grid (per-block maxima).
__global__ void k_intensity_grid_max(const double2* __restrict__ coeff, int KMAX, int LMAX, double dq, int nth,
                                     int nph, double* __restrict__ bmax) {
  __shared__ double red[256];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)KMAX * nth * nph;
  double v = -1e300;
  if (i < n) {
    const int k = (int)(i / ((long long)nth * nph)) + 1;
    const int rem = (int)(i % ((long long)nth * nph));
    const int it = rem / nph, ip = rem % nph;
    const double th = (it + 0.5) * 3.141592653589793 / nth, ph = (ip + 0.5) * 6.283185307179586 / nph;
    const double q = k * dq;
    v = intensity_at(coeff, KMAX, LMAX, dq, q * sin(th) * cos(ph), q * sin(th) * sin(ph), q * cos(th));
  }
  red[threadIdx.x] = v;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) bmax[blockIdx.x] = red[0];
}

}  // namespace

extern "C" {

int tp3_histogram_pictures(tp3_ctx* c, int n_pictures, const void* d_photons, int64_t n_photons,
                           const int64_t* d_offsets, double dq, int N, int K2, int K3, unsigned long long* d_c1,
                           unsigned long long* d_c2, unsigned long long* d_c3) {
  if (int r = tp3::ctx_check(c)) return r;
  if (n_pictures < 1 || !d_photons || n_photons < 0 || !d_offsets || !d_c1 || !d_c2 || !d_c3 || !(dq > 0.0) ||
      N < 1 || K2 < 1 || K3 < 1 || K3 > K2)
    return tp3::ctx_fail(c, TP3_ERR_ARG, "bad histogram arguments");
  k_bin_pictures<<<n_pictures, kBinThreads, 0, c->stream>>>((const double2*)d_photons, (const long long*)d_offsets,
                                                           (long long)n_photons, dq, N, K2, K3, d_c1, d_c2, d_c3,
                                                           c->d_err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "histogram pictures");
  return TP3_OK;
}

int tp3_sample_pictures_ex(tp3_ctx* c, int n_pictures, int64_t first_picture, const void* d_coeff, int KMAX,
                           int LMAX, double dq, double qcut, double envelope_sigma, int incident_photons,
                           int incident_photon_variance, double beamstop_width, int stream, double lambda,
                           double max_intensity, uint64_t seed, int max_out, void* d_photons, int* d_counts) {
  if (int r = tp3::ctx_check(c)) return r;
  if (n_pictures < 1 || !d_coeff || !d_photons || !d_counts || KMAX < 1 || LMAX < 1 || !(dq > 0.0) ||
      !(qcut > 0.0) || !(envelope_sigma > 0.0) || incident_photons < 0 || incident_photons > kMaxIncident ||
      incident_photon_variance < 0 || !(beamstop_width >= 0.0) || stream < 0 || stream > 15 ||
      !(max_intensity > 0.0) || max_out < 1 || !(lambda >= 0.0) || qcut * lambda > 4.0 * 3.141592653589793)
    return tp3::ctx_fail(c, TP3_ERR_ARG, "bad sampling arguments");
  k_sample_pictures<<<n_pictures, 256, 0, c->stream>>>((const double2*)d_coeff, KMAX, LMAX, dq, qcut, envelope_sigma,
                                                       incident_photons, incident_photon_variance, beamstop_width,
                                                       stream, lambda, max_intensity, seed, max_out,
                                                       (double2*)d_photons, d_counts, (long long)first_picture);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "sample pictures");
  return TP3_OK;
}

int tp3_sample_pictures(tp3_ctx* c, int n_pictures, int64_t first_picture, const void* d_coeff, int KMAX, int LMAX,
                        double dq, double qcut, double envelope_sigma, int incident_photons, double lambda,
                        double max_intensity, uint64_t seed, int max_out, void* d_photons, int* d_counts) {
  return tp3_sample_pictures_ex(c, n_pictures, first_picture, d_coeff, KMAX, LMAX, dq, qcut, envelope_sigma,
                                incident_photons, 0, 0.0, 0, lambda, max_intensity, seed, max_out, d_photons,
                                d_counts);
}

int tp3_intensity_max(tp3_ctx* c, const void* d_coeff, int KMAX, int LMAX, double dq, int n_theta, int n_phi,
                      double* out) {
  if (int r = tp3::ctx_check(c)) return r;
  if (!d_coeff || !out || KMAX < 1 || LMAX < 1 || n_theta < 1 || n_phi < 1 || !(dq > 0.0))
    return tp3::ctx_fail(c, TP3_ERR_ARG, "bad arguments");
  const long long n = (long long)KMAX * n_theta * n_phi;
  const int nb = (int)((n + 255) / 256);
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, nb * sizeof(double));
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "intensity max scratch");
  k_intensity_grid_max<<<nb, 256, 0, c->stream>>>((const double2*)d_coeff, KMAX, LMAX, dq, n_theta, n_phi, d);
  std::vector<double> h(nb);
  if ((e = cudaGetLastError()) == cudaSuccess &&
      (e = cudaMemcpyAsync(h.data(), d, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream)) == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "intensity max");
  double m = -1e300;
  for (double v : h) m = v > m ? v : m;
  *out = m;
  return TP3_OK;
}

}  // extern "C"
