// Structure -> spherical-harmonic coefficients on the device, FP64: the role of
// createSphericalHarmonicsStructure (src/structure.jl:125-134), the step that turns a
// molecule into the intensity coefficients the hot path scores, for many molecules
// at once.
//
// Surfaces are sampled on the reference's grid (getSurface / i_to_ang,
// src/spherical_harmonics.jl:203-210, 228-235: size = 2 LMAX, sample
// itheta * size + iphi at phi = 2 pi iphi / size, theta = pi (2 itheta + 1) / (2 size))
// and transformed with the semantics of the s2kit forward / inverse transforms the
// reference calls with bandwidth LMAX (transform / backtransform,
// src/spherical_harmonics.jl:127-148; src/sh/s2kit_interface.c:72-178):
//   c(l, m) = sum_theta w_theta Ptilde_l^|m|(cos theta) s_m F_m(theta),
//   F_m(theta) = sqrt(2 pi) / size sum_phi f(theta, phi) e^{-i m phi},
// with the Driscoll-Healy weights w, Legendre functions normalised to unit L2 norm on
// [-1, 1] with the Condon-Shortley phase, and s_m = (-1)^|m| for m < 0 (1 otherwise);
// the inverse is the exact synthesis sum c(l, m) Y_lm on the same grid.  Sums are
// direct (no FFT): size (2 LMAX - 1) terms per Fourier value, size per coefficient.
//
// Routes:
//   TP3_SH_INTENSITY: intensity shells |F(q)|^2 of Gaussian atoms (getIntensity_cartesian,
//     src/structure.jl:89-102) at q_k = k pi / rmax (the reference's intensityShell).
//   TP3_SH_REFERENCE: density shells at r_k = k rmax / KMAX (getDensity_cartesian,
//     src/structure.jl:72-86, atoms cut at |x - a|^2 < 5) -> forward transform ->
//     spherical Bessel transform (sphBesselTransform with frdr and the J_{l+1/2} matrices,
//     src/spherical_harmonics.jl:291-347) -> inverse transform, |.|^2, forward transform
//     (absoluteSquare, src/spherical_harmonics.jl:376-381).
//
// The same grid and synthesis serve the post-processing fit, fitStructures_random
// (src/data_processing.jl:51-75): random-restart search over rotations of a structure
// onto a reference, scored by similarity = the mean over K_range of the per-shell Pearson
// correlation of the two intensities on the synthesis grid (shell_correlation_ISC,
// similarity, src/spherical_harmonics.jl:398-435).  All repetitions advance in lockstep:
// per step one kernel rotates the K_range shells of every repetition's proposal (orders
// 2:2:L, rotateStructure), one synthesises their surfaces and one correlates them with
// the reference's, and the host keeps each repetition's state and accept decisions.
//
// retrieveSolution (src/correlations.jl:261-319), the start structure from a two-photon
// correlation c2: one thread per shell pair fits the pair's c2 slice (symmetrised in
// alpha at lambda = 0) by least squares against (1/4pi) P_l(cos alpha*), l = 0:2:upperL
// (normal equations, Cholesky, FP64), giving G_l[k1, k2]; one warp per order l runs cyclic
// Jacobi on G_l (K2 x K2, rotations' row and column updates across the lanes); the host
// keeps the top 2l+1 eigenpairs (each eigenvector's largest entry made positive), forms
// sqrt(w) v^T in the real SH basis, maps it to complex coefficients with Umat(l)^* and
// negates the result when negativityCheck (src/spherical_harmonics.jl:622-625) on the
// synthesis grid exceeds 0.33.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "ctx_internal.h"
#include "shellrot.cuh"

namespace {

constexpr int kShMaxLMAX = 48;  // Fourier table of one surface: 2 LMAX x (2 LMAX - 1) complex in shared memory
constexpr double kPi = 3.141592653589793;

// grid: (ceil(P / 256), KMAX, n_mol); block 256.  atoms [n][5] = x, y, z, R, B.
__global__ void __launch_bounds__(256) k_sh_sample(const double* __restrict__ atoms, const int* __restrict__ mol_start,
                                                   int size, int KMAX, double rmax, int density,
                                                   double2* __restrict__ out) {
  const int P = size * size;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y + 1, mol = blockIdx.z;
  if (p >= P) return;
  const int it = p / size, ip = p - it * size;
  const double phi = 2.0 * kPi * ip / size;
  const double theta = kPi * (2 * it + 1) / (2.0 * size);
  const double st = sin(theta);
  const double ux = cos(phi) * st, uy = sin(phi) * st, uz = cos(theta);
  const int a0 = mol_start[mol], a1 = mol_start[mol + 1];
  double v;
  if (density) {
    const double r = k * (rmax / KMAX);
    const double x = r * ux, y = r * uy, z = r * uz;
    v = 0.0;
    for (int a = a0; a < a1; ++a) {
      const double* at = atoms + 5 * (size_t)a;
      const double dx = x - at[0], dy = y - at[1], dz = z - at[2];
      const double d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < 5.0) {
        const double R = at[3], s = R * sqrt(2.0 * kPi);
        v += at[4] / (s * s * s) * exp(-d2 / (2.0 * R * R));
      }
    }
  } else {
    const double q = k * kPi / rmax;
    const double x = q * ux, y = q * uy, z = q * uz;
    double sc = 0.0, ss = 0.0;
    for (int a = a0; a < a1; ++a) {
      const double* at = atoms + 5 * (size_t)a;
      const double f = at[4] * exp(-0.5 * at[3] * at[3] * q * q);
      double sn, cs;
      sincos(x * at[0] + y * at[1] + z * at[2], &sn, &cs);
      sc += f * cs;
      ss += f * sn;
    }
    v = sc * sc + ss * ss;
  }
  out[((size_t)mol * KMAX + (k - 1)) * P + p] = make_double2(v, 0.0);
}

// grid: surfaces; block 256; dynamic shared memory size (2 bw - 1) double2.
// Forward transform of complex samples [surface][size^2] into [surface][bw^2] (seanindex).
// plm [l][m][theta] (0 <= m <= l < bw), w [theta], root [size] = e^{2 pi i j / size},
// lm [bw^2] = (l, m) of each seanindex slot.
__global__ void __launch_bounds__(256) k_sht_forward(const double2* __restrict__ in, int bw,
                                                     const double* __restrict__ plm, const double* __restrict__ w,
                                                     const double2* __restrict__ root, const int2* __restrict__ lm,
                                                     double2* __restrict__ out) {
  extern __shared__ double2 sF[];  // [theta][m + bw - 1]
  const int size = 2 * bw, nm = 2 * bw - 1;
  const double2* f = in + (size_t)blockIdx.x * size * size;
  const double sc = sqrt(2.0 * kPi) / size;
  for (int i = threadIdx.x; i < size * nm; i += blockDim.x) {
    const int t = i / nm, m = i - t * nm - (bw - 1);
    double re = 0.0, im = 0.0;
    const int mm = ((m % size) + size) % size;
    for (int j = 0; j < size; ++j) {
      const double2 v = f[t * size + j];
      const double2 e = root[(size - (mm * j) % size) % size];  // e^{-i m phi_j}
      re += v.x * e.x - v.y * e.y;
      im += v.x * e.y + v.y * e.x;
    }
    sF[i] = make_double2(re * sc, im * sc);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < bw * bw; i += blockDim.x) {
    const int2 q = lm[i];
    const int l = q.x, m = q.y, ma = m < 0 ? -m : m;
    const double* pl = plm + ((size_t)l * bw + ma) * size;
    double re = 0.0, im = 0.0;
    for (int t = 0; t < size; ++t) {
      const double c = w[t] * pl[t];
      const double2 v = sF[t * nm + m + bw - 1];
      re += c * v.x;
      im += c * v.y;
    }
    if (m < 0 && (ma & 1)) re = -re, im = -im;
    out[(size_t)blockIdx.x * bw * bw + i] = make_double2(re, im);
  }
}

// grid: surfaces; block 256; dynamic shared memory size (2 bw - 1) double2.
// Synthesis sum_lm c(l, m) Y_lm on the grid, Y_lm = Ptilde_l^|m| s_m e^{i m phi} / sqrt(2 pi).
// idx [m + bw - 1][l] = seanindex slot of (l, m) (read only for l >= |m|).
__global__ void __launch_bounds__(256) k_sht_inverse(const double2* __restrict__ in, int bw,
                                                     const double* __restrict__ plm, const double2* __restrict__ root,
                                                     const int* __restrict__ idx, double2* __restrict__ out) {
  extern __shared__ double2 sG[];  // [theta][m + bw - 1]
  const int size = 2 * bw, nm = 2 * bw - 1;
  const double2* c = in + (size_t)blockIdx.x * bw * bw;
  const double isq = 1.0 / sqrt(2.0 * kPi);
  for (int i = threadIdx.x; i < size * nm; i += blockDim.x) {
    const int t = i / nm, mi = i - t * nm, m = mi - (bw - 1), ma = m < 0 ? -m : m;
    double re = 0.0, im = 0.0;
    for (int l = ma; l < bw; ++l) {
      const double p = plm[((size_t)l * bw + ma) * size + t];
      const double2 v = c[idx[mi * bw + l]];
      re += p * v.x;
      im += p * v.y;
    }
    const double s = (m < 0 && (ma & 1)) ? -isq : isq;
    sG[i] = make_double2(re * s, im * s);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < size * size; i += blockDim.x) {
    const int t = i / size, j = i - t * size;
    double re = 0.0, im = 0.0;
    for (int mi = 0; mi < nm; ++mi) {
      const int m = mi - (bw - 1);
      const int mm = ((m % size) + size) % size;
      const double2 e = root[(mm * j) % size];  // e^{+i m phi_j}
      const double2 v = sG[t * nm + mi];
      re += v.x * e.x - v.y * e.y;
      im += v.x * e.y + v.y * e.x;
    }
    out[(size_t)blockIdx.x * size * size + i] = make_double2(re, im);
  }
}

// In place: |f|^2 of every sample (the square of absoluteSquare).
__global__ void k_abs2(double2* __restrict__ f, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double2 v = f[i];
    f[i] = make_double2(v.x * v.x + v.y * v.y, 0.0);
  }
}

// grid: (ceil(bw^2 / 128), KMAX, n_mol); block 128.  Forward spherical Bessel transform
// along the shells of every coefficient: out[k'] = i^l sqrt(1/k') sum_k J[l][k'][k] h[k] in[k].
__global__ void __launch_bounds__(128) k_sh_hankel(const double2* __restrict__ in, int bw, int KMAX,
                                                   const double* __restrict__ J, const double* __restrict__ h,
                                                   const int2* __restrict__ lm, double2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int kp = blockIdx.y, mol = blockIdx.z;
  const int nco = bw * bw;
  if (i >= nco) return;
  const int l = lm[i].x;
  const double* Jr = J + ((size_t)l * KMAX + kp) * KMAX;
  const double2* src = in + (size_t)mol * KMAX * nco + i;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < KMAX; ++k) {
    const double2 v = src[(size_t)k * nco];
    const double c = Jr[k] * h[k];
    re += c * v.x;
    im += c * v.y;
  }
  const double s = sqrt(1.0 / (kp + 1));
  re *= s;
  im *= s;
  double2 o;
  switch (l & 3) {  // multiply by i^l
    case 0: o = make_double2(re, im); break;
    case 1: o = make_double2(-im, re); break;
    case 2: o = make_double2(-re, -im); break;
    default: o = make_double2(im, -re); break;
  }
  out[((size_t)mol * KMAX + kp) * nco + i] = o;
}

// grid: (nsets * nk); block 128.  Set r, shell j: copy the volume's shell k0 + j to
// out[r][j] and rotate its orders 2, 4, ..., lend by the set's Euler angles (theta, phi,
// gamma) -- rotationMatrix convention -- when rotate is set.
__global__ void __launch_bounds__(128) k_fit_rotate(const double2* __restrict__ vol, double2* __restrict__ out,
                                                    const double* __restrict__ euler, int k0, int nk, int LMAX,
                                                    int lend, int nrot, const double* __restrict__ delta,
                                                    const int* __restrict__ doff) {
  __shared__ double2 xs[4][2 * tp3::kMaxRotL + 1], ys[4][2 * tp3::kMaxRotL + 1];
  const int ncoef = LMAX * LMAX;
  const int set = blockIdx.x / nk, j = blockIdx.x - set * nk;
  const double2* c = vol + (size_t)(k0 + j) * ncoef;
  double2* o = out + (size_t)blockIdx.x * ncoef;
  for (int e = threadIdx.x; e < ncoef; e += blockDim.x) o[e] = c[e];
  __syncthreads();
  if (j >= nrot) return;
  const double th = euler[3 * set], ph = euler[3 * set + 1], ga = euler[3 * set + 2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nord = lend / 2;  // orders 2 .. lend (even)
  for (int i = warp; i < nord; i += nw) {
    const int l = lend - 2 * i;  // largest orders first
    tp3::rotate_order_warp(o, o, l, LMAX, th, ph, ga, delta + doff[l], xs[warp], ys[warp], lane);
  }
}

// grid: nsets * nk; block 256.  Pearson correlation of the real parts of surface
// (set, j) and reference surface j over the P grid points (two passes, FP64).
__global__ void __launch_bounds__(256) k_fit_corr(const double2* __restrict__ surf, const double2* __restrict__ ref,
                                                  int nk, int P, double* __restrict__ corr) {
  __shared__ double sa[256], sb[256], sc[256];
  const int j = blockIdx.x % nk;
  const double2* a = surf + (size_t)blockIdx.x * P;
  const double2* b = ref + (size_t)j * P;
  double ma = 0.0, mb = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    ma += a[i].x;
    mb += b[i].x;
  }
  sa[threadIdx.x] = ma;
  sb[threadIdx.x] = mb;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      sa[threadIdx.x] += sa[threadIdx.x + h];
      sb[threadIdx.x] += sb[threadIdx.x + h];
    }
    __syncthreads();
  }
  ma = sa[0] / P;
  mb = sb[0] / P;
  __syncthreads();
  double sab = 0.0, saa = 0.0, sbb = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const double x = a[i].x - ma, y = b[i].x - mb;
    sab += x * y;
    saa += x * x;
    sbb += y * y;
  }
  sa[threadIdx.x] = sab;
  sb[threadIdx.x] = saa;
  sc[threadIdx.x] = sbb;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      sa[threadIdx.x] += sa[threadIdx.x + h];
      sb[threadIdx.x] += sb[threadIdx.x + h];
      sc[threadIdx.x] += sc[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) corr[blockIdx.x] = sa[0] / sqrt(sb[0] * sc[0]);
}

// P_l(x), the Legendre polynomial by its three-term recurrence.
__device__ inline double rs_legendre(int l, double x) {
  double p0 = 1.0, p1 = x;
  if (l == 0) return p0;
  for (int n = 1; n < l; ++n) {
    const double p2 = ((2.0 * n + 1.0) * x * p1 - n * p0) / (n + 1.0);
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// One thread per shell pair (k1 >= k2 of lo..hi): least-squares coefficients of the c2
// slice c2[alpha][k2 - 1][k1 - 1] (c2 is [N][Kd][Kd]) on (1/4pi) P_{2j}(cos alpha*),
// j = 0..upperL/2, written to G[j][k1 - lo][k2 - lo] and its mirror (G zeroed before).
__global__ void k_rs_fit(const double* __restrict__ c2, int N, int Kd, int lo, int hi, int L, double dq,
                         double lambda, double* __restrict__ G) {
  const int n = hi - lo + 1;
  const int pair = blockIdx.x * blockDim.x + threadIdx.x;
  if (pair >= n * (n + 1) / 2) return;
  int a1 = 0;
  while ((a1 + 1) * (a1 + 2) / 2 <= pair) ++a1;
  const int a2 = pair - a1 * (a1 + 1) / 2;  // a2 <= a1
  const int k1 = lo + a1, k2 = lo + a2;
  const int upperL = min(L, 2 * min(k1, k2) - 2);
  const int J = upperL / 2 + 1;
  constexpr int kMaxJ = 32;
  if (J > kMaxJ) return;
  double M[kMaxJ * (kMaxJ + 1) / 2], r[kMaxJ], p[kMaxJ];
  for (int i = 0; i < J * (J + 1) / 2; ++i) M[i] = 0.0;
  for (int i = 0; i < J; ++i) r[i] = 0.0;
  const double t1 = acos(k1 * dq * lambda / (4.0 * kPi)), t2 = acos(k2 * dq * lambda / (4.0 * kPi));
  const double s12 = sin(t1) * sin(t2), c12 = cos(t1) * cos(t2);
  for (int a = 0; a < N; ++a) {
    double sl = c2[((size_t)a * Kd + (k2 - 1)) * Kd + (k1 - 1)];
    if (lambda == 0.0) sl = 0.5 * (sl + c2[((size_t)(N - 1 - a) * Kd + (k2 - 1)) * Kd + (k1 - 1)]);
    const double al = (a + 0.5) * (kPi / N);
    const double x = cos(acos(fmin(fmax(s12 * cos(al) + c12, -1.0), 1.0)));
    for (int j = 0; j < J; ++j) p[j] = rs_legendre(2 * j, x) / (4.0 * kPi);
    for (int i = 0; i < J; ++i) {
      r[i] += p[i] * sl;
      for (int j = 0; j <= i; ++j) M[i * (i + 1) / 2 + j] += p[i] * p[j];
    }
  }
  // Cholesky M = C C^T in place (lower triangle), then forward and back substitution
  for (int i = 0; i < J; ++i) {
    for (int j = 0; j <= i; ++j) {
      double v = M[i * (i + 1) / 2 + j];
      for (int k = 0; k < j; ++k) v -= M[i * (i + 1) / 2 + k] * M[j * (j + 1) / 2 + k];
      M[i * (i + 1) / 2 + j] = i == j ? sqrt(fmax(v, 0.0)) : v / M[j * (j + 1) / 2 + j];
    }
  }
  for (int i = 0; i < J; ++i) {
    double v = r[i];
    for (int k = 0; k < i; ++k) v -= M[i * (i + 1) / 2 + k] * r[k];
    r[i] = v / M[i * (i + 1) / 2 + i];
  }
  for (int i = J - 1; i >= 0; --i) {
    double v = r[i];
    for (int k = i + 1; k < J; ++k) v -= M[k * (k + 1) / 2 + i] * r[k];
    r[i] = v / M[i * (i + 1) / 2 + i];
  }
  for (int j = 0; j < J; ++j) {
    G[((size_t)j * n + a1) * n + a2] = r[j];
    G[((size_t)j * n + a2) * n + a1] = r[j];
  }
}

// One warp per matrix G[j] (n x n, symmetric): cyclic Jacobi until the off-diagonal
// norm is below 1e-15 of the Frobenius norm (at most 60 sweeps).  Writes the eigenvalues
// to w[j][i] and the eigenvectors as columns of V[j].  dynamic shared memory: 2 n^2 doubles.
__global__ void __launch_bounds__(32) k_rs_eig(const double* __restrict__ G, int n, double* __restrict__ w,
                                               double* __restrict__ V) {
  extern __shared__ double sm_eig[];
  double* A = sm_eig;           // [n][n]
  double* Q = sm_eig + n * n;   // [n][n] eigenvectors (columns)
  const int lane = threadIdx.x;
  const double* g = G + (size_t)blockIdx.x * n * n;
  for (int i = lane; i < n * n; i += 32) {
    A[i] = g[i];
    Q[i] = (i / n == i % n) ? 1.0 : 0.0;
  }
  __syncwarp();
  double fro = 0.0;
  for (int i = lane; i < n * n; i += 32) fro += A[i] * A[i];
  for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int i = lane; i < n * n; i += 32)
      if (i / n != i % n) off += A[i] * A[i];
    for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
    if (off <= 1e-30 * fro) break;
    for (int pp = 0; pp < n - 1; ++pp)
      for (int qq = pp + 1; qq < n; ++qq) {
        const double apq = A[pp * n + qq];
        if (fabs(apq) <= 1e-300) continue;
        const double app = A[pp * n + pp], aqq = A[qq * n + qq];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        __syncwarp();
        // columns p, q of A (then rows, by symmetry) and of Q
        for (int i = lane; i < n; i += 32) {
          const double aip = A[i * n + pp], aiq = A[i * n + qq];
          A[i * n + pp] = c * aip - s * aiq;
          A[i * n + qq] = s * aip + c * aiq;
          const double qip = Q[i * n + pp], qiq = Q[i * n + qq];
          Q[i * n + pp] = c * qip - s * qiq;
          Q[i * n + qq] = s * qip + c * qiq;
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
          const double api = A[pp * n + i], aqi = A[qq * n + i];
          A[pp * n + i] = c * api - s * aqi;
          A[qq * n + i] = s * api + c * aqi;
        }
        __syncwarp();
      }
  }
  for (int i = lane; i < n; i += 32) w[(size_t)blockIdx.x * n + i] = A[i * n + i];
  for (int i = lane; i < n * n; i += 32) V[(size_t)blockIdx.x * n * n + i] = Q[i];
}

int seanindex0(int l, int m, int bw) {
  const int bigL = bw - 1;
  if (m >= 0) return m * (bigL + 1) - (m * (m - 1)) / 2 + (l - m);
  return (bigL * (bigL + 3)) / 2 + 1 + ((bigL + m) * (bigL + m + 1)) / 2 + (l - (m < 0 ? -m : m));
}

// Host tables, FP64.
struct ShTables {
  std::vector<double> plm, w, J, h;
  std::vector<double2> root;
  std::vector<int2> lm;
  std::vector<int> idx;
};

void build_sh_tables(int bw, int KMAX, bool hankel, ShTables& T) {
  const int size = 2 * bw;
  T.plm.assign((size_t)bw * bw * size, 0.0);
  T.w.assign(size, 0.0);
  for (int t = 0; t < size; ++t) {
    const double th = kPi * (2 * t + 1) / (2.0 * size);
    double s = 0.0;
    for (int k = 0; k < bw; ++k) s += std::sin((2 * k + 1) * th) / (2 * k + 1);
    T.w[t] = 2.0 / bw * std::sin(th) * s;
    // normalised associated Legendre functions by the standard three-term recurrence in l
    const double x = std::cos(th), sx = std::sqrt(std::fmax(0.0, 1.0 - x * x));
    double pmm = std::sqrt(0.5);
    for (int m = 0; m < bw; ++m) {
      if (m > 0) pmm = -pmm * sx * std::sqrt((2.0 * m + 1.0) / (2.0 * m));
      double p2 = 0.0, p1 = pmm;
      T.plm[((size_t)m * bw + m) * size + t] = pmm;
      for (int l = m + 1; l < bw; ++l) {
        double p;
        if (l == m + 1) {
          p = x * std::sqrt(2.0 * m + 3.0) * pmm;
        } else {
          const double a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
          const double b = std::sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
          p = a * (x * p1 - b * p2);
        }
        T.plm[((size_t)l * bw + m) * size + t] = p;
        p2 = p1;
        p1 = p;
      }
    }
  }
  T.root.resize(size);
  for (int j = 0; j < size; ++j) {
    const double a = 2.0 * kPi * j / size;
    T.root[j] = make_double2(std::cos(a), std::sin(a));
  }
  T.lm.resize((size_t)bw * bw);
  T.idx.assign((size_t)(2 * bw - 1) * bw, 0);
  for (int l = 0; l < bw; ++l)
    for (int m = -l; m <= l; ++m) {
      T.lm[seanindex0(l, m, bw)] = make_int2(l, m);
      T.idx[(size_t)(m + bw - 1) * bw + l] = seanindex0(l, m, bw);
    }
  if (hankel) {
    // J_{l+1/2}(pi k' k / KMAX) = sqrt(2x / pi) j_l(x); frdr weights on r = 1..KMAX
    T.J.assign((size_t)bw * KMAX * KMAX, 0.0);
    for (int l = 0; l < bw; ++l)
      for (int kp = 1; kp <= KMAX; ++kp)
        for (int k = 1; k <= KMAX; ++k) {
          const double x = kPi / KMAX * kp * k;
          T.J[((size_t)l * KMAX + (kp - 1)) * KMAX + (k - 1)] =
              std::sqrt(2.0 * x / kPi) * std::sph_bessel((unsigned)l, x);
        }
    T.h.assign(KMAX, 0.0);
    for (int j = 1; j <= KMAX; ++j) {
      double res;
      if (j == 1) res = std::sqrt(0.5) * 9.0;                         // sqrt(1/2) (r1 + r2)^2
      else if (j == KMAX) res = 4.0 * j * j - (2.0 * j - 1.0) * (2.0 * j - 1.0);  // 4 r_l^2 - (r_{l-1} + r_l)^2
      else res = 2.0 * 4.0 * j;                                        // (r_{j+1} - r_{j-1})(r_{j-1} + 2 r_j + r_{j+1})
      T.h[j - 1] = kPi / 4.0 * std::pow(res, 1.5);
    }
  }
}

template <class T>
cudaError_t upload(const std::vector<T>& v, T** d, cudaStream_t s) {
  cudaError_t e = cudaMalloc(d, v.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

}  // namespace

int tp3_structure_sh(tp3_ctx* c, const double* atoms, const int* mol_start, int n_mol, int LMAX, int KMAX,
                     double rmax, int route, double* density, double* amplitude, double* intensity) {
  if (int r = tp3::ctx_check(c)) return r;
  if (!atoms || !mol_start || n_mol < 1 || n_mol > 65535 || LMAX < 2 || LMAX > kShMaxLMAX || KMAX < 2 ||
      KMAX > 4096 || !(rmax > 0.0) ||
      (route != TP3_SH_INTENSITY && route != TP3_SH_REFERENCE) ||
      (route == TP3_SH_INTENSITY && (density || amplitude)) || (!density && !amplitude && !intensity))
    return tp3::ctx_fail(c, TP3_ERR_ARG, "bad structure_sh arguments");
  if (mol_start[0] != 0) return tp3::ctx_fail(c, TP3_ERR_ARG, "mol_start[0] must be 0");
  for (int i = 0; i < n_mol; ++i)
    if (mol_start[i + 1] < mol_start[i]) return tp3::ctx_fail(c, TP3_ERR_ARG, "mol_start must not decrease");
  const int n_atoms = mol_start[n_mol];
  for (int64_t i = 0; i < 5LL * n_atoms; ++i)
    if (!std::isfinite(atoms[i])) return tp3::ctx_fail(c, TP3_ERR_ARG, "non-finite atom data");
  for (int a = 0; a < n_atoms; ++a)
    if (!(atoms[5 * a + 3] > 0.0)) return tp3::ctx_fail(c, TP3_ERR_ARG, "atom width R must be > 0");
  const int bw = LMAX, size = 2 * bw, P = size * size, nco = bw * bw;
  const bool ref = route == TP3_SH_REFERENCE;
  ShTables T;
  build_sh_tables(bw, KMAX, ref, T);
  cudaStream_t s = c->stream;
  const size_t nsurf = (size_t)n_mol * KMAX;
  double *d_atoms = nullptr, *d_plm = nullptr, *d_w = nullptr, *d_J = nullptr, *d_h = nullptr;
  double2 *d_root = nullptr, *d_samp = nullptr, *d_c0 = nullptr, *d_c1 = nullptr;
  int2* d_lm = nullptr;
  int *d_idx = nullptr, *d_ms = nullptr;
  const size_t smem = (size_t)size * (2 * bw - 1) * sizeof(double2);
  std::vector<int> ms(mol_start, mol_start + n_mol + 1);
  std::vector<double> at(atoms, atoms + 5 * (size_t)n_atoms);
  if (at.empty()) at.assign(5, 1.0);  // keeps the device copy non-empty; no molecule reads it
  cudaError_t e;
  auto cleanup = [&]() {
    cudaFree(d_atoms); cudaFree(d_plm); cudaFree(d_w); cudaFree(d_J); cudaFree(d_h); cudaFree(d_root);
    cudaFree(d_samp); cudaFree(d_c0); cudaFree(d_c1); cudaFree(d_lm); cudaFree(d_idx); cudaFree(d_ms);
  };
  if ((e = upload(at, &d_atoms, s)) != cudaSuccess || (e = upload(ms, &d_ms, s)) != cudaSuccess ||
      (e = upload(T.plm, &d_plm, s)) != cudaSuccess || (e = upload(T.w, &d_w, s)) != cudaSuccess ||
      (e = upload(T.root, &d_root, s)) != cudaSuccess || (e = upload(T.lm, &d_lm, s)) != cudaSuccess ||
      (e = upload(T.idx, &d_idx, s)) != cudaSuccess ||
      (ref && ((e = upload(T.J, &d_J, s)) != cudaSuccess || (e = upload(T.h, &d_h, s)) != cudaSuccess)) ||
      (e = cudaMalloc(&d_samp, nsurf * P * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&d_c0, nsurf * nco * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&d_c1, nsurf * nco * sizeof(double2))) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_sht_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(k_sht_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
          cudaSuccess) {
    cleanup();
    cudaGetLastError();
    return tp3::ctx_cuda_fail(c, e, "structure_sh setup");
  }
  const dim3 gs((P + 255) / 256, KMAX, n_mol);
  const size_t nbytes = nsurf * nco * sizeof(double2);
  k_sh_sample<<<gs, 256, 0, s>>>(d_atoms, d_ms, size, KMAX, rmax, ref ? 1 : 0, d_samp);
  k_sht_forward<<<(unsigned)nsurf, 256, smem, s>>>(d_samp, bw, d_plm, d_w, d_root, d_lm, d_c0);
  if (ref) {
    if (density) e = cudaMemcpyAsync(density, d_c0, nbytes, cudaMemcpyDeviceToHost, s);
    k_sh_hankel<<<dim3((nco + 127) / 128, KMAX, n_mol), 128, 0, s>>>(d_c0, bw, KMAX, d_J, d_h, d_lm, d_c1);
    if (e == cudaSuccess && amplitude) e = cudaMemcpyAsync(amplitude, d_c1, nbytes, cudaMemcpyDeviceToHost, s);
    k_sht_inverse<<<(unsigned)nsurf, 256, smem, s>>>(d_c1, bw, d_plm, d_root, d_idx, d_samp);
    const size_t ns = nsurf * P;
    k_abs2<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(d_samp, ns);
    k_sht_forward<<<(unsigned)nsurf, 256, smem, s>>>(d_samp, bw, d_plm, d_w, d_root, d_lm, d_c0);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess && intensity) e = cudaMemcpyAsync(intensity, d_c0, nbytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "structure_sh");
  return TP3_OK;
}

int tp3_fit_structures_random(tp3_ctx* c, const double* volume, const double* reference, int k_lo, int k_hi, int L,
                              double stepsizefactor, int repetitions, const double* draws, double* best,
                              double* rotated) {
  if (int r = tp3::ctx_check(c)) return r;
  const int K = c->b.K, LMAX = c->b.LMAX;
  if (!volume || !reference || !draws || !best || repetitions < 1 || repetitions > 4096 || k_lo < 1 ||
      k_hi < k_lo || k_hi > K || L < 0 || !(stepsizefactor > 0.0 && stepsizefactor < 1.0) || LMAX > kShMaxLMAX)
    return tp3::ctx_fail(c, TP3_ERR_ARG, "bad fit arguments");
  const int lend = std::min(L, LMAX - 1) & ~1;
  const double pi = kPi;
  int S = 0;
  for (double st = pi; st > pi / 180.0; st *= stepsizefactor)
    if (++S > 10000000) return tp3::ctx_fail(c, TP3_ERR_ARG, "step size factor too close to 1");
  if (int r = tp3::ctx_ensure_rot_tables(c, std::max(lend, 0))) return r;
  const int bw = LMAX, size = 2 * bw, P = size * size, ncoef = LMAX * LMAX;
  const int nk = k_hi - k_lo + 1, R = repetitions;
  ShTables T;
  build_sh_tables(bw, 1, false, T);
  cudaStream_t s = c->stream;
  double *d_plm = nullptr, *d_w = nullptr, *d_eu = nullptr, *d_corr = nullptr;
  double2 *d_root = nullptr, *d_vol = nullptr, *d_ref = nullptr, *d_rot = nullptr, *d_surf = nullptr,
          *d_refs = nullptr;
  int2* d_lm = nullptr;
  int* d_idx = nullptr;
  const size_t smem = (size_t)size * (2 * bw - 1) * sizeof(double2);
  std::vector<double2> hv((size_t)K * ncoef), hr((size_t)K * ncoef);
  for (size_t i = 0; i < hv.size(); ++i) {
    hv[i] = make_double2(volume[2 * i], volume[2 * i + 1]);
    hr[i] = make_double2(reference[2 * i], reference[2 * i + 1]);
  }
  cudaError_t e;
  auto cleanup = [&]() {
    cudaFree(d_plm); cudaFree(d_w); cudaFree(d_eu); cudaFree(d_corr); cudaFree(d_root); cudaFree(d_vol);
    cudaFree(d_ref); cudaFree(d_rot); cudaFree(d_surf); cudaFree(d_refs); cudaFree(d_lm); cudaFree(d_idx);
  };
  if ((e = upload(T.plm, &d_plm, s)) != cudaSuccess || (e = upload(T.w, &d_w, s)) != cudaSuccess ||
      (e = upload(T.root, &d_root, s)) != cudaSuccess || (e = upload(T.lm, &d_lm, s)) != cudaSuccess ||
      (e = upload(T.idx, &d_idx, s)) != cudaSuccess || (e = upload(hv, &d_vol, s)) != cudaSuccess ||
      (e = upload(hr, &d_ref, s)) != cudaSuccess ||
      (e = cudaMalloc(&d_eu, (size_t)R * 3 * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&d_corr, (size_t)R * nk * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&d_rot, (size_t)std::max(R * nk, K) * ncoef * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&d_surf, (size_t)R * nk * P * sizeof(double2))) != cudaSuccess ||
      (e = cudaMalloc(&d_refs, (size_t)nk * P * sizeof(double2))) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_sht_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
          cudaSuccess) {
    cleanup();
    cudaGetLastError();
    return tp3::ctx_cuda_fail(c, e, "fit setup");
  }
  // the reference's surfaces of the K_range shells, once
  k_sht_inverse<<<nk, 256, smem, s>>>(d_ref + (size_t)(k_lo - 1) * ncoef, bw, d_plm, d_root, d_idx, d_refs);
  // repetition state: (theta, phi, gamma, best similarity); draws [R][3 + 3 S]
  const size_t nd = 3 + 3 * (size_t)S;
  std::vector<double> th(R), ph(R), ga(R), sc(R, 0.0), eu(3 * R), corr((size_t)R * nk);
  for (int r = 0; r < R; ++r) {
    const double* d = draws + (size_t)r * nd;
    ph[r] = 2.0 * pi * d[0];
    th[r] = std::acos(d[1]);
    ga[r] = 2.0 * pi * d[2];
  }
  double st = pi;
  for (int step = 0; step < S && e == cudaSuccess; ++step, st *= stepsizefactor) {
    for (int r = 0; r < R; ++r) {
      const double* d = draws + (size_t)r * nd + 3 + 3 * (size_t)step;
      eu[3 * r] = th[r] + d[0] * st / 2;
      eu[3 * r + 1] = ph[r] + d[1] * st;
      eu[3 * r + 2] = ga[r] + d[2] * st;
    }
    if ((e = cudaMemcpyAsync(d_eu, eu.data(), eu.size() * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
      break;
    k_fit_rotate<<<R * nk, 128, 0, s>>>(d_vol, d_rot, d_eu, k_lo - 1, nk, LMAX, lend, nk, c->d_delta, c->d_doff);
    k_sht_inverse<<<R * nk, 256, smem, s>>>(d_rot, bw, d_plm, d_root, d_idx, d_surf);
    k_fit_corr<<<R * nk, 256, 0, s>>>(d_surf, d_refs, nk, P, d_corr);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(corr.data(), d_corr, corr.size() * sizeof(double), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      break;
    for (int r = 0; r < R; ++r) {
      double m = 0.0;
      for (int j = 0; j < nk; ++j) m += corr[(size_t)r * nk + j];
      m /= nk;
      if (m > sc[r]) {
        sc[r] = m;
        th[r] = eu[3 * r];
        ph[r] = eu[3 * r + 1];
        ga[r] = eu[3 * r + 2];
      }
    }
  }
  int rb = 0;
  for (int r = 1; r < R; ++r)
    if (sc[r] > sc[rb]) rb = r;
  if (e == cudaSuccess) {
    best[0] = sc[rb];
    best[1] = th[rb];
    best[2] = ph[rb];
    best[3] = ga[rb];
    if (rotated) {
      // rotateStructure(volume, theta, phi, gamma, k_hi, 2:2:L): shells past k_hi unchanged
      eu[0] = th[rb];
      eu[1] = ph[rb];
      eu[2] = ga[rb];
      if ((e = cudaMemcpyAsync(d_eu, eu.data(), 3 * sizeof(double), cudaMemcpyHostToDevice, s)) == cudaSuccess) {
        k_fit_rotate<<<K, 128, 0, s>>>(d_vol, d_rot, d_eu, 0, K, LMAX, lend, k_hi, c->d_delta, c->d_doff);
        e = cudaGetLastError();
      }
      std::vector<double2> out((size_t)K * ncoef);
      if (e == cudaSuccess &&
          (e = cudaMemcpyAsync(out.data(), d_rot, out.size() * sizeof(double2), cudaMemcpyDeviceToHost, s)) ==
              cudaSuccess &&
          (e = cudaStreamSynchronize(s)) == cudaSuccess)
        for (size_t i = 0; i < out.size(); ++i) {
          rotated[2 * i] = out[i].x;
          rotated[2 * i + 1] = out[i].y;
        }
    }
  }
  cleanup();
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "fit");
  return TP3_OK;
}

int tp3_retrieve_solution(tp3_ctx* c, const double* c2, int N, int Kd, int L, int LMAX, int k_lo, int k_hi,
                          double qmax, double lambda, double* out) {
  if (int r = tp3::ctx_check(c)) return r;
  const int n = k_hi - k_lo + 1;
  if (!c2 || !out || N < 2 || Kd < 1 || k_lo < 1 || k_hi > Kd || k_hi < k_lo || L < 0 || (L & 1) ||
      LMAX < L + 1 || LMAX > kShMaxLMAX || n > 64 || L / 2 + 1 > 32 || !(qmax > 0.0) || !(lambda >= 0.0) ||
      !(2 * L < n))
    return tp3::ctx_fail(c, TP3_ERR_ARG, "bad retrieve_solution arguments (needs L < K2 / 2, K2 <= 64)");
  const double dq = qmax / k_hi;
  if (k_hi * dq * lambda / (4.0 * kPi) > 1.0) return tp3::ctx_fail(c, TP3_ERR_ARG, "lambda too large for qmax");
  const int nl = L / 2 + 1;
  cudaStream_t s = c->stream;
  std::vector<double> hc2(c2, c2 + (size_t)N * Kd * Kd);
  double *d_c2 = nullptr, *d_G = nullptr, *d_w = nullptr, *d_V = nullptr;
  cudaError_t e;
  const size_t esmem = 2 * (size_t)n * n * sizeof(double);
  auto cleanup = [&]() { cudaFree(d_c2); cudaFree(d_G); cudaFree(d_w); cudaFree(d_V); };
  if ((e = upload(hc2, &d_c2, s)) != cudaSuccess ||
      (e = cudaMalloc(&d_G, (size_t)nl * n * n * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&d_w, (size_t)nl * n * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&d_V, (size_t)nl * n * n * sizeof(double))) != cudaSuccess ||
      (e = cudaMemsetAsync(d_G, 0, (size_t)nl * n * n * sizeof(double), s)) != cudaSuccess ||
      (e = cudaFuncSetAttribute(k_rs_eig, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem)) != cudaSuccess) {
    cleanup();
    cudaGetLastError();
    return tp3::ctx_cuda_fail(c, e, "retrieve_solution setup");
  }
  const int npairs = n * (n + 1) / 2;
  k_rs_fit<<<(npairs + 63) / 64, 64, 0, s>>>(d_c2, N, Kd, k_lo, k_hi, L, dq, lambda, d_G);
  k_rs_eig<<<nl, 32, esmem, s>>>(d_G, n, d_w, d_V);
  std::vector<double> w((size_t)nl * n), V((size_t)nl * n * n);
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(w.data(), d_w, w.size() * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(V.data(), d_V, V.size() * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess) {
    cleanup();
    return tp3::ctx_cuda_fail(c, e, "retrieve_solution");
  }
  cleanup();
  // top 2l+1 eigenpairs -> real SH coefficients -> complex (Umat(l)^* applied per shell)
  const int ncoef = LMAX * LMAX;
  std::vector<double2> res((size_t)k_hi * ncoef, make_double2(0.0, 0.0));
  for (int j = 0; j < nl; ++j) {
    const int l = 2 * j, d = 2 * l + 1;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return w[(size_t)j * n + a] < w[(size_t)j * n + b]; });
    // real coefficients r[k][u], u = -l..l: u-th of the top d eigenpairs in ascending order
    std::vector<double> rr((size_t)n * d, 0.0);
    for (int u = 0; u < d && u < n; ++u) {
      const int col = order[n - d + u];
      const double* vcol = &V[(size_t)j * n * n];
      int imax = 0;
      for (int i = 1; i < n; ++i)
        if (std::fabs(vcol[i * n + col]) > std::fabs(vcol[imax * n + col])) imax = i;
      const double sg = vcol[imax * n + col] < 0.0 ? -1.0 : 1.0;
      const double sw = std::sqrt(std::max(0.0, w[(size_t)j * n + col]));
      for (int k = 0; k < n; ++k) rr[(size_t)k * d + u] = sw * sg * vcol[k * n + col];
    }
    // complex c_m = sum_u conj(Umat[u][m]) r_u, Umat(l) of src/spherical_harmonics.jl:445-457
    const double is2 = 1.0 / std::sqrt(2.0);
    for (int k = 0; k < n; ++k)
      for (int m = -l; m <= l; ++m) {
        double re = 0.0, im = 0.0;
        for (int u = -l; u <= l; ++u) {
          const double ru = rr[(size_t)k * d + (u + l)];
          double ur = 0.0, ui = 0.0;  // Umat[u][m]
          const double sgm = (m & 1) ? -1.0 : 1.0;
          if (m == 0 && u == 0) ur += 1.0;
          if (u > 0 && m == u) ur += is2;
          if (u < 0 && m == u) ui += is2 * sgm;
          if (u < 0 && m == -u) ui -= is2;
          if (u > 0 && m == -u) ur += is2 * sgm;
          re += ur * ru;
          im -= ui * ru;
        }
        res[(size_t)(k_lo - 1 + k) * ncoef + seanindex0(l, m, LMAX)] = make_double2(re, im);
      }
  }
  // negativityCheck on the synthesis grid of the scored shells
  {
    const int bw = LMAX, size = 2 * bw, P = size * size;
    ShTables T;
    build_sh_tables(bw, 1, false, T);
    double *d_plm = nullptr;
    double2 *d_root = nullptr, *d_co = nullptr, *d_surf = nullptr;
    int* d_idx = nullptr;
    const size_t smem = (size_t)size * (2 * bw - 1) * sizeof(double2);
    std::vector<double2> co(res.begin() + (size_t)(k_lo - 1) * ncoef, res.end());
    std::vector<double2> surf((size_t)n * P);
    auto clean2 = [&]() { cudaFree(d_plm); cudaFree(d_root); cudaFree(d_co); cudaFree(d_surf); cudaFree(d_idx); };
    if ((e = upload(T.plm, &d_plm, s)) != cudaSuccess || (e = upload(T.root, &d_root, s)) != cudaSuccess ||
        (e = upload(T.idx, &d_idx, s)) != cudaSuccess || (e = upload(co, &d_co, s)) != cudaSuccess ||
        (e = cudaMalloc(&d_surf, surf.size() * sizeof(double2))) != cudaSuccess ||
        (e = cudaFuncSetAttribute(k_sht_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess) {
      clean2();
      cudaGetLastError();
      return tp3::ctx_cuda_fail(c, e, "negativity setup");
    }
    k_sht_inverse<<<n, 256, smem, s>>>(d_co, bw, d_plm, d_root, d_idx, d_surf);
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(surf.data(), d_surf, surf.size() * sizeof(double2), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
      clean2();
      return tp3::ctx_cuda_fail(c, e, "negativity");
    }
    clean2();
    double neg = 0.0;
    for (int k = 0; k < n; ++k) {
      double sneg = 0.0, sabs = 0.0;
      for (int i = 0; i < P; ++i) {
        const double2 v = surf[(size_t)k * P + i];
        sneg += std::fabs(std::min(v.x, 0.0));
        sabs += std::fabs(v.x);
      }
      if (sabs > 0.0) neg += std::max(sneg / sabs, 0.0);
    }
    const double sg = neg > 0.33 ? -1.0 : 1.0;
    for (size_t i = 0; i < res.size(); ++i) {
      out[2 * i] = sg * res[i].x;
      out[2 * i + 1] = sg * res[i].y;
    }
  }
  return TP3_OK;
}

