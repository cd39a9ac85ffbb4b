/*
 * Reference-form CPU path of ThreePhotons.jl's c3 (oracle; C + OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY: the CPU baseline and a checker.  The product
 * library never links it.
 *
 * Restates, with the reference's mixed precision:
 *   tp3ref_tables  calculate_basis' table fill (src/correlations.jl:133-148):
 *                  B[g, j] = f32(cos(m2 a + m3 b)), g = a_index + N * b_index;
 *                  h_P[j, ki] = f32(w_j sphPlm(l1,m1,th_k1) sphPlm(l2,m2,th_k2) sphPlm(l3,m3,th_k3)).
 *   tp3ref_pa      calculate_triple_products_fast (src/correlations.jl:157-176):
 *                  one task per PAcombos column, As = sum_j w_j Re(ck1[i1] ck2[i2] ck3[i3])
 *                  in f64, PA[jstart:jstart+mcombos-1, ki] = As * h_P[...] (f64).
 * The product c3 = B * PA (src/correlations.jl:182) is a plain matrix product and
 * runs through the host BLAS in oracle/refcpu.py.
 */
#include <math.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* B: G x basislen col-major f32; hP: basislen x klength col-major f32.
 * indices: 9 x basislen col-major (1-based seanindex x3, l1, m1, l2, m2, l3, m3).
 * klist: klength x 3 row-major, 1-based (k1, k2, k3).
 * Y: K x ncoef, Y[k * ncoef + sean - 1] = sphPlm(l, m, theta_k). */
void tp3ref_tables(int N, int64_t basislen, const int64_t* indices, int K, int64_t klength,
                   const int64_t* klist, const double* w, const double* Y, int ncoef, float* B, float* hP) {
  const int64_t G = 2LL * N * N;
  const double pi = 3.14159265358979323846;
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < basislen; ++j) {
    const int64_t* ix = indices + 9 * j;
    const double m2 = (double)ix[6], m3 = (double)ix[8];
    for (int64_t g = 0; g < G; ++g) {
      const int64_t ia = g % N, ib = g / N;
      const double a = (ia + 0.5) * pi / N;
      const double b = (ib + 0.5) * pi / N;
      B[g + G * j] = (float)cos(m2 * a + m3 * b);
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t ki = 0; ki < klength; ++ki) {
    const int64_t k1 = klist[3 * ki] - 1, k2 = klist[3 * ki + 1] - 1, k3 = klist[3 * ki + 2] - 1;
    for (int64_t j = 0; j < basislen; ++j) {
      const int64_t* ix = indices + 9 * j;
      const double v = w[j] * Y[k1 * ncoef + ix[0] - 1] * Y[k2 * ncoef + ix[1] - 1] * Y[k3 * ncoef + ix[2] - 1];
      hP[j + basislen * ki] = (float)v;
    }
  }
}

/* coeff: K x ncoef complex, interleaved (re, im), shell-major.
 * combos: 9 x ncombo col-major, 1-based (k1, k2, k3, ki, l1, l2, l3, jstart, mcombos). */
void tp3ref_pa(int ncoef, const double* coeff, int64_t basislen, const double* w, const int64_t* indices,
               int64_t ncombo, const int64_t* combos, const float* hP, double* PA) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < ncombo; ++i) {
    const int64_t* cb = combos + 9 * i;
    const int64_t k1 = cb[0] - 1, k2 = cb[1] - 1, k3 = cb[2] - 1, ki = cb[3] - 1;
    const int64_t jstart = cb[7] - 1, mcombos = cb[8];
    const double* c1 = coeff + 2 * ncoef * k1;
    const double* c2 = coeff + 2 * ncoef * k2;
    const double* c3 = coeff + 2 * ncoef * k3;
    double As = 0.0;
    for (int64_t n = 0; n < mcombos; ++n) {
      const int64_t j = jstart + n;
      const int64_t* ix = indices + 9 * j;
      const double ar = c1[2 * (ix[0] - 1)], ai = c1[2 * (ix[0] - 1) + 1];
      const double br = c2[2 * (ix[1] - 1)], bi = c2[2 * (ix[1] - 1) + 1];
      const double cr = c3[2 * (ix[2] - 1)], ci = c3[2 * (ix[2] - 1) + 1];
      /* ck1 * ck2 * ck3, real part */
      const double pr = ar * br - ai * bi, pi_ = ar * bi + ai * br;
      As += w[j] * (pr * cr - pi_ * ci);
    }
    for (int64_t n = 0; n < mcombos; ++n) {
      const int64_t j = jstart + n;
      PA[j + basislen * ki] = As * (double)hP[j + basislen * ki];
    }
  }
}

int tp3ref_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* T[ki][lt] = sum_{j in lt} w_j Re(ck1[i1] ck2[i2] ck3[i3]) in FP64 (the As sums of
 * correlations.jl:157-176), row-major klength x n_lt; lt ranges are 0-based. */
void tp3ref_T(int ncoef, const double* coeff, const double* w, const int64_t* indices, int n_lt,
              const int64_t* lt_start, const int64_t* lt_count, int64_t klength, const int64_t* klist, double* T) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t ki = 0; ki < klength; ++ki) {
    const int64_t k1 = klist[3 * ki] - 1, k2 = klist[3 * ki + 1] - 1, k3 = klist[3 * ki + 2] - 1;
    const double* c1 = coeff + 2 * ncoef * k1;
    const double* c2 = coeff + 2 * ncoef * k2;
    const double* c3 = coeff + 2 * ncoef * k3;
    for (int lt = 0; lt < n_lt; ++lt) {
      double As = 0.0;
      for (int64_t j = lt_start[lt]; j < lt_start[lt] + lt_count[lt]; ++j) {
        const int64_t* ix = indices + 9 * j;
        const double ar = c1[2 * (ix[0] - 1)], ai = c1[2 * (ix[0] - 1) + 1];
        const double br = c2[2 * (ix[1] - 1)], bi = c2[2 * (ix[1] - 1) + 1];
        const double cr = c3[2 * (ix[2] - 1)], ci = c3[2 * (ix[2] - 1) + 1];
        const double pr = ar * br - ai * bi, pi_ = ar * bi + ai * br;
        As += w[j] * (pr * cr - pi_ * ci);
      }
      T[ki * n_lt + lt] = As;
    }
  }
}
