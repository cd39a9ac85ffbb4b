// Host-side FP64 table builder for the c3 + Bayes hot path.
//
// Builds, once per context, every table the device kernels read:
//   * the basis of non-zero Wigner-3j terms in the reference's order
//     (src/correlations.jl:87-131: l1, l2, l3 over 0:2:L, then m1, m2, m3), with
//     the reference's non-zero rule |w| > 100 eps evaluated on exact 3j values;
//   * the shell-triple list k1 >= k2 >= k3 (correlations.jl:72-81) and the
//     triplet factors (datagen.jl:166-174);
//   * the angular table F[g][lt] = sum_{j in lt} w_j Y(l1,m1) Y(l2,m2) Y(l3,m3)
//     cos(m2 alpha_a + m3 beta_b) at lambda = 0 (the B and h_P product of
//     correlations.jl:141-142 regrouped by l-triple; Y = sphPlm at theta = pi/2);
//   * the grid symmetry fold used at lambda = 0 (see fold_grid()).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace tp3 {

// Wigner 3j symbol (j1 j2 j3; m1 m2 m3) for integer arguments.  Exact zero test
// (big-integer Racah sum), value correct to a few ulp.  Role of GSL
// gsl_sf_coupling_3j as called by src/spherical_harmonics.jl:63-65.
double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3);

// Orthonormalised associated Legendre function with the Condon-Shortley phase at
// cosine x; for m < 0 returns (-1)^|m| times the |m| value.  Role of
// gsl_sf_legendre_sphPlm as wrapped by src/spherical_harmonics.jl:69-76.
double sphPlm_x(int l, int m, double x);

// Wigner small-d at beta = pi/2, d^l_{ms}(pi/2), in the convention of the
// reference's d_work (src/spherical_harmonics.jl:572-586); exact big-integer sum.
// d^l(beta) then factorises as P Delta E(beta) Delta^T P^* with Delta = d^l(pi/2),
// P = diag(i^m), E = diag(e^{i m beta}).
double wigner_d_half_pi(int l, int m, int s);

// 0-based seanindex (src/spherical_harmonics.jl:163-170 minus one).
int seanindex0(int l, int m, int LMAX);

struct Basis {
  int L = 0, LMAX = 0, N = 0, K = 0;
  double lambda = 0.0, dq = 0.0;

  // compact coefficient layout: even l <= L, m = -l..l; index coff[l/2] + m + l
  int nl = 0, nc = 0;
  std::vector<int> coff;       // [nl]
  std::vector<int> c_sean;     // [nc] compact -> 0-based seanindex
  std::vector<int> c_l, c_m;   // [nc]

  // basis entries j (reference order)
  std::vector<double> w;                     // 3j value
  std::vector<int> l1, m1, l2, m2, l3, m3;   // m3 is the reference's stored -m3
  std::vector<int> i1, i2, i3;               // compact coefficient indices
  int basislen() const { return (int)w.size(); }

  // l-triples in reference order (mcombolist)
  std::vector<int> lt_l1, lt_l2, lt_l3, lt_jstart, lt_jcount;
  int n_lt() const { return (int)lt_l1.size(); }

  // shell triples
  int klength = 0;
  std::vector<int> k1s, k2s, k3s;   // 0-based
  std::vector<double> tf;

  // grid
  int G = 0;          // 2 N^2 full grid points, g = a + N*b
  int Gu = 0;         // unique points actually evaluated
  int mult = 1;       // orbit size of each unique point (4 when folded, else 1)
  std::vector<int> u_to_g;        // [Gu] representative full-grid index
  std::vector<int> g_to_u;        // [G]
};

// Enumerate the basis and index tables.  Returns "" on success or an error text.
std::string build_basis(Basis& b, int L, int LMAX, int N, int K, double lambda, double dq);

// Decide and build the grid fold.  At lambda = 0 every Legendre factor is taken at
// theta = pi/2, where sphPlm(l, m) vanishes for odd l + m; with even l only even
// m survive, so c3(alpha, beta) = c3(alpha, beta + pi) = c3(pi - alpha, pi - beta).
// For even N the four images (a,b), (a,b+N), (N-1-a,N-1-b), (N-1-a,2N-1-b) are
// distinct grid points and the N x N/2 points with b < N/2 represent them all.
void fold_grid(Basis& b, bool allow_fold);

// F[u][lt] (FP64, row-major Gu x n_lt) on the unique grid points, lambda = 0.
void build_F(const Basis& b, std::vector<double>& F);

}  // namespace tp3
