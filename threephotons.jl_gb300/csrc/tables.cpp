// FP64 table builder (see tables.h).
#include "tables.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

namespace tp3 {
namespace {

// Minimal non-negative big integer (base 2^32) for the exact Racah sum.
struct Big {
  std::vector<uint32_t> d;  // little endian, no leading zeros; empty = 0
  static Big from(uint64_t v) {
    Big b;
    while (v) { b.d.push_back((uint32_t)v); v >>= 32; }
    return b;
  }
  bool zero() const { return d.empty(); }
  void trim() { while (!d.empty() && d.back() == 0) d.pop_back(); }
  void mul_small(uint32_t m) {
    uint64_t carry = 0;
    for (auto& x : d) {
      uint64_t t = (uint64_t)x * m + carry;
      x = (uint32_t)t;
      carry = t >> 32;
    }
    if (carry) d.push_back((uint32_t)carry);
    if (m == 0) d.clear();
  }
  static Big mul(const Big& a, const Big& b) {
    Big r;
    if (a.zero() || b.zero()) return r;
    r.d.assign(a.d.size() + b.d.size(), 0);
    for (size_t i = 0; i < a.d.size(); ++i) {
      uint64_t carry = 0;
      for (size_t j = 0; j < b.d.size(); ++j) {
        uint64_t t = (uint64_t)a.d[i] * b.d[j] + r.d[i + j] + carry;
        r.d[i + j] = (uint32_t)t;
        carry = t >> 32;
      }
      size_t k = i + b.d.size();
      while (carry) {
        uint64_t t = (uint64_t)r.d[k] + carry;
        r.d[k] = (uint32_t)t;
        carry = t >> 32;
        ++k;
      }
    }
    r.trim();
    return r;
  }
  static int cmp(const Big& a, const Big& b) {
    if (a.d.size() != b.d.size()) return a.d.size() < b.d.size() ? -1 : 1;
    for (size_t i = a.d.size(); i-- > 0;)
      if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    return 0;
  }
  static Big add(const Big& a, const Big& b) {
    Big r;
    size_t n = std::max(a.d.size(), b.d.size());
    r.d.assign(n + 1, 0);
    uint64_t carry = 0;
    for (size_t i = 0; i < n; ++i) {
      uint64_t t = carry;
      if (i < a.d.size()) t += a.d[i];
      if (i < b.d.size()) t += b.d[i];
      r.d[i] = (uint32_t)t;
      carry = t >> 32;
    }
    r.d[n] = (uint32_t)carry;
    r.trim();
    return r;
  }
  static Big sub(const Big& a, const Big& b) {  // requires a >= b
    Big r;
    r.d.assign(a.d.size(), 0);
    int64_t borrow = 0;
    for (size_t i = 0; i < a.d.size(); ++i) {
      int64_t t = (int64_t)a.d[i] - borrow - (i < b.d.size() ? (int64_t)b.d[i] : 0);
      borrow = t < 0;
      if (t < 0) t += (int64_t)1 << 32;
      r.d[i] = (uint32_t)t;
    }
    r.trim();
    return r;
  }
  // value = mant * 2^exp with mant in [0.5, 1)
  void to_ld(long double& mant, long& exp) const {
    if (zero()) { mant = 0; exp = 0; return; }
    long double v = 0;
    size_t n = d.size();
    size_t lo = n >= 3 ? n - 3 : 0;
    for (size_t i = n; i-- > lo;) v = v * 4294967296.0L + (long double)d[i];
    int e2 = 0;
    mant = frexpl(v, &e2);
    exp = (long)e2 + 32L * (long)lo;
  }
};

// signed accumulator built from two magnitudes
struct SBig {
  Big pos, neg;
  void add(const Big& v, bool negative) {
    if (negative) neg = Big::add(neg, v); else pos = Big::add(pos, v);
  }
  // returns sign and magnitude
  int finish(Big& mag) const {
    int c = Big::cmp(pos, neg);
    if (c == 0) { mag = Big(); return 0; }
    if (c > 0) { mag = Big::sub(pos, neg); return 1; }
    mag = Big::sub(neg, pos);
    return -1;
  }
};

Big range_prod(long lo_excl, long hi_incl) {  // prod_{i=lo+1}^{hi} i
  Big r = Big::from(1);
  for (long i = lo_excl + 1; i <= hi_incl; ++i) r.mul_small((uint32_t)i);
  return r;
}
Big fact(long n) { return range_prod(0, n); }

}  // namespace

double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
  if (j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  const long a = j3 - j2 + m1, b = j3 - j1 - m2, c = j1 + j2 - j3, dd = j1 - m1, e = j2 + m2;
  const long kmin = std::max({0L, -a, -b});
  const long kmax = std::min({c, dd, e});
  if (kmin > kmax) return 0.0;
  // Racah sum S = sum_k (-1)^k / [k!(a+k)!(b+k)!(c-k)!(d-k)!(e-k)!], scaled by the
  // common denominator M = kmax!(a+kmax)!(b+kmax)!(c-kmin)!(d-kmin)!(e-kmin)! so that
  // every term is an integer product of consecutive ranges.
  SBig acc;
  for (long k = kmin; k <= kmax; ++k) {
    Big t = range_prod(k, kmax);
    t = Big::mul(t, range_prod(a + k, a + kmax));
    t = Big::mul(t, range_prod(b + k, b + kmax));
    t = Big::mul(t, range_prod(c - k, c - kmin));
    t = Big::mul(t, range_prod(dd - k, dd - kmin));
    t = Big::mul(t, range_prod(e - k, e - kmin));
    acc.add(t, (k & 1) != 0);
  }
  Big S;
  int sgnS = acc.finish(S);
  if (sgnS == 0) return 0.0;
  // M
  Big M = Big::mul(fact(kmax), fact(a + kmax));
  M = Big::mul(M, fact(b + kmax));
  M = Big::mul(M, fact(c - kmin));
  M = Big::mul(M, fact(dd - kmin));
  M = Big::mul(M, fact(e - kmin));
  // w^2 = Delta * prod (j+-m)! * S^2 / M^2
  Big num = Big::mul(fact(j1 + j2 - j3), fact(j1 - j2 + j3));
  num = Big::mul(num, fact(-j1 + j2 + j3));
  num = Big::mul(num, fact(j1 + m1));
  num = Big::mul(num, fact(j1 - m1));
  num = Big::mul(num, fact(j2 + m2));
  num = Big::mul(num, fact(j2 - m2));
  num = Big::mul(num, fact(j3 + m3));
  num = Big::mul(num, fact(j3 - m3));
  num = Big::mul(num, Big::mul(S, S));
  Big den = Big::mul(fact(j1 + j2 + j3 + 1), Big::mul(M, M));
  long double mn, md;
  long en, ed;
  num.to_ld(mn, en);
  den.to_ld(md, ed);
  long double r = mn / md;
  long ex = en - ed;
  if (ex & 1) { r *= 2.0L; ex -= 1; }
  long double w = sqrtl(r) * ldexpl(1.0L, (int)(ex / 2));
  int phase = ((j1 - j2 - m3) % 2 != 0) ? -1 : 1;
  return (double)(phase * sgnS * w);
}

double wigner_d_half_pi(int l, int m, int s) {
  if (l < 0 || std::abs(m) > l || std::abs(s) > l) return 0.0;
  // d^l_{ms}(pi/2) = 2^-l sqrt((l+m)!(l-m)!(l+s)!(l-s)!)
  //                  * sum_v (-1)^(v+s-m) / [(l+m-v)! v! (s-m+v)! (l-s-v)!]
  // (the factorial sum of src/spherical_harmonics.jl:572-586 at beta = pi/2, where
  // cos(beta/2)^a sin(beta/2)^b = 2^-l for every term).  The sum is exact in big
  // integers over the common denominator M = (l+m-vmin)! vmax! (s-m+vmax)! (l-s-vmin)!.
  const long a = l + m, c = s - m, e = l - s;
  const long vmin = std::max(0L, -c), vmax = std::min(e, a);
  if (vmin > vmax) return 0.0;
  SBig acc;
  for (long v = vmin; v <= vmax; ++v) {
    Big t = range_prod(a - v, a - vmin);
    t = Big::mul(t, range_prod(v, vmax));
    t = Big::mul(t, range_prod(c + v, c + vmax));
    t = Big::mul(t, range_prod(e - v, e - vmin));
    acc.add(t, (v & 1) != 0);
  }
  Big S;
  const int sgnS = acc.finish(S);
  if (sgnS == 0) return 0.0;
  Big M = Big::mul(fact(a - vmin), fact(vmax));
  M = Big::mul(M, fact(c + vmax));
  M = Big::mul(M, fact(e - vmin));
  Big num = Big::mul(fact(l + m), fact(l - m));
  num = Big::mul(num, fact(l + s));
  num = Big::mul(num, fact(l - s));
  num = Big::mul(num, Big::mul(S, S));
  const Big den = Big::mul(M, M);
  long double mn, md;
  long en, ed;
  num.to_ld(mn, en);
  den.to_ld(md, ed);
  long double r = mn / md;
  long ex = en - ed - 2L * l;  // the 2^-l factor, squared
  if (ex & 1) { r *= 2.0L; ex -= 1; }
  const long double w = sqrtl(r) * ldexpl(1.0L, (int)(ex / 2));
  const int phase = (c % 2 != 0) ? -1 : 1;  // (-1)^(s-m)
  return (double)(phase * sgnS * w);
}

double sphPlm_x(int l, int m, double x) {
  int ma = std::abs(m);
  if (ma > l) return 0.0;
  double pmm = 1.0 / std::sqrt(4.0 * M_PI);
  double somx2 = std::sqrt(std::max(0.0, (1.0 - x) * (1.0 + x)));
  for (int i = 1; i <= ma; ++i) pmm *= -somx2 * std::sqrt((2.0 * i + 1.0) / (2.0 * i));
  double val;
  if (l == ma) {
    val = pmm;
  } else {
    double pmmp1 = x * std::sqrt(2.0 * ma + 3.0) * pmm;
    if (l == ma + 1) {
      val = pmmp1;
    } else {
      double p2 = pmm, p1 = pmmp1;
      for (int ll = ma + 2; ll <= l; ++ll) {
        double aa = std::sqrt((4.0 * ll * ll - 1.0) / ((double)ll * ll - (double)ma * ma));
        double bb = std::sqrt((((double)ll - 1.0) * (ll - 1.0) - (double)ma * ma) /
                              (4.0 * ((double)ll - 1.0) * (ll - 1.0) - 1.0));
        double pl = aa * (x * p1 - bb * p2);
        p2 = p1;
        p1 = pl;
      }
      val = p1;
    }
  }
  if (m < 0 && (ma & 1)) val = -val;
  return val;
}

int seanindex0(int l, int m, int LMAX) {
  const int bigL = LMAX - 1;
  if (m >= 0) return m * (bigL + 1) - (m * (m - 1)) / 2 + (l - m);
  return (bigL * (bigL + 3)) / 2 + 1 + ((bigL + m) * (bigL + m + 1)) / 2 + (l - std::abs(m));
}

std::string build_basis(Basis& b, int L, int LMAX, int N, int K, double lambda, double dq) {
  if (L < 0 || L > 64) return "L out of range (0..64)";
  if (LMAX < L + 1) return "LMAX must be >= L+1: a bandwidth-LMAX coefficient vector holds l <= LMAX-1";
  if (N < 1 || N > 4096) return "N out of range (1..4096)";
  if (K < 1 || K > 256) return "K out of range (1..256)";
  if (!std::isfinite(lambda) || !std::isfinite(dq)) return "lambda and dq must be finite";
  b = Basis();
  b.L = L; b.LMAX = LMAX; b.N = N; b.K = K; b.lambda = lambda; b.dq = dq;
  b.nl = L / 2 + 1;
  b.coff.resize(b.nl);
  int off = 0;
  for (int il = 0; il < b.nl; ++il) {
    int l = 2 * il;
    b.coff[il] = off;
    for (int m = -l; m <= l; ++m) {
      b.c_sean.push_back(seanindex0(l, m, LMAX));
      b.c_l.push_back(l);
      b.c_m.push_back(m);
    }
    off += 2 * l + 1;
  }
  b.nc = off;
  auto cidx = [&](int l, int m) { return b.coff[l / 2] + m + l; };
  const double thr = 100.0 * 2.220446049250313e-16;
  int j = 0;
  for (int l1 = 0; l1 <= L; l1 += 2)
    for (int l2 = 0; l2 <= L; l2 += 2)
      for (int l3 = 0; l3 <= L; l3 += 2) {
        int count = 0, start = j;
        for (int mm1 = -l1; mm1 <= l1; ++mm1)
          for (int mm2 = -l2; mm2 <= l2; ++mm2) {
            int mloop3 = mm1 + mm2;  // wigner(l1,m1,l2,m2,l3,-m3) needs m3 = m1 + m2
            if (std::abs(mloop3) > l3) continue;
            double w = wigner3j(l1, l2, l3, mm1, mm2, -mloop3);
            if (std::fabs(w) > thr) {
              b.w.push_back(w);
              b.l1.push_back(l1); b.m1.push_back(mm1);
              b.l2.push_back(l2); b.m2.push_back(mm2);
              b.l3.push_back(l3); b.m3.push_back(-mloop3);
              b.i1.push_back(cidx(l1, mm1));
              b.i2.push_back(cidx(l2, mm2));
              b.i3.push_back(cidx(l3, -mloop3));
              ++j;
              ++count;
            }
          }
        if (count > 0) {
          b.lt_l1.push_back(l1); b.lt_l2.push_back(l2); b.lt_l3.push_back(l3);
          b.lt_jstart.push_back(start); b.lt_jcount.push_back(count);
        }
      }
  for (int k1 = 0; k1 < K; ++k1)
    for (int k2 = 0; k2 <= k1; ++k2)
      for (int k3 = 0; k3 <= k2; ++k3) {
        b.k1s.push_back(k1); b.k2s.push_back(k2); b.k3s.push_back(k3);
        double t = (k1 == k2 && k2 == k3) ? 1.0 : ((k1 == k2 || k1 == k3 || k2 == k3) ? 3.0 : 6.0);
        b.tf.push_back(t);
      }
  b.klength = (int)b.k1s.size();
  b.G = 2 * N * N;
  return "";
}

void fold_grid(Basis& b, bool allow_fold) {
  const int N = b.N;
  b.g_to_u.assign(b.G, -1);
  b.u_to_g.clear();
  if (allow_fold && b.lambda == 0.0 && N % 2 == 0) {
    b.mult = 4;
    for (int bb = 0; bb < N / 2; ++bb)
      for (int a = 0; a < N; ++a) {
        int u = (int)b.u_to_g.size();
        int g = a + N * bb;
        b.u_to_g.push_back(g);
        b.g_to_u[g] = u;
        b.g_to_u[a + N * (bb + N)] = u;
        b.g_to_u[(N - 1 - a) + N * (N - 1 - bb)] = u;
        b.g_to_u[(N - 1 - a) + N * (2 * N - 1 - bb)] = u;
      }
  } else {
    b.mult = 1;
    for (int g = 0; g < b.G; ++g) { b.u_to_g.push_back(g); b.g_to_u[g] = g; }
  }
  b.Gu = (int)b.u_to_g.size();
}

void build_F(const Basis& b, std::vector<double>& F) {
  const int N = b.N, nlt = b.n_lt();
  F.assign((size_t)b.Gu * nlt, 0.0);
  // Y(l, m) at theta = pi/2 (cosine exactly 0)
  std::vector<double> Y(b.nc);
  for (int c = 0; c < b.nc; ++c) Y[c] = sphPlm_x(b.c_l[c], b.c_m[c], 0.0);
  std::vector<double> al(N), be(2 * N);
  for (int a = 0; a < N; ++a) al[a] = (a + 0.5) * M_PI / N;
  for (int q = 0; q < 2 * N; ++q) be[q] = (q + 0.5) * M_PI / N;
  for (int t = 0; t < nlt; ++t) {
    for (int jj = 0; jj < b.lt_jcount[t]; ++jj) {
      int j = b.lt_jstart[t] + jj;
      double P = b.w[j] * Y[b.i1[j]] * Y[b.i2[j]] * Y[b.i3[j]];
      if (P == 0.0) continue;
      const double m2 = b.m2[j], m3 = b.m3[j];
      for (int u = 0; u < b.Gu; ++u) {
        int g = b.u_to_g[u];
        int a = g % N, q = g / N;
        F[(size_t)u * nlt + t] += P * std::cos(m2 * al[a] + m3 * be[q]);
      }
    }
  }
}

}  // namespace tp3
