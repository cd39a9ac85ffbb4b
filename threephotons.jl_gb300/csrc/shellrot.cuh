// Per-shell SO(3) rotations of spherical-harmonic coefficients on the device
// (the Wigner-D rotation of src/spherical_harmonics.jl:572-603: Dlms,
// rotationMatrix, rotateStructure), shared by the rotation entry point and the
// per-shell chain moves.
//
// Convention.  rotationMatrix(theta, phi, gamma, l)[m, s] =
//     exp(-i s gamma - i m phi) d^l_{ms}(theta)
// with d^l the reference's d_work, and rotateStructure replaces the coefficient
// vector c_l (m = -l..l) of every shell by D c_l.  This is the action on the
// coefficients of the rotation R = Rz(phi) Ry(-theta) Rz(gamma) of the function
// (f'(n) = f(R^T n)), a homomorphism: D(R1 R2) = D(R1) D(R2).
//
// Evaluation.  d^l(theta) = P Delta E(theta) Delta^T P^*, Delta = d^l(pi/2),
// P = diag(i^m), E = diag(e^{i m theta}) (the rotation about y written as a
// rotation about z between two fixed 90-degree rotations), so
//     x_s  = e^{-i s (gamma + pi/2)} c_s
//     y_k  = e^{i k theta} sum_s Delta[s][k] x_s
//     c'_m = e^{i m (pi/2 - phi)} sum_k Delta[m][k] y_k
// costs 2 (2l+1)^2 real-by-complex products per order instead of the (2l+1)^3 of
// forming D.  Delta is exact (big-integer sums on the host) and symmetric up to
// sign: Delta[m][k] = (-1)^(m+k) Delta[k][m], which lets both products read Delta
// rows contiguously.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace tp3 {

constexpr int kMaxRotL = 62;  // largest order rotated (2l+1 <= 125)

__host__ __device__ inline int sean0(int l, int m, int LMAX) {  // 0-based seanindex
  const int bigL = LMAX - 1;
  if (m >= 0) return m * (bigL + 1) - (m * (m - 1)) / 2 + (l - m);
  return (bigL * (bigL + 3)) / 2 + 1 + ((bigL + m) * (bigL + m + 1)) / 2 + (l + m);
}

// Euler angles of the reference's rotationMatrix for the rotation exp([v]x)
// (axis v/|v|, angle |v|): with R = Rz(a) Ry(b) Rz(c), b in [0, pi], the action of
// R is rotationMatrix(theta = -b, phi = a, gamma = c).
__host__ __device__ inline void axis_angle_euler(double vx, double vy, double vz, double& theta, double& phi,
                                                 double& gamma) {
  const double a = sqrt(vx * vx + vy * vy + vz * vz);
  double R11 = 1, R13 = 0, R21 = 0, R23 = 0, R31 = 0, R32 = 0, R33 = 1;
  if (a > 0.0) {
    const double ux = vx / a, uy = vy / a, uz = vz / a;
    const double sh = sin(0.5 * a);
    const double c = cos(a), s = sin(a), C = 2.0 * sh * sh;  // 1 - cos(a) without cancellation
    R11 = c + C * ux * ux;
    R13 = C * ux * uz + s * uy;
    R21 = C * ux * uy + s * uz;
    R23 = C * uy * uz - s * ux;
    R31 = C * uz * ux - s * uy;
    R32 = C * uz * uy + s * ux;
    R33 = c + C * uz * uz;
  }
  const double sb = sqrt(R13 * R13 + R23 * R23);
  const double b = atan2(sb, R33);
  if (sb > 1e-12) {
    theta = -b;
    phi = atan2(R23, R13);
    gamma = atan2(R32, -R31);
  } else if (R33 > 0.0) {  // b = 0: R = Rz(phi)
    theta = 0.0;
    phi = atan2(R21, R11);
    gamma = 0.0;
  } else {  // b = pi: R = Rz(phi) Ry(pi)
    theta = -3.141592653589793;
    phi = atan2(-R21, -R11);
    gamma = 0.0;
  }
}

// One warp applies D^l(theta, phi, gamma) to the 2l+1 coefficients of order l of
// one shell (seanindex layout, LMAX^2 entries from `c`), writing `o` (may alias c).
// delta: Delta^l row-major [(2l+1) x (2l+1)]; xs, ys: per-warp scratch of 2l+1.
__device__ inline void rotate_order_warp(const double2* c, double2* o, int l, int LMAX, double theta, double phi,
                                         double gamma, const double* __restrict__ delta, double2* xs, double2* ys,
                                         int lane) {
  const int d = 2 * l + 1;
  const double hp = 1.5707963267948966;
  for (int t = lane; t < d; t += 32) {
    const int s = t - l;
    const double2 v = c[sean0(l, s, LMAX)];
    double sn, cs;
    sincos(-(double)s * (gamma + hp), &sn, &cs);
    xs[t] = make_double2(cs * v.x - sn * v.y, cs * v.y + sn * v.x);
  }
  __syncwarp();
  for (int t = lane; t < d; t += 32) {  // t = k + l
    double re = 0.0, im = 0.0;
    for (int u = 0; u < d; ++u) {
      const double w = delta[u * d + t];
      re = fma(w, xs[u].x, re);
      im = fma(w, xs[u].y, im);
    }
    double sn, cs;
    sincos((double)(t - l) * theta, &sn, &cs);
    ys[t] = make_double2(cs * re - sn * im, cs * im + sn * re);
  }
  __syncwarp();
  for (int t = lane; t < d; t += 32) {  // t = m + l
    double re = 0.0, im = 0.0;
    for (int u = 0; u < d; ++u) {
      // Delta[m][k] = (-1)^(m+k) Delta[k][m]
      const double w = ((t + u) & 1) ? -delta[u * d + t] : delta[u * d + t];
      re = fma(w, ys[u].x, re);
      im = fma(w, ys[u].y, im);
    }
    double sn, cs;
    sincos((double)(t - l) * (hp - phi), &sn, &cs);
    o[sean0(l, t - l, LMAX)] = make_double2(cs * re - sn * im, cs * im + sn * re);
  }
  __syncwarp();
}

}  // namespace tp3
