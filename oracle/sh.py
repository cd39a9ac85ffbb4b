"""FP64 spherical-harmonic primitives of the ThreePhotons.jl hot path (oracle).

TEST INFRASTRUCTURE ONLY.  This module is the oracle: tests, the smoke check and
the CPU-baseline leg of bench.py may call it, as the checker.  The product
library never imports it.

Restates, in plain Python/numpy, the conventions the reference's correlation
code relies on:

* ``seanindex``  -- src/spherical_harmonics.jl:163-170 (1-based linear index of
  (l, m) in a bandwidth-LMAX coefficient vector: m >= 0 blocks first, then
  m = -(LMAX-1) .. -1).
* ``wigner3j``   -- src/spherical_harmonics.jl:63-65, which calls GSL
  ``gsl_sf_coupling_3j``.  GSL is not vendored by the reference; this is the
  Racah closed form evaluated with exact rational arithmetic (Python integers),
  so exact zeros are exact and non-zero values are correctly rounded.
* ``sphPlm``     -- src/spherical_harmonics.jl:69-76, which calls GSL
  ``gsl_sf_legendre_sphPlm`` (orthonormalised associated Legendre function with
  the Condon-Shortley phase); for m < 0 the reference multiplies the |m| value
  by (-1)^|m|.  Evaluated with the standard three-term recurrence in FP64.
* ``Umat``       -- src/spherical_harmonics.jl:445-457, complex -> real SH
  transformation matrix of order l.
* ``d_work`` / ``rotation_matrix`` / ``rotate_structure`` -- src/spherical_harmonics.jl:
  572-603, the Wigner-D rotation of coefficients (factorial sum evaluated in 60-digit
  mpmath arithmetic, so the oracle is free of the sum's cancellation).
"""
from __future__ import annotations

import math
from fractions import Fraction
from functools import lru_cache

import numpy as np

_FACT = [1]
for _i in range(1, 400):
    _FACT.append(_FACT[-1] * _i)


def seanindex(l: int, m: int, LMAX: int) -> int:
    """1-based index of coefficient (l, m) for bandwidth LMAX (spherical_harmonics.jl:163-170)."""
    bigL = LMAX - 1
    if m >= 0:
        return m * (bigL + 1) - (m * (m - 1)) // 2 + (l - m) + 1
    return (bigL * (bigL + 3)) // 2 + 1 + ((bigL + m) * (bigL + m + 1)) // 2 + (l - abs(m)) + 1


def num_coeff(LMAX: int) -> int:
    """Coefficients per shell for bandwidth LMAX (spherical_harmonics.jl:99)."""
    return LMAX * LMAX


@lru_cache(maxsize=None)
def wigner3j_exact(j1: int, j2: int, j3: int, m1: int, m2: int, m3: int):
    """Exact square and sign of the Wigner 3j symbol (j1 j2 j3; m1 m2 m3).

    Returns (sign, Fraction w^2); sign is 0 for an exact zero.
    Racah formula, integer arguments only (the reference passes integer l, m).
    """
    if m1 + m2 + m3 != 0:
        return 0, Fraction(0)
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0, Fraction(0)
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return 0, Fraction(0)
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        den = (_FACT[k] * _FACT[j3 - j2 + k + m1] * _FACT[j3 - j1 + k - m2]
               * _FACT[j1 + j2 - j3 - k] * _FACT[j1 - k - m1] * _FACT[j2 - k + m2])
        s += Fraction((-1) ** k, den)
    if s == 0:
        return 0, Fraction(0)
    delta = Fraction(_FACT[j1 + j2 - j3] * _FACT[j1 - j2 + j3] * _FACT[-j1 + j2 + j3],
                     _FACT[j1 + j2 + j3 + 1])
    pre = (_FACT[j1 + m1] * _FACT[j1 - m1] * _FACT[j2 + m2] * _FACT[j2 - m2]
           * _FACT[j3 + m3] * _FACT[j3 - m3])
    sq = delta * pre * s * s
    sign = (1 if s > 0 else -1) * (-1 if (j1 - j2 - m3) % 2 else 1)
    return sign, sq


def _sqrt_fraction(q: Fraction) -> float:
    """Correctly rounded sqrt of a positive rational (64 guard bits)."""
    e = 128
    num = q.numerator << (2 * e)
    r = math.isqrt(num * q.denominator)
    return float(Fraction(r, q.denominator << e))


@lru_cache(maxsize=None)
def wigner3j(j1: int, j2: int, j3: int, m1: int, m2: int, m3: int) -> float:
    """Wigner 3j symbol in FP64 (role of gsl_sf_coupling_3j, spherical_harmonics.jl:64)."""
    sign, sq = wigner3j_exact(j1, j2, j3, m1, m2, m3)
    if sign == 0:
        return 0.0
    return sign * _sqrt_fraction(sq)


def wigner(l1: int, m1: int, l2: int, m2: int, l3: int, m3: int) -> float:
    """Reference argument order: wigner(l1,m1,l2,m2,l3,m3) = (l1 l2 l3; m1 m2 m3)."""
    return wigner3j(l1, l2, l3, m1, m2, m3)


def sphPlm_pos(l: int, m: int, x: float) -> float:
    """Orthonormalised associated Legendre function, m >= 0, CS phase included.

    sqrt((2l+1)/4pi) sqrt((l-m)!/(l+m)!) P_l^m(x), P_l^m with (-1)^m.
    Standard recurrence: start from P_m^m, step to P_{m+1}^m, then upward in l.
    """
    if m < 0 or m > l:
        raise ValueError("need 0 <= m <= l")
    # P_m^m normalised: (-1)^m sqrt((2m+1)/(4pi) * (2m-1)!!/(2m)!!) (1-x^2)^{m/2}
    pmm = 1.0 / math.sqrt(4.0 * math.pi)
    somx2 = math.sqrt(max(0.0, (1.0 - x) * (1.0 + x)))
    for i in range(1, m + 1):
        pmm *= -somx2 * math.sqrt((2.0 * i + 1.0) / (2.0 * i))
    if l == m:
        return pmm
    pmmp1 = x * math.sqrt(2.0 * m + 3.0) * pmm
    if l == m + 1:
        return pmmp1
    plm2, plm1 = pmm, pmmp1
    for ll in range(m + 2, l + 1):
        a = math.sqrt((4.0 * ll * ll - 1.0) / (ll * ll - m * m))
        b = math.sqrt(((ll - 1.0) ** 2 - m * m) / (4.0 * (ll - 1.0) ** 2 - 1.0))
        pl = a * (x * plm1 - b * plm2)
        plm2, plm1 = plm1, pl
    return plm1


def sphPlm(l: int, m: int, theta: float) -> float:
    """Reference wrapper semantics (spherical_harmonics.jl:69-76): x = cos(theta)."""
    x = math.cos(theta)
    if m >= 0:
        return sphPlm_pos(l, m, x)
    return (-1.0) ** abs(m) * sphPlm_pos(l, -m, x)


def sphPlm_x(l: int, m: int, x: float) -> float:
    """sphPlm with the cosine given directly (x = 0 exactly at theta = pi/2)."""
    if m >= 0:
        return sphPlm_pos(l, m, x)
    return (-1.0) ** abs(m) * sphPlm_pos(l, -m, x)


def Umat(l: int) -> np.ndarray:
    """Complex -> real SH transformation of order l (spherical_harmonics.jl:445-457).

    Rows u = -l..l, columns m = -l..l.
    """
    d = 2 * l + 1
    U = np.zeros((d, d), dtype=np.complex128)
    s = 1.0 / math.sqrt(2.0)
    for iu, u in enumerate(range(-l, l + 1)):
        for im, m in enumerate(range(-l, l + 1)):
            v = 0j
            if m == 0 and u == 0:
                v += 1.0
            if u > 0 and m == u:
                v += s
            if u < 0 and m == u:
                v += s * 1j * (-1) ** m
            if u < 0 and m == -u:
                v += s * (-1j)
            if u > 0 and m == -u:
                v += s * (-1) ** m
            U[iu, im] = v
    return U


def alpharange(N: int) -> np.ndarray:
    """alpha_i = (i - 1/2) pi / N, i = 1..N (correlations.jl:247-250)."""
    return (np.arange(N, dtype=np.float64) + 0.5) * (math.pi / N)


def alpharange_2pi(N2: int) -> np.ndarray:
    """beta_j = (j - 1/2) 2pi / N2, j = 1..N2 (correlations.jl:253-256); called with N2 = 2N."""
    return (np.arange(N2, dtype=np.float64) + 0.5) * (2.0 * math.pi / N2)


def tripletFactor(k1: int, k2: int, k3: int) -> float:
    """Multiplicity of a shell triple (datagen.jl:166-174)."""
    if k1 == k2 == k3:
        return 1.0
    if k1 == k2 or k1 == k3 or k2 == k3:
        return 3.0
    return 6.0


def d_work(l: int, m1: int, m2: int, beta: float) -> float:
    """Wigner small-d d^l_{m1 m2}(beta) (spherical_harmonics.jl:572-586), 60 digits."""
    import mpmath
    with mpmath.workdps(60):
        b = mpmath.mpf(beta) / 2
        cb, sb = mpmath.cos(b), mpmath.sin(b)
        f = mpmath.factorial
        val = mpmath.mpf(0)
        for s in range(max(0, m1 - m2), min(l - m2, l + m1) + 1):
            val += (cb ** (2 * l + m1 - m2 - 2 * s) * sb ** (m2 - m1 + 2 * s) * (-1) ** (s + m2 - m1)
                    / (f(l + m1 - s) * f(s) * f(m2 - m1 + s) * f(l - m2 - s)))
        val *= mpmath.sqrt(f(l + m1) * f(l - m1) * f(l + m2) * f(l - m2))
        return float(val)


def rotation_matrix(theta: float, phi: float, gamma: float, l: int) -> np.ndarray:
    """rotationMatrix (spherical_harmonics.jl:588-592): D[m, s] = e^{-i s gamma - i m phi} d_ms(theta)."""
    d = 2 * l + 1
    D = np.empty((d, d), dtype=np.complex128)
    for im, m in enumerate(range(-l, l + 1)):
        for js, s_ in enumerate(range(-l, l + 1)):
            D[im, js] = np.exp(-1j * s_ * gamma - 1j * m * phi) * d_work(l, m, s_, theta)
    return D


def rotate_structure(coeff: np.ndarray, theta: float, phi: float, gamma: float, K: int, lrange, LMAX: int) -> np.ndarray:
    """rotateStructure (spherical_harmonics.jl:595-603) on coeff[K', LMAX^2] (seanindex order)."""
    out = np.array(coeff, dtype=np.complex128, copy=True)
    for l in lrange:
        D = rotation_matrix(theta, phi, gamma, l)
        idx = [seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)]
        for k in range(K):
            out[k, idx] = D @ coeff[k, idx]
    return out


def axis_angle_euler(v) -> tuple:
    """(theta, phi, gamma) with rotation_matrix(theta, phi, gamma, l) = the coefficient action of the
    rotation R = exp([v]x) on functions (f'(n) = f(R^T n)).  rotationMatrix(theta, phi, gamma) is that
    action for R = Rz(phi) Ry(-theta) Rz(gamma), so with R = Rz(a) Ry(b) Rz(c), b in [0, pi]:
    theta = -b, phi = a, gamma = c."""
    v = np.asarray(v, dtype=np.float64)
    a = float(np.linalg.norm(v))
    if a == 0.0:
        R = np.eye(3)
    else:
        u = v / a
        Kx = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
        R = math.cos(a) * np.eye(3) + math.sin(a) * Kx + 2.0 * math.sin(0.5 * a) ** 2 * np.outer(u, u)
    sb = math.hypot(R[0, 2], R[1, 2])
    b = math.atan2(sb, R[2, 2])
    if sb > 1e-12:
        return -b, math.atan2(R[1, 2], R[0, 2]), math.atan2(R[2, 1], -R[2, 0])
    if R[2, 2] > 0:                      # b = 0: R = Rz(phi)
        return 0.0, math.atan2(R[1, 0], R[0, 0]), 0.0
    return -math.pi, math.atan2(-R[1, 0], -R[0, 0]), 0.0   # b = pi: R = Rz(phi) Ry(pi)


_WD_CACHE: dict = {}


def _Ylm_rows(l: int, dirs: np.ndarray) -> np.ndarray:
    """Y_lm(dirs[i]) for m = -l..l (any fixed orthonormal complex SH convention works here)."""
    th = np.arccos(np.clip(dirs[:, 2], -1.0, 1.0))
    ph = np.arctan2(dirs[:, 1], dirs[:, 0])
    ms = np.arange(-l, l + 1)
    try:
        from scipy.special import sph_harm_y
        return sph_harm_y(l, ms[None, :], th[:, None], ph[:, None])
    except ImportError:                      # scipy < 1.15: (m, l, azimuth, polar)
        from scipy.special import sph_harm
        return sph_harm(ms[None, :], l, ph[:, None], th[:, None])


def wigner_D_sampled(l: int, R: np.ndarray) -> np.ndarray:
    """Matrix S (2l+1 x 2l+1) with sum_m c_m Y_lm(R^T n) = sum_m' (S c)_m' Y_lm'(n) for every n:
    the action of the rotation R on the order-l coefficients of a function (f'(n) = f(R^T n)),
    a homomorphism S(R1 R2) = S(R1) S(R2).  Obtained by least squares on fixed random
    directions (exact up to rounding for a band-limited order-l function)."""
    if l not in _WD_CACHE:
        rng = np.random.default_rng(1000 + l)
        n = rng.normal(size=(4 * (2 * l + 1) + 16, 3))
        n /= np.linalg.norm(n, axis=1)[:, None]
        _WD_CACHE[l] = (n, np.linalg.pinv(_Ylm_rows(l, n)))
    n, pinv = _WD_CACHE[l]
    return pinv @ _Ylm_rows(l, n @ R)


def random_rotation3(rng: np.random.Generator) -> np.ndarray:
    """Haar-random SO(3) matrix."""
    Q, Rr = np.linalg.qr(rng.normal(size=(3, 3)))
    Q = Q * np.sign(np.diag(Rr))
    if np.linalg.det(Q) < 0:
        Q[:, 0] *= -1
    return Q
