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
    """Matrix D (2l+1 x 2l+1) with sum_m c_m Y_lm(R^T n) = sum_m' (c D)_m' Y_lm'(n) for every n:
    the action of the rotation R on SH coefficients of order l, obtained by least squares on
    fixed random directions (exact up to rounding for a band-limited order-l function)."""
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
