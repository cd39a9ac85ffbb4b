"""Oracle (test infrastructure only): the reference's structure -> SH coefficient pipeline.

Restates, in FP64 numpy, the steps of createSphericalHarmonicsStructure
(src/structure.jl:125-134):

* ``dh_angles``: the surface sampling of getSurface / i_to_ang
  (src/spherical_harmonics.jl:203-210, 228-235): size = 2 LMAX points per angle,
  sample i = itheta * size + iphi at phi = 2 pi iphi / size,
  theta = pi (2 itheta + 1) / (2 size), positions from sphericalToCartesian
  (src/utilities.jl:105-110).
* ``forward`` / ``inverse``: the spherical-harmonic transform that transform /
  backtransform (src/spherical_harmonics.jl:127-148) run through the vendored s2kit
  (src/sh/s2kit_interface.c:72-178, FST_semi_memo with complex samples, bandwidth LMAX).
  The s2kit library needs FFTW, which is not on this machine, so it is not built; its
  published algorithm is restated instead: Driscoll-Healy sampling and weights
  w_j = 2/B sin(theta_j) sum_{k<B} sin((2k+1) theta_j)/(2k+1) (the formula s2kit's
  makeweights.c states), an FFT along phi scaled by sqrt(2 pi)/size, and a Legendre
  sum with L2-normalised associated Legendre functions that carry the Condon-Shortley
  phase (s2kit's Pmm_L2 starts its recurrence with (-1)^m); orders m < 0 use the FFT
  bin size - |m| and the factor (-1)^|m|.  The result is f_hat(l, m) = <f, Y_lm> with
  orthonormal Y_lm = Ptilde_l^m(cos theta) e^{i m phi} / sqrt(2 pi), in seanindex order
  (src/spherical_harmonics.jl:163-170).
* ``density_route``: getDensity (src/spherical_harmonics.jl:237-247,
  getDensity_cartesian src/structure.jl:72-86 with its r^2 < 5 cut), the forward
  spherical Bessel transform (sphBesselTransform, frdr, hat!, precalcImatrices,
  src/spherical_harmonics.jl:291-347) and absoluteSquare (src/spherical_harmonics.jl:
  376-381).

The product's ``tp3.structure.intensity_coefficients`` evaluates the intensity
analytically; tests compare it with ``forward`` applied to getIntensity_cartesian
samples (the reference's intensityShell route); the device route of
``tp3_structure_sh`` is compared with ``forward`` and ``density_route``.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import jv

# (R, B) per element (src/structure.jl:8-16)
ATOM_FACTORS = {
    "C": (0.7, 6.0), "N": (0.65, 7.0), "S": (1.0, 16.0), "O": (0.6, 8.0),
    "P": (0.65, 15.0), "H": (0.3, 1.0), "D": (0.3, 1.0),
}


def seanindex0(l: int, m: int, LMAX: int) -> int:
    """0-based seanindex (src/spherical_harmonics.jl:163-170 minus one)."""
    bigL = LMAX - 1
    if m >= 0:
        return m * (bigL + 1) - (m * (m - 1)) // 2 + (l - m)
    return (bigL * (bigL + 3)) // 2 + 1 + ((bigL + m) * (bigL + m + 1)) // 2 + (l - abs(m))


def dh_angles(bw: int):
    """(phi[size], theta[size]) of the sampling grid, size = 2 bw."""
    size = 2 * bw
    i = np.arange(size)
    return 2.0 * math.pi * i / size, math.pi * (2 * i + 1) / (2 * size)


def dh_weights(bw: int) -> np.ndarray:
    """Driscoll-Healy quadrature weights for 2 bw colatitudes (sum = 2)."""
    th = dh_angles(bw)[1]
    k = np.arange(bw)
    return (2.0 / bw) * np.sin(th) * (np.sin(np.outer(th, 2 * k + 1)) / (2 * k + 1)).sum(axis=1)


def plm_l2(bw: int, x: np.ndarray) -> np.ndarray:
    """P[l, m, j]: associated Legendre functions normalised to int_{-1}^{1} P^2 dx = 1,
    with the (-1)^m Condon-Shortley phase, 0 <= m <= l < bw, at the cosines x."""
    P = np.zeros((bw, bw, x.size))
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    pmm = np.full(x.size, math.sqrt(0.5))  # P_0^0 = 1/sqrt(2)
    for m in range(bw):
        if m > 0:
            pmm = -pmm * s * math.sqrt((2.0 * m + 1.0) / (2.0 * m))
        P[m, m] = pmm
        if m + 1 < bw:
            P[m + 1, m] = x * math.sqrt(2.0 * m + 3.0) * pmm
        for l in range(m + 2, bw):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            P[l, m] = a * (x * P[l - 1, m] - b * P[l - 2, m])
    return P


def forward(samples: np.ndarray, bw: int) -> np.ndarray:
    """Coefficients (complex [bw^2], seanindex order) of complex surface samples laid
    out as [itheta * size + iphi] (transform, src/spherical_harmonics.jl:127-136)."""
    size = 2 * bw
    f = np.asarray(samples, dtype=np.complex128).reshape(size, size)
    F = np.fft.fft(f, axis=1) * (math.sqrt(2.0 * math.pi) / size)      # [theta, frequency]
    th = dh_angles(bw)[1]
    wP = plm_l2(bw, np.cos(th)) * dh_weights(bw)[None, None, :]          # [l, m, theta]
    out = np.zeros(bw * bw, dtype=np.complex128)
    for m in range(bw):
        vals = wP[m:, m, :] @ F[:, m]
        for l in range(m, bw):
            out[seanindex0(l, m, bw)] = vals[l - m]
        if m > 0:
            vals = wP[m:, m, :] @ F[:, size - m] * (-1.0) ** m
            for l in range(m, bw):
                out[seanindex0(l, -m, bw)] = vals[l - m]
    return out


def inverse(coeff: np.ndarray, bw: int) -> np.ndarray:
    """Surface samples [size^2] of coefficients (backtransform, src/spherical_harmonics.jl:
    139-148): f = sum c_lm Y_lm on the same grid."""
    size = 2 * bw
    phi, th = dh_angles(bw)
    P = plm_l2(bw, np.cos(th)) / math.sqrt(2.0 * math.pi)
    G = np.zeros((size, size), dtype=np.complex128)                      # [theta, frequency]
    for m in range(bw):
        for l in range(m, bw):
            G[:, m] += coeff[seanindex0(l, m, bw)] * P[l, m]
            if m > 0:
                G[:, size - m] += coeff[seanindex0(l, -m, bw)] * (-1.0) ** m * P[l, m]
    return (np.fft.ifft(G, axis=1) * size).reshape(-1)


def _cartesian(r: float, bw: int) -> np.ndarray:
    phi, th = dh_angles(bw)
    T, Ph = np.meshgrid(th, phi, indexing="ij")
    return np.stack([r * np.cos(Ph) * np.sin(T), r * np.sin(Ph) * np.sin(T), r * np.cos(T)], axis=-1).reshape(-1, 3)


def intensity_samples(atoms: list, q: float, bw: int) -> np.ndarray:
    """getIntensity_cartesian (src/structure.jl:89-102) on the sampling grid of radius q."""
    pos = np.array([a.pos for a in atoms])
    RB = np.array([ATOM_FACTORS.get(a.element, (0.7, 6.0)) for a in atoms])
    pts = _cartesian(q, bw)
    f = RB[:, 1] * np.exp(-0.5 * RB[:, 0] ** 2 * q * q)
    ph = pts @ pos.T
    return (np.cos(ph) @ f) ** 2 + (np.sin(ph) @ f) ** 2


def density_samples(atoms: list, r: float, bw: int) -> np.ndarray:
    """getDensity_cartesian (src/structure.jl:72-86): Gaussian atoms cut at |x - a|^2 < 5."""
    pos = np.array([a.pos for a in atoms])
    RB = np.array([ATOM_FACTORS.get(a.element, (0.7, 6.0)) for a in atoms])
    pts = _cartesian(r, bw)
    d2 = ((pts[:, None, :] - pos[None, :, :]) ** 2).sum(axis=-1)
    g = RB[:, 1] / (RB[:, 0] * math.sqrt(2.0 * math.pi)) ** 3 * np.exp(-d2 / (2.0 * RB[:, 0] ** 2))
    return np.where(d2 < 5.0, g, 0.0).sum(axis=1)


def _frdr(f: np.ndarray, r: np.ndarray) -> np.ndarray:
    """frdr (src/spherical_harmonics.jl:291-303)."""
    n = r.size
    res = np.empty(n)
    res[0] = math.sqrt(0.5) * (r[0] + r[1]) ** 2
    res[1:n - 1] = (r[2:] - r[:n - 2]) * (r[:n - 2] + 2 * r[1:n - 1] + r[2:])
    res[n - 1] = 4 * r[n - 1] ** 2 - (r[n - 2] + r[n - 1]) ** 2
    return math.pi / 4 * res ** 1.5 * f


def sph_bessel_forward(coeff: np.ndarray, LMAX: int, KMAX: int) -> np.ndarray:
    """Forward sphBesselTransform (src/spherical_harmonics.jl:305-347) of [KMAX, LMAX^2]
    density coefficients: per (l, m), hat! with I = J_{l+1/2}(k r^T), r = 1..KMAX,
    k = pi/KMAX (1..KMAX), then the factor i^l sqrt(1/k)."""
    r = np.arange(1.0, KMAX + 1)
    kk = math.pi / KMAX * r
    out = np.zeros_like(coeff)
    for l in range(LMAX):
        I = jv(l + 0.5, np.outer(kk, r))
        for m in range(-l, l + 1):
            i = seanindex0(l, m, LMAX)
            rho = coeff[:, i]
            s = I @ _frdr(rho.real, r) + 1j * (I @ _frdr(rho.imag, r))
            out[:, i] = (1j ** l) * np.sqrt(1.0 / r) * s
    return out


def density_route(atoms: list, LMAX: int, KMAX: int, rmax: float):
    """(density, amplitude, intensity) coefficients, each [KMAX, LMAX^2], by the
    reference's route: density shells at r = k rmax / KMAX -> forward -> spherical Bessel
    transform -> |.|^2 on the surface -> forward (getDensity, forward(::SphericalHarmonicsVolume),
    absoluteSquare).  Shell k of the amplitude and intensity sits at q_k = k pi / rmax."""
    dr = rmax / KMAX
    dens = np.stack([forward(density_samples(atoms, k * dr, LMAX), LMAX) for k in range(1, KMAX + 1)])
    amp = sph_bessel_forward(dens, LMAX, KMAX)
    inten = np.stack([forward(np.abs(inverse(a, LMAX)) ** 2 + 0j, LMAX) for a in amp])
    return dens, amp, inten
