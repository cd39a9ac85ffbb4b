"""Post-processing fit of a determined structure to a reference (src/data_processing.jl:51-78,
src/spherical_harmonics.jl:400-440).

``similarity`` is the reference's intensity-shell correlation: per shell the Pearson
correlation of the two intensities sampled on the equiangular grid of the SH
backtransform (2B x 2B points, theta_j = pi (2j+1) / (4B), phi_k = 2 pi k / (2B),
B = LMAX), averaged over the shells of K_range.  ``fitStructures_random`` is its random
restart search over rotations (rotateStructure with orders 2:2:L), step size pi shrunk
by stepsizefactor per proposal down to one degree.  Host-side; each proposal costs a
few small matrix products.
"""
from __future__ import annotations

import math

import numpy as np

from .api import rotationMatrix
from .structure import _sph_plm_table, seanindex0


class _Grid:
    def __init__(self, LMAX: int):
        B = LMAX
        self.LMAX = LMAX
        th = math.pi * (2 * np.arange(2 * B) + 1) / (4 * B)
        self.phi = 2 * math.pi * np.arange(2 * B) / (2 * B)
        self.P = _sph_plm_table(LMAX, np.cos(th))                     # [l, m, j]
        self.E = np.exp(1j * np.outer(np.arange(LMAX), self.phi))     # [m, k]
        self.idx = np.array([[seanindex0(l, m, LMAX) if m <= l else 0 for m in range(LMAX)] for l in range(LMAX)])
        self.mask = np.array([[1.0 if m <= l else 0.0 for m in range(LMAX)] for l in range(LMAX)])

    def surfaces(self, coeff: np.ndarray) -> np.ndarray:
        """Real surfaces [..., 2B, 2B] of coefficients [..., LMAX^2] (real functions)."""
        c = coeff[..., self.idx] * self.mask                            # [..., l, m]
        g = np.einsum("...lm,lmj->...mj", c, self.P)                    # [..., m, j]
        g[..., 1:, :] *= 2.0
        return np.einsum("...mj,mk->...jk", g, self.E).real


_GRIDS: dict = {}


def _grid(LMAX: int) -> _Grid:
    if LMAX not in _GRIDS:
        _GRIDS[LMAX] = _Grid(LMAX)
    return _GRIDS[LMAX]


def shell_correlation_ISC(coeff1: np.ndarray, coeff2: np.ndarray, LMAX: int, K_range) -> np.ndarray:
    """Per-shell Pearson correlation of the two intensities on the backtransform grid."""
    ks = [k - 1 for k in K_range]
    g = _grid(LMAX)
    a = g.surfaces(np.asarray(coeff1)[ks]).reshape(len(ks), -1)
    b = g.surfaces(np.asarray(coeff2)[ks]).reshape(len(ks), -1)
    a = a - a.mean(axis=1, keepdims=True)
    b = b - b.mean(axis=1, keepdims=True)
    return (a * b).sum(axis=1) / np.sqrt((a * a).sum(axis=1) * (b * b).sum(axis=1))


def similarity(coeff1: np.ndarray, coeff2: np.ndarray, LMAX: int, K_range) -> float:
    """Mean intensity-shell correlation over K_range (src/spherical_harmonics.jl:432-435)."""
    return float(np.mean(shell_correlation_ISC(coeff1, coeff2, LMAX, K_range)))


_HALF_PI: dict = {}


def _rotation_matrix(theta: float, phi: float, gamma: float, l: int) -> np.ndarray:
    """rotationMatrix(theta, phi, gamma, l) from the cached exact d^l(pi/2) = Delta (libtp3):
    d(theta) = A diag(e^{i m theta}) A^H with A = diag(i^m) Delta."""
    if l not in _HALF_PI:
        delta = rotationMatrix(math.pi / 2, 0.0, 0.0, l).real
        m = np.arange(-l, l + 1)
        _HALF_PI[l] = (1j ** m)[:, None] * delta
    A = _HALF_PI[l]
    m = np.arange(-l, l + 1)
    d = (A * np.exp(1j * m * theta)[None, :]) @ A.conj().T
    return np.exp(-1j * m * phi)[:, None] * d.real * np.exp(-1j * m * gamma)[None, :]


def rotateStructure(coeff: np.ndarray, theta: float, phi: float, gamma: float, K: int, lrange, LMAX: int) -> np.ndarray:
    """rotateStructure (src/spherical_harmonics.jl:595-603) on a coefficient array."""
    out = np.array(coeff, dtype=np.complex128, copy=True)
    for l in lrange:
        D = _rotation_matrix(theta, phi, gamma, l)
        idx = [seanindex0(l, m, LMAX) for m in range(-l, l + 1)]
        out[:K, idx] = out[:K, idx] @ D.T
    return out


def fit_draws(repetitions: int, stepsizefactor: float, seed: int = 0) -> np.ndarray:
    """The random numbers of fitStructures_random in the order the host search draws them:
    per restart three uniforms, then three normals per step; [repetitions][3 + 3 S]."""
    S, st = 0, math.pi
    while st > math.pi / 180.0:
        S += 1
        st *= stepsizefactor
    rng = np.random.default_rng(seed)
    out = np.empty((repetitions, 3 + 3 * S))
    for r in range(repetitions):
        out[r, :3] = [rng.random() for _ in range(3)]
        out[r, 3:] = [rng.normal() for _ in range(3 * S)]
    return out


def fitStructures_random(coeff: np.ndarray, reference: np.ndarray, LMAX: int, K_range, L: int,
                         stepsizefactor: float, repetitions: int = 4, seed: int = 0, basis=None):
    """Best rotation of `coeff` onto `reference` by random-restart local search
    (src/data_processing.jl:51-72).  Returns (rotated coefficients, similarity, theta, phi, gamma).
    With `basis` (a context of the structure's K and LMAX) the search runs on its device
    (tp3_fit_structures_random) with the same random numbers."""
    if basis is not None:
        from . import _lib
        ks = list(K_range)
        if ks != list(range(ks[0], ks[-1] + 1)):
            raise ValueError("K_range must be consecutive shells")
        vol = np.ascontiguousarray(coeff, dtype=np.complex128)
        ref = np.ascontiguousarray(reference, dtype=np.complex128)
        draws = np.ascontiguousarray(fit_draws(repetitions, stepsizefactor, seed))
        best = np.zeros(4)
        rotated = np.zeros_like(vol)
        _lib.check(basis._lib.tp3_fit_structures_random(basis._ctx, vol.ctypes.data, ref.ctypes.data, ks[0], ks[-1], L,
                                                        float(stepsizefactor), repetitions, draws.ctypes.data,
                                                        best.ctypes.data, rotated.ctypes.data), basis._ctx)
        return rotated, float(best[0]), float(best[1]), float(best[2]), float(best[3])
    rng = np.random.default_rng(seed)
    K = max(K_range)
    lr = range(2, L + 1, 2)
    results = []
    for _ in range(repetitions):
        stepsize = math.pi
        phi, theta, gamma = 2 * math.pi * rng.random(), math.acos(rng.random()), 2 * math.pi * rng.random()
        best = 0.0
        while stepsize > math.pi / 180.0:
            nt = theta + rng.normal() * stepsize / 2
            npf = phi + rng.normal() * stepsize
            ng = gamma + rng.normal() * stepsize
            sc = similarity(reference, rotateStructure(coeff, nt, npf, ng, K, lr, LMAX), LMAX, K_range)
            if sc > best:
                best, theta, phi, gamma = sc, nt, npf, ng
            stepsize *= stepsizefactor
        results.append((best, theta, phi, gamma))
    results.sort(key=lambda r: -r[0])
    best, theta, phi, gamma = results[0]
    return rotateStructure(coeff, theta, phi, gamma, K, lr, LMAX), best, theta, phi, gamma
