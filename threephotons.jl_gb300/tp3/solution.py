"""Start structures from the two-photon correlation (src/correlations.jl:229-327).

``twoPhotons`` is the model c2 of an intensity, ``retrieveSolution`` its inversion:
for every even l the shell Gram matrix G_l[k1, k2] = sum_m c_k1lm conj(c_k2lm) is fitted
from the c2 slices by least squares against (1/4pi) P_l(cos alpha*), and the
coefficients are the top 2l+1 eigenvectors of G_l scaled by the square roots of their
eigenvalues (real SH basis, then real_to_comp).  The result matches the data up to one
rotation in O(2l+1) per l — the ambiguity the annealer removes; eigenvector signs are
fixed by making each one's largest entry positive, and the whole structure is negated
when the reference's negativityCheck exceeds 0.33.  Small host-side
eigenproblems (K2 x K2 per l), run once per chain start; nothing here is on the
per-proposal path.
"""
from __future__ import annotations

import math

import numpy as np

from .api import Umat
from .structure import seanindex0


def _legendre(l: int, x: np.ndarray) -> np.ndarray:
    """P_l(x) (gsl_sf_legendre_Plm(l, 0, x) as called by src/spherical_harmonics.jl:79-86)."""
    c = np.zeros(l + 1)
    c[l] = 1.0
    return np.polynomial.legendre.legval(x, c)


def alpharange(N: int) -> np.ndarray:
    """(i - 1/2) pi / N, i = 1..N (src/correlations.jl:247-250)."""
    return (np.arange(N) + 0.5) * (math.pi / N)


def alpha_star(alpha, k1: int, k2: int, dq: float, lambda_: float):
    """Ewald-curvature corrected angle (src/datagen.jl:49-53)."""
    t1 = math.acos(k1 * dq * lambda_ / (4 * math.pi))
    t2 = math.acos(k2 * dq * lambda_ / (4 * math.pi))
    return np.arccos(np.clip(math.sin(t1) * math.sin(t2) * np.cos(alpha) + math.cos(t1) * math.cos(t2), -1, 1))


def twoPhotons(coeff: np.ndarray, LMAX: int, L: int, N: int, K2: int, dq: float, lambda_: float = 0.0,
               minimal: bool = False, normalize: bool = False) -> np.ndarray:
    """Model c2[N, K2, K2] (alpha, k2, k1) of intensity coefficients coeff[>=K2, LMAX^2]
    (src/correlations.jl:229-244); orders 0:2:L."""
    c = np.zeros((N, K2, K2))
    a = alpharange(N)
    for k1 in range(1, K2 + 1):
        for k2 in range(1, (k1 if minimal else K2) + 1):
            sl = np.zeros(N)
            for l in range(0, L + 1, 2):
                idx = [seanindex0(l, m, LMAX) for m in range(-l, l + 1)]
                fac = np.vdot(coeff[k1 - 1, idx], coeff[k2 - 1, idx])
                sl = sl + fac.real * _legendre(l, np.cos(alpha_star(a, k1, k2, dq, lambda_)))
            c[:, k2 - 1, k1 - 1] = sl
    return c / np.sum(np.abs(c)) if normalize else c / (4 * math.pi)


def _negativity(coeff: np.ndarray, LMAX: int, krange) -> float:
    """negativityCheck (src/spherical_harmonics.jl:622-625): over the shells of krange, the
    sum of sum|min(Re I, 0)| / sum|I| of the intensity surfaces on the backtransform grid
    (2 LMAX x 2 LMAX, theta_j = pi (2j+1) / (4 LMAX), phi_k = 2 pi k / (2 LMAX))."""
    from .postprocess import _grid
    ks = [k - 1 for k in krange]
    I = _grid(LMAX).surfaces(np.asarray(coeff)[ks])
    tot = 0.0
    for Ik in I:
        s = np.sum(np.abs(Ik))
        tot += max(np.sum(np.abs(np.minimum(Ik, 0.0))) / s, 0.0) if s > 0 else 0.0
    return tot


def _canonical(v: np.ndarray) -> np.ndarray:
    """Eigenvector columns with the sign that makes each one's largest-magnitude entry
    positive (the first such entry on ties); eigensolvers leave the sign free."""
    v = v.copy()
    for j in range(v.shape[1]):
        i = int(np.argmax(np.abs(v[:, j])))
        if v[i, j] < 0:
            v[:, j] = -v[:, j]
    return v


def retrieveSolution(c2: np.ndarray, L: int, LMAX: int, K2_range, qmax: float, lambda_: float = 0.0,
                     basis=None) -> np.ndarray:
    """Intensity coefficients [K2_high, LMAX^2] consistent with c2 (src/correlations.jl:261-319).
    With `basis` (any context) the fits and eigenproblems run on its device
    (tp3_retrieve_solution)."""
    N = c2.shape[0]
    krange = list(K2_range)
    if basis is not None:
        from . import _lib
        if krange != list(range(krange[0], krange[-1] + 1)):
            raise ValueError("K2_range must be consecutive shells")
        cc = np.ascontiguousarray(c2, dtype=np.float64)
        out = np.zeros((krange[-1], LMAX * LMAX), dtype=np.complex128)
        _lib.check(basis._lib.tp3_retrieve_solution(basis._ctx, cc.ctypes.data, N, cc.shape[1], L, LMAX, krange[0],
                                                    krange[-1], float(qmax), float(lambda_), out.ctypes.data),
                   basis._ctx)
        return out
    K2, lo, hi = len(krange), min(krange), max(krange)
    if not L < K2 / 2:
        raise ValueError("retrieveSolution needs L < K2 / 2")
    dq = qmax / hi
    a = alpharange(N)
    real = np.zeros((hi, LMAX * LMAX))
    for l in range(0, L + 1, 2):
        G = np.zeros((K2, K2))
        for k1 in krange:
            for k2 in range(lo, k1 + 1):
                sl = c2[:, k2 - 1, k1 - 1].astype(np.float64)
                if lambda_ == 0.0:
                    sl = 0.5 * (sl + sl[::-1])
                upperL = min(L, min(k1, k2) * 2 - 2)
                x = np.cos(alpha_star(a, k1, k2, dq, lambda_))
                A = np.stack([_legendre(lp, x) / (4 * math.pi) for lp in range(0, upperL + 1, 2)], axis=1)
                fac = np.linalg.lstsq(A, sl, rcond=None)[0]
                if l <= upperL:
                    G[k2 - lo, k1 - lo] = G[k1 - lo, k2 - lo] = fac[l // 2]
        w, v = np.linalg.eigh(G)
        w, v = w[K2 - (2 * l + 1):], _canonical(v[:, K2 - (2 * l + 1):])
        m = np.diag(np.sqrt(np.maximum(0.0, w))) @ v.T          # (2l+1) x K2, real SH basis
        idx = [seanindex0(l, mm, LMAX) for mm in range(-l, l + 1)]
        for k in krange:
            real[k - 1, idx] = m[:, k - lo]
    out = np.zeros((hi, LMAX * LMAX), dtype=np.complex128)
    for l in range(LMAX):
        idx = [seanindex0(l, mm, LMAX) for mm in range(-l, l + 1)]
        out[:, idx] = real[:, idx] @ Umat(l).conj()                # real_to_comp: U^H r per shell
    if _negativity(out, LMAX, krange) > 0.33:
        out = -out
    return out
