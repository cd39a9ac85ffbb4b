"""Three-photon correlation c3 and the Bayes energy (oracle, FP64).

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).

Forms implemented here:

* ``triple_products``   T[ki, lt] = sum_{j in lt} w_j Re(c_k1[i1] c_k2[i2] c_k3[i3])
                         (correlations.jl:157-176, the ``As`` sum), FP64.
* ``c3_reference_form`` the reference CPU path restated with its mixed precision:
                         f32 B and h_P, f64 T / PA / accumulation
                         (correlations.jl:157-193).  PA[j, ki] = T * h_P[j, ki]; c3 = B * PA.
* ``c3_lt_form``        c3 = F T^T with an FP64 F table (lambda = 0).  Mathematically the
                         same sum regrouped by l-triple; used as the FP64 oracle.
* ``energy_bayes``      correlations.jl:196-226 with tripletFactor (datagen.jl:166-174).
* ``load_histogram``    the c3ref contract of loadHistograms (datagen.jl:432-475).

Coefficient input everywhere: complex128 array ``coeff[K', LMAX^2]`` in seanindex
order (row k-1 is shell k), the reference's ``intensity.coeff[k]``.
"""
from __future__ import annotations

import math

import numpy as np

from .basis import OracleBasis, lt_of_entry
from .sh import tripletFactor


def triple_products(b: OracleBasis, coeff: np.ndarray) -> np.ndarray:
    """T[ki, lt] in FP64 (the As accumulator of correlations.jl:169-172)."""
    coeff = np.asarray(coeff, dtype=np.complex128)
    ks = b.klist - 1
    i1 = b.indices[0] - 1
    i2 = b.indices[1] - 1
    i3 = b.indices[2] - 1
    T = np.zeros((b.klength, b.n_lt), dtype=np.float64)
    c1 = coeff[ks[:, 0]]
    c2 = coeff[ks[:, 1]]
    c3 = coeff[ks[:, 2]]
    for t, (_, _, _, mc, js) in enumerate(b.mcombolist):
        sl = slice(js - 1, js - 1 + mc)
        prod = c1[:, i1[sl]] * c2[:, i2[sl]] * c3[:, i3[sl]]
        T[:, t] = prod.real @ b.wignerlist[sl]
    return T


def c3_reference_form(b: OracleBasis, coeff: np.ndarray, B32: np.ndarray, P32: np.ndarray) -> np.ndarray:
    """Reference CPU c3 (G x klength, f64) with the reference's f32 tables.

    PA[j, ki] = As(ki, lt(j)) * h_P[j, ki]  (correlations.jl:173)
    c3 = B * PA                              (correlations.jl:182)
    """
    T = triple_products(b, coeff)
    lt = lt_of_entry(b)
    PA = T[:, lt].T * P32.astype(np.float64)          # [basislen, klength]
    return B32.astype(np.float64) @ PA


def c3_lt_form(F: np.ndarray, T: np.ndarray) -> np.ndarray:
    """c3[g, ki] = sum_lt F[g, lt] T[ki, lt] (FP64)."""
    return F @ T.T


def neumaier_sum(values) -> float:
    s = 0.0
    c = 0.0
    for v in values:
        t = s + v
        if abs(s) >= abs(v):
            c += (s - t) + v
        else:
            c += (v - t) + s
        s = t
    return s + c


def slab_energies(c3: np.ndarray, c3ref: np.ndarray, K: int, N: int, K3_range=None) -> np.ndarray:
    """Per-slab terms tf(k) * (-sum q^ log p^) of the Bayes energy (correlations.jl:203-224).

    c3: G x klength raw correlation (column ki in k1>=k2>=k3 order).
    c3ref: N x 2N x K3 x K3 x K3 histogram (c3ref[:, :, k3, k2, k1]).
    """
    if K3_range is None:
        K3_range = range(1, K + 1)
    p_all = np.maximum(c3, 1e-30)
    kmin = min(K3_range)
    out = []
    i = 0
    for k1 in K3_range:
        for k2 in range(kmin, k1 + 1):
            for k3 in range(kmin, k2 + 1):
                p = p_all[:, i].reshape(N, 2 * N, order="F")
                i += 1
                q = c3ref[:, :, k3 - 1, k2 - 1, k1 - 1]
                p = p / np.sum(np.abs(p))
                q = q / np.sum(np.abs(q))
                out.append(-1.0 * np.sum(q * np.log(p)) * tripletFactor(k1, k2, k3))
    return np.asarray(out)


def energy_bayes(c3: np.ndarray, c3ref: np.ndarray, K: int, N: int, K3_range=None) -> float:
    """Bayes energy (correlations.jl:196-226) with a compensated slab sum."""
    return neumaier_sum(slab_energies(c3, c3ref, K, N, K3_range).tolist())


def load_histogram(c3_full: np.ndarray, K3: int) -> np.ndarray:
    """loadHistograms' c3 contract (datagen.jl:445-468): double an N x N histogram to
    N x 2N, clamp at 1e-30, cut to K3 shells, normalise globally (L1)."""
    NA, NB = c3_full.shape[0], c3_full.shape[1]
    if NA == NB:
        c3_full = np.concatenate([c3_full, c3_full], axis=1)
    c3_full = np.maximum(c3_full, 1e-30)
    c3 = c3_full[:, :, :K3, :K3, :K3]
    return c3 / np.sum(np.abs(c3))


def c3_to_5d(c3: np.ndarray, K: int, N: int) -> np.ndarray:
    """FullCorrelation_parallized's non-raw layout: t[:, :, k3, k2, k1] (correlations.jl:186-191)."""
    t = np.zeros((N, 2 * N, K, K, K), dtype=np.float64, order="F")
    i = 0
    for k1 in range(1, K + 1):
        for k2 in range(1, k1 + 1):
            for k3 in range(1, k2 + 1):
                t[:, :, k3 - 1, k2 - 1, k1 - 1] = c3[:, i].reshape(N, 2 * N, order="F")
                i += 1
    return t


def c3_pair_form(b: OracleBasis, coeff: np.ndarray) -> np.ndarray:
    """c3 for any lambda in FP64, grouped by Fourier pair (m2, m3) up to sign:
    c3[g, ki] = sum_q cos(m2 a + m3 b) H[q, ki],  H[q, ki] = sum_{j in q} P_j(ki) T[ki, lt(j)],
    P_j(ki) = w_j sphPlm(l1,m1,th_k1) sphPlm(l2,m2,th_k2) sphPlm(l3,m3,th_k3) with
    th_k = acos(k lambda dq / 4pi) (correlations.jl:94, 137-148)."""
    from .basis import qlist
    from .sh import sphPlm, alpharange, alpharange_2pi
    T = triple_products(b, coeff)
    lt = lt_of_entry(b)
    th = qlist(b)
    Y = {(k, l, m): sphPlm(l, m, th[k]) for k in range(b.K) for l in b.lrange for m in range(-l, l + 1)}
    ks = b.klist - 1
    l1, m1, l2, m2, l3, m3 = (b.indices[r] for r in range(3, 9))
    qid = {}
    Hrows = []
    for j in range(b.basislen):
        key = (int(m2[j]), int(m3[j]))
        if key[0] < 0 or (key[0] == 0 and key[1] < 0):
            key = (-key[0], -key[1])
        if key not in qid:
            qid[key] = len(Hrows)
            Hrows.append(np.zeros(b.klength))
        y1 = np.array([Y[(k, l1[j], m1[j])] for k in range(b.K)])
        y2 = np.array([Y[(k, l2[j], m2[j])] for k in range(b.K)])
        y3 = np.array([Y[(k, l3[j], m3[j])] for k in range(b.K)])
        P = b.wignerlist[j] * y1[ks[:, 0]] * y2[ks[:, 1]] * y3[ks[:, 2]]
        Hrows[qid[key]] += P * T[:, lt[j]]
    N = b.N
    A, Bg = np.meshgrid(alpharange(N), alpharange_2pi(2 * N), indexing="ij")
    a = A.reshape(-1, order="F")
    be = Bg.reshape(-1, order="F")
    keys = sorted(qid, key=qid.get)
    Cq = np.cos(np.outer(a, [k[0] for k in keys]) + np.outer(be, [k[1] for k in keys]))
    return Cq @ np.stack(Hrows)


def c3_pair_form_fast(b: OracleBasis, T: np.ndarray, chunk: int = 2048) -> np.ndarray:
    """``c3_pair_form`` for a given FP64 T [klength, n_lt], vectorised over basis entries in
    chunks (the same sum: H[q, ki] = sum_{j in q} P_j(ki) T[ki, lt(j)], c3 = Cq H), for
    shapes where the per-entry loop is too slow (L18 K26)."""
    from .basis import qlist
    from .sh import sphPlm, alpharange, alpharange_2pi
    th = qlist(b)
    L = max(b.lrange)
    Yk = np.zeros((b.K, L + 1, 2 * L + 1))
    for k in range(b.K):
        for l in b.lrange:
            for m in range(-l, l + 1):
                Yk[k, l, m + L] = sphPlm(l, m, th[k])
    lt = lt_of_entry(b)
    l1, m1, l2, m2, l3, m3 = (b.indices[r].astype(np.int64) for r in range(3, 9))
    flip = (m2 < 0) | ((m2 == 0) & (m3 < 0))
    qm2, qm3 = np.where(flip, -m2, m2), np.where(flip, -m3, m3)
    keys, qid = np.unique(qm2 * 4096 + qm3, return_inverse=True)
    ks = b.klist - 1
    H = np.zeros((keys.size, b.klength))
    from scipy.sparse import csr_matrix
    for c0 in range(0, b.basislen, chunk):
        sl = slice(c0, min(b.basislen, c0 + chunk))
        P = (b.wignerlist[sl][None, :] * Yk[ks[:, 0:1], l1[None, sl], m1[None, sl] + L]
             * Yk[ks[:, 1:2], l2[None, sl], m2[None, sl] + L] * Yk[ks[:, 2:3], l3[None, sl], m3[None, sl] + L])
        P *= T[:, lt[sl]]
        n = P.shape[1]
        S = csr_matrix((np.ones(n), (qid[sl], np.arange(n))), shape=(keys.size, n))
        H += S @ P.T
    N = b.N
    A, Bg = np.meshgrid(alpharange(N), alpharange_2pi(2 * N), indexing="ij")
    a = A.reshape(-1, order="F")
    be = Bg.reshape(-1, order="F")
    km2 = np.floor_divide(keys + 2048, 4096)
    km3 = keys - km2 * 4096
    Cq = np.cos(np.outer(a, km2) + np.outer(be, km3))
    return Cq @ H
