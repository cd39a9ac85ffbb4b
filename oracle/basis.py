"""Basis enumeration of the three-photon correlation (oracle, FP64).

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).

Restates ``calculate_basis`` / ``calculate_combolist`` of the reference
(src/correlations.jl:68-153) with the same loop order and the same non-zero
rule: an entry j = (l1, m1, l2, m2, l3, m3) of the basis exists iff
|wigner(l1, m1, l2, m2, l3, -m3)| > 100 eps (correlations.jl:92, 114-116).  The
3j values come from the exact Racah sum, so the test is "exactly non-zero".
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .sh import seanindex, wigner, sphPlm, sphPlm_x, alpharange, alpharange_2pi

EPS = np.finfo(np.float64).eps


@dataclass
class OracleBasis:
    L: int
    LMAX: int
    N: int
    K: int
    lam: float = 0.0
    dq: float = 0.0
    # per basis entry j (0-based), reference order
    wignerlist: np.ndarray = field(default=None)   # f64 [basislen]
    indices: np.ndarray = field(default=None)      # i64 [9, basislen], as the reference (1-based seanindex)
    mcombolist: list = field(default=None)         # [(l1,l2,l3,mcombos,jstart(1-based))]
    klist: np.ndarray = field(default=None)        # i64 [klength, 3] (k1,k2,k3), 1-based, reference order

    @property
    def basislen(self) -> int:
        return len(self.wignerlist)

    @property
    def klength(self) -> int:
        return self.K * (self.K + 1) * (self.K + 2) // 6

    @property
    def n_lt(self) -> int:
        return len(self.mcombolist)

    @property
    def lrange(self):
        return list(range(0, self.L + 1, 2))


def enumerate_basis(L: int, LMAX: int, N: int, K: int, lam: float = 0.0, dq: float = 0.0) -> OracleBasis:
    """Enumerate basis entries exactly as correlations.jl:87-131 (forIntensity=true)."""
    if LMAX < L + 1:
        raise ValueError(f"LMAX={LMAX} must be >= L+1={L + 1}: coefficients hold l <= LMAX-1")
    lrange = range(0, L + 1, 2)
    w_list, idx_list, mcombolist = [], [], []
    i = 1
    for l1 in lrange:
        for l2 in lrange:
            for l3 in lrange:
                mcombos = 0
                istart = i
                for m1 in range(-l1, l1 + 1):
                    for m2 in range(-l2, l2 + 1):
                        # wigner(l1,m1,l2,m2,l3,-m3) is non-zero only for m3 = m1 + m2
                        m3 = m1 + m2
                        if abs(m3) > l3:
                            continue
                        w = wigner(l1, m1, l2, m2, l3, -m3)
                        if abs(w) > 100 * EPS:
                            w_list.append(w)
                            idx_list.append((seanindex(l1, m1, LMAX), seanindex(l2, m2, LMAX),
                                             seanindex(l3, -m3, LMAX), l1, m1, l2, m2, l3, -m3))
                            i += 1
                            mcombos += 1
                if mcombos > 0:
                    mcombolist.append((l1, l2, l3, mcombos, istart))
    klist = [(k1, k2, k3) for k1 in range(1, K + 1) for k2 in range(1, k1 + 1) for k3 in range(1, k2 + 1)]
    b = OracleBasis(L=L, LMAX=LMAX, N=N, K=K, lam=lam, dq=dq)
    b.wignerlist = np.asarray(w_list, dtype=np.float64)
    b.indices = np.asarray(idx_list, dtype=np.int64).T.copy()
    b.mcombolist = mcombolist
    b.klist = np.asarray(klist, dtype=np.int64)
    return b


def combolist(b: OracleBasis) -> np.ndarray:
    """PAcombos (correlations.jl:68-84): 9 x (klength * n_lt), 1-based."""
    rows = []
    ki = 1
    for (k1, k2, k3) in b.klist:
        for (l1, l2, l3, mcombos, jstart) in b.mcombolist:
            rows.append((k1, k2, k3, ki, l1, l2, l3, jstart, mcombos))
        ki += 1
    return np.asarray(rows, dtype=np.int64).T.copy()


def qlist(b: OracleBasis) -> np.ndarray:
    """theta_k = acos(k lambda dq / 4pi), k = 1..K (correlations.jl:94)."""
    return np.array([math.acos(k * b.lam * b.dq / (4 * math.pi)) for k in range(1, b.K + 1)])


def reference_tables(b: OracleBasis):
    """B (f32, 2N^2 x basislen) and h_P (f32, basislen x klength) as correlations.jl:133-148.

    B[:, j] = cos(m2 a + m3 b) with m3 = indices[8] (the stored -m3), column-major over
    (a in alpharange(N), b in alpharange_2pi(2N)), i.e. row = a + N*b.
    h_P[j, ki] = w_j sphPlm(l1,m1,th_k1) sphPlm(l2,m2,th_k2) sphPlm(l3,m3,th_k3), rounded to f32.
    theta is computed exactly as the reference does (acos of the scaled k), so at
    lambda = 0 the cosine is cos(acos(0)) ~ 6e-17 rather than 0.
    """
    N = b.N
    al = alpharange(N)
    be = alpharange_2pi(2 * N)
    A, Bg = np.meshgrid(al, be, indexing="ij")  # [N, 2N]
    a_flat = A.reshape(-1, order="F")
    b_flat = Bg.reshape(-1, order="F")
    m2 = b.indices[6].astype(np.float64)
    m3 = b.indices[8].astype(np.float64)
    B = np.cos(np.outer(a_flat, m2) + np.outer(b_flat, m3)).astype(np.float32)
    th = qlist(b)
    # sphPlm values per (k, l, m)
    Y = {}
    for k in range(b.K):
        for l in b.lrange:
            for m in range(-l, l + 1):
                Y[(k, l, m)] = sphPlm(l, m, th[k])
    l1, mm1, l2, mm2, l3, mm3 = (b.indices[r] for r in range(3, 9))
    P = np.empty((b.basislen, b.klength), dtype=np.float32)
    ks = b.klist - 1
    for j in range(b.basislen):
        y1 = np.array([Y[(k, l1[j], mm1[j])] for k in range(b.K)])
        y2 = np.array([Y[(k, l2[j], mm2[j])] for k in range(b.K)])
        y3 = np.array([Y[(k, l3[j], mm3[j])] for k in range(b.K)])
        P[j, :] = (b.wignerlist[j] * y1[ks[:, 0]] * y2[ks[:, 1]] * y3[ks[:, 2]]).astype(np.float32)
    return B, P


def lt_of_entry(b: OracleBasis) -> np.ndarray:
    """0-based l-triple index of each basis entry."""
    out = np.empty(b.basislen, dtype=np.int64)
    for t, (_, _, _, mc, js) in enumerate(b.mcombolist):
        out[js - 1: js - 1 + mc] = t
    return out


def angular_Y_exact(b: OracleBasis) -> dict:
    """sphPlm(l, m, theta_k) with cos(theta_k) = k lambda dq / 4pi exactly (0 at lambda = 0)."""
    Y = {}
    for k in range(1, b.K + 1):
        x = k * b.lam * b.dq / (4 * math.pi)
        for l in b.lrange:
            for m in range(-l, l + 1):
                Y[(k, l, m)] = sphPlm_x(l, m, x)
    return Y


def lt_form_F(b: OracleBasis) -> np.ndarray:
    """F[g, lt] = sum_{j in lt} w_j Y1 Y2 Y3 cos(m2 a + m3 b), FP64, lambda = 0 only.

    At lambda = 0 every theta_k is pi/2, so the Legendre factors do not depend on
    the shells and c3 = F . T exactly (T = triple products per l-triple).
    Grid order: g = a + N*b over the full N x 2N grid.
    """
    if b.lam != 0.0:
        raise ValueError("lt-form table needs lambda = 0")
    N = b.N
    al = alpharange(N)
    be = alpharange_2pi(2 * N)
    A, Bg = np.meshgrid(al, be, indexing="ij")
    a_flat = A.reshape(-1, order="F")
    b_flat = Bg.reshape(-1, order="F")
    Y = angular_Y_exact(b)
    l1, mm1, l2, mm2, l3, mm3 = (b.indices[r] for r in range(3, 9))
    P = np.array([b.wignerlist[j] * Y[(1, l1[j], mm1[j])] * Y[(1, l2[j], mm2[j])] * Y[(1, l3[j], mm3[j])]
                  for j in range(b.basislen)])
    lt = lt_of_entry(b)
    F = np.zeros((2 * N * N, b.n_lt), dtype=np.float64)
    nz = np.nonzero(P)[0]
    for j in nz:
        F[:, lt[j]] += P[j] * np.cos(mm2[j] * a_flat + mm3[j] * b_flat)
    return F
