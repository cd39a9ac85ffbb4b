"""Reference-form CPU path (oracle/refcpu.c + host BLAS): the CPU baseline.

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).

``RefCPU(L, LMAX, N, K)`` materialises the reference's tables once
(B: 2N^2 x basislen f32, h_P: basislen x klength f32, src/correlations.jl:133-148)
and evaluates, per proposal, exactly the reference CPU sequence:
  PA  = calculate_triple_products_fast   (oracle/refcpu.c, OpenMP)
  c3  = B * PA                           (f32 B promoted to f64 once, host BLAS dgemm)
  E   = energy(..., "Bayes")              (src/correlations.jl:201-226, numpy FP64)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .basis import enumerate_basis, combolist, qlist
from .c3 import energy_bayes
from .sh import sphPlm, seanindex

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "librefcpu.so")
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from . import build
            build.build()
        _lib = ctypes.CDLL(LIB)
        vp, i64, ci = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        _lib.tp3ref_tables.argtypes = [ci, i64, vp, ci, i64, vp, vp, vp, ci, vp, vp]
        _lib.tp3ref_tables.restype = None
        _lib.tp3ref_pa.argtypes = [ci, vp, i64, vp, vp, i64, vp, vp, vp]
        _lib.tp3ref_pa.restype = None
        _lib.tp3ref_threads.restype = ci
        _lib.tp3ref_T.argtypes = [ci, vp, vp, vp, ci, vp, vp, i64, vp, vp]
        _lib.tp3ref_T.restype = None
    return _lib


def triple_products_fast(b, coeff) -> np.ndarray:
    """FP64 T[ki, lt] (klength x n_lt) with the C + OpenMP loop (same sums as oracle.c3.triple_products)."""
    lib = load()
    c = np.ascontiguousarray(np.asarray(coeff)[: b.K], dtype=np.complex128)
    indices = np.ascontiguousarray(b.indices.T)
    starts = np.array([js - 1 for (_, _, _, mc, js) in b.mcombolist], dtype=np.int64)
    counts = np.array([mc for (_, _, _, mc, js) in b.mcombolist], dtype=np.int64)
    klist = np.ascontiguousarray(b.klist)
    T = np.empty((b.klength, b.n_lt), dtype=np.float64)
    lib.tp3ref_T(b.LMAX * b.LMAX, c.ctypes.data, b.wignerlist.ctypes.data, indices.ctypes.data, b.n_lt,
                 starts.ctypes.data, counts.ctypes.data, b.klength, klist.ctypes.data, T.ctypes.data)
    return T


def threads() -> int:
    return int(load().tp3ref_threads())


class RefCPU:
    def __init__(self, L: int, LMAX: int, N: int, K: int, lam: float = 0.0, dq: float = 0.0):
        lib = load()
        b = enumerate_basis(L, LMAX, N, K, lam, dq)
        self.b = b
        self.N, self.K, self.LMAX = N, K, LMAX
        th = qlist(b)
        ncoef = LMAX * LMAX
        Y = np.zeros((K, ncoef))
        for k in range(K):
            for l in b.lrange:
                for m in range(-l, l + 1):
                    Y[k, seanindex(l, m, LMAX) - 1] = sphPlm(l, m, th[k])
        self.indices = np.ascontiguousarray(b.indices.T)          # basislen x 9
        self.combos = np.ascontiguousarray(combolist(b).T)        # ncombo x 9
        klist = np.ascontiguousarray(b.klist)
        G = 2 * N * N
        B = np.empty((G, b.basislen), dtype=np.float32, order="F")
        hP = np.empty((b.basislen, b.klength), dtype=np.float32, order="F")
        lib.tp3ref_tables(N, b.basislen, self.indices.ctypes.data, K, b.klength, klist.ctypes.data,
                          b.wignerlist.ctypes.data, Y.ctypes.data, ncoef, B.ctypes.data, hP.ctypes.data)
        self.B32 = B
        self.hP = hP
        self.B64 = np.asfortranarray(B, dtype=np.float64)
        self.PA = np.empty((b.basislen, b.klength), dtype=np.float64, order="F")

    def c3(self, coeff: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(np.asarray(coeff)[: self.K], dtype=np.complex128)
        load().tp3ref_pa(self.LMAX * self.LMAX, c.ctypes.data, self.b.basislen, self.b.wignerlist.ctypes.data,
                         self.indices.ctypes.data, self.combos.shape[0], self.combos.ctypes.data,
                         self.hP.ctypes.data, self.PA.ctypes.data)
        return self.B64 @ self.PA

    def energy(self, coeff: np.ndarray, c3ref: np.ndarray) -> float:
        return energy_bayes(self.c3(coeff), c3ref, self.K, self.N)
