"""All-to-all triplet binning of photon pictures (oracle, FP64).

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).

Restates histogramCorrelationsInPicture_alltoall (src/datagen.jl:228-277) with
angle_between (src/utilities.jl:61-72), tripletFactor / doubletFactor
(src/datagen.jl:166-184) and countTriplets (src/datagen.jl:478-483), as integer
entry counts per bin plus the reference's weights.
"""
from __future__ import annotations

import math

import numpy as np

from .sh import tripletFactor


def angle_between(p1, p2) -> float:
    """utilities.jl:61-72 for detector vectors (z = 0): acos of the clamped cosine, mirrored to
    2 pi - angle when cross(p1, p2)[3] > 0, and exactly 0 when the cosine is exactly 0."""
    n1 = math.sqrt(p1[0] * p1[0] + p1[1] * p1[1])
    n2 = math.sqrt(p2[0] * p2[0] + p2[1] * p2[1])
    val = min(max((p1[0] * p2[0] + p1[1] * p2[1]) / (n1 * n2), -1.0), 1.0)
    if abs(val) > 0.0:
        a = math.acos(val)
        if p1[0] * p2[1] - p1[1] * p2[0] > 0:
            a = 2.0 * math.pi - a
        return a
    return 0.0


def doubletFactor(k1: int, k2: int) -> float:
    return 2.0 if k1 != k2 else 1.0


def bin_picture(picture: np.ndarray, dq: float, N: int, K2: int, K3: int, c1, c2, c3) -> int:
    """Add one picture's entry counts (c1[K2], c2[N, K2, K2], c3[N, 2N, K3, K3, K3], 0-based
    arrays indexed like the reference's 1-based ones).  Returns the triplets binned."""
    pts = [p for p in np.asarray(picture, dtype=np.float64)
           if 1 <= int(np.rint(math.sqrt(p[0] * p[0] + p[1] * p[1]) / dq)) <= K2]
    if len(pts) < 3:
        return 0
    pts.sort(key=lambda p: math.sqrt(p[0] * p[0] + p[1] * p[1]))
    ks = [int(np.rint(math.sqrt(p[0] * p[0] + p[1] * p[1]) / dq)) for p in pts]
    da = math.pi / N
    ntrip = 0
    for i in range(len(pts)):
        k1 = ks[i]
        c1[k1 - 1] += 1
        for j in range(i):
            k2 = ks[j]
            alpha = angle_between(pts[i], pts[j])
            alpha_s = 2 * math.pi - alpha if alpha > math.pi else alpha
            ai = int(math.floor(alpha_s / da)) % N
            c2[ai, k2 - 1, k1 - 1] += 1
            for k in range(j):
                k3 = ks[k]
                if k1 <= K3 and k2 <= K3 and k3 <= K3:
                    beta = angle_between(pts[i], pts[k])
                    if alpha > math.pi:
                        beta = 2 * math.pi - beta
                    bi = int(math.floor(beta / da)) % (2 * N)
                    c3[ai, bi, k3 - 1, k2 - 1, k1 - 1] += 1
                    ntrip += 1
    return ntrip


def weights(c1, c2, c3):
    """The reference's weighted histograms from entry counts."""
    K2 = c1.shape[0]
    K3 = c3.shape[2]
    k = np.arange(1, K2 + 1, dtype=np.float64)
    w1 = c1 / k
    df = np.where(k[:, None] != k[None, :], 2.0, 1.0)
    w2 = c2 / (df * k[:, None] * k[None, :])[None]
    tf = np.array([[[tripletFactor(a, b, c) * a * b * c for a in range(1, K3 + 1)] for b in range(1, K3 + 1)]
                   for c in range(1, K3 + 1)])            # [k3, k2, k1]
    w3 = c3 / tf[None, None]
    return w1, w2, w3


def countTriplets(c3w) -> float:
    """datagen.jl:478-483: sum |c3| tripletFactor k1 k2 k3."""
    K3 = c3w.shape[2]
    tf = np.array([[[tripletFactor(a, b, c) * a * b * c for a in range(1, K3 + 1)] for b in range(1, K3 + 1)]
                   for c in range(1, K3 + 1)])
    return float(np.sum(np.abs(c3w) * tf[None, None]))
