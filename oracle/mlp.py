"""FP64 restatement of the learned-proposal network and its gradient (oracle).

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).  The network has no counterpart in
the reference; this module is the CPU checker of the library's forward and
backward kernels.  It reproduces every BF16 rounding the device makes (weights,
hidden activations, output gradient dO, gated gradients dZ) and accumulates in
FP64, so the device (FP32 accumulation on the tensor cores) agrees with it to
accumulation rounding.

Parameter vector (FP32): W1 (H x n_in), b1, W2 (H x H), b2, W3, b3, W4 (6 x H), b4.
Head: u = o[0:3] (drift direction), s = -3 + 4 tanh(o[3:6]) (log-scale).
Loss over candidates j of K consecutive rows with targets (t_j, lambda_j):
    sum_j lambda_j (t_j - sum_k u_k . v_k)^2 / 2
  + sum_r w_r sum_d [s_d + v_d^2 exp(-2 s_d) / 2 + log(2 pi) / 2].
"""
from __future__ import annotations

import math

import numpy as np

S_MID, S_HALF = -3.0, 4.0
DRIFT_GAMMA, DRIFT_EPS = 16.0, 0.1
N_GHIST = 8


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def f32(x) -> np.ndarray:
    """Round to FP32 (the device's bias precision), returned as float64."""
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def split_params(p: np.ndarray, n_in: int, H: int):
    p = np.asarray(p, dtype=np.float64)
    shapes = [(H, n_in), (H, H), (H, H), (6, H)]
    out, o = [], 0
    for (a, b) in shapes:
        W = p[o:o + a * b].reshape(a, b); o += a * b
        bb = p[o:o + a]; o += a
        out.append((W, bb))
    assert o == p.size
    return out


def forward(p, X, n_in: int, H: int):
    """Raw outputs O (R x 6) and the cached BF16 activations."""
    layers = split_params(p, n_in, H)
    A = [bf16(X[:, :n_in])]
    for l in range(3):
        W, b = layers[l]
        A.append(bf16(np.maximum(A[-1] @ bf16(W).T + f32(b), 0.0)))
    W, b = layers[3]
    O = A[-1] @ bf16(W).T + f32(b)
    return O, A


def head(O):
    return np.asarray(O[:, :3], dtype=np.float64), S_MID + S_HALF * np.tanh(O[:, 3:6])


def loss_grad(p, X, v, w, n_in: int, H: int, tw=None, K: int = 1):
    """(loss, gradient vector in the parameter layout); tw: (t_j, lambda_j) per candidate
    of K rows (None: no regression term)."""
    layers = split_params(p, n_in, H)
    O, A = forward(p, X, n_in, H)
    u, ts = O[:, :3], np.tanh(O[:, 3:6])
    s = S_MID + S_HALF * ts
    is2 = np.exp(-2.0 * s)
    loss = float(np.sum(w[:, None] * (s + 0.5 * v * v * is2 + 0.5 * math.log(2 * math.pi))))
    du = np.zeros_like(u)
    if tw is not None:
        R = O.shape[0]
        nc = R // K
        pred = np.sum((u[:nc * K] * v[:nc * K]).reshape(nc, K * 3), axis=1)
        res = tw[:nc, 0] - pred
        loss += float(np.sum(0.5 * tw[:nc, 1] * res * res))
        rr = f32(tw[:nc, 1] * res)  # the device keeps the weighted residual in FP32
        du[:nc * K] = -np.repeat(rr, K)[:, None] * v[:nc * K]
    ds = 1.0 - v * v * is2
    dO = bf16(np.concatenate([du, w[:, None] * ds * S_HALF * (1 - ts * ts)], axis=1))
    grads = []
    W4, _ = layers[3]
    gW = dO.T @ A[3]
    gb = dO.sum(axis=0)
    grads.append((gW, gb))
    dZ = bf16((dO @ bf16(W4)) * (A[3] > 0))
    for l in (2, 1, 0):
        gW = dZ.T @ A[l]
        gb = dZ.sum(axis=0)
        grads.append((gW, gb))
        if l > 0:
            W, _ = layers[l]
            dZ = bf16((dZ @ bf16(W)) * (A[l] > 0))
    grads = grads[::-1]
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def init_params(n_in: int, H: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for (a, b, sc) in [(H, n_in, 1.0), (H, H, 1.0), (H, H, 1.0), (6, H, 0.05)]:
        lim = math.sqrt(6.0 / b) * sc
        parts.append(rng.uniform(-lim, lim, size=a * b))
        parts.append(rng.uniform(-0.1, 0.1, size=a))
    return np.concatenate(parts).astype(np.float32)


def shell_features(coeff: np.ndarray, L: int, LMAX: int, hist, T: float, stride: int, ghist=None,
                   L_used: int = None) -> np.ndarray:
    """Feature rows (K x stride, BF16 values) of a state's shells: (L+1)^2 real SH
    coefficients x = Umat(l) c_l scaled to norm 8, the 8 history values dE/T clipped to
    +-10 and divided by 10, log10(T)/4, the shell's gradient estimates of the last 8
    launches (ghist [8][K][3], newest first; FP32, clipped to +-8 and halved), zeros.
    L_used (a ragged chain's own L <= L): coefficient columns of orders above it are zero."""
    from .sh import Umat, seanindex
    K = coeff.shape[0]
    nf = (L + 1) ** 2
    out = np.zeros((K, stride))
    h = np.clip(np.nan_to_num(np.asarray(hist, dtype=np.float64), nan=10.0), -10, 10) / 10.0
    for k in range(K):
        x = []
        for l in range(L + 1):
            if L_used is not None and l > L_used:
                x.extend([0.0] * (2 * l + 1))
                continue
            idx = [seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)]
            x.extend((Umat(l) @ coeff[k, idx]).real)
        x = np.asarray(x, dtype=np.float32).astype(np.float64)
        nrm = math.sqrt(float(np.sum(x * x)))
        out[k, :nf] = x * (8.0 / nrm) if nrm > 0 else 0.0
        out[k, nf:nf + 8] = h
        out[k, nf + 8] = math.log10(T) / 4.0
        if ghist is not None:
            gk = np.asarray(ghist, dtype=np.float32)[:, k, :].astype(np.float64)  # [8][3]
            out[k, nf + 9:nf + 9 + 3 * N_GHIST] = 0.5 * np.clip(gk, -8.0, 8.0).reshape(-1)
    return bf16(out)
