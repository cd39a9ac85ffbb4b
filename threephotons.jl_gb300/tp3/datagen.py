"""Histogram synthesis on the device (the role of src/datagen.jl's histogramming).

``generateHistogram`` (src/datagen.jl:363-429 without its file I/O and noise model)
samples photon pictures of an SH intensity on the GPU (tp3_sample_pictures, the role of
pointsPerOrientation, src/datagen.jl:88-144) and bins them there.
``histogram_pictures`` bins many photon pictures at once with the all-to-all rule of
histogramCorrelationsInPicture_alltoall (src/datagen.jl:228-277) on the GPU
(tp3_histogram_pictures) and returns the reference's weighted c1, c2, c3 arrays
(weights 1/k1, 1/(doubletFactor k1 k2), 1/(tripletFactor k1 k2 k3) applied to exact
entry counts).  ``countTriplets`` is src/datagen.jl:478-483.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import TP3Error, check


def _tf(k1, k2, k3):
    if k1 == k2 == k3:
        return 1.0
    if k1 == k2 or k1 == k3 or k2 == k3:
        return 3.0
    return 6.0


def _weights(K2: int, K3: int):
    k = np.arange(1, K2 + 1, dtype=np.float64)
    w1 = 1.0 / k
    w2 = 1.0 / (np.where(k[:, None] != k[None, :], 2.0, 1.0) * k[:, None] * k[None, :])   # [k2, k1]
    w3 = np.array([[[1.0 / (_tf(a, b, c) * a * b * c) for a in range(1, K3 + 1)] for b in range(1, K3 + 1)]
                   for c in range(1, K3 + 1)])                                                # [k3, k2, k1]
    return w1, w2, w3


def histogram_pictures(basis, pictures, dq: float, N: int, K2: int, K3: int, return_counts: bool = False):
    """Weighted (c1[K2], c2[N, K2, K2], c3[N, 2N, K3, K3, K3]) of a list of pictures (each an
    [n, 2] or [n, 3] array of detector vectors; z is ignored), computed on the GPU."""
    import torch
    pics = [np.asarray(p, dtype=np.float64)[:, :2] for p in pictures]
    if not pics:
        raise TP3Error(_lib.TP3_ERR_ARG, "no pictures")
    offs = np.zeros(len(pics) + 1, dtype=np.int64)
    offs[1:] = np.cumsum([len(p) for p in pics])
    dev = torch.device("cuda")
    d_p = torch.from_numpy(np.ascontiguousarray(np.concatenate(pics)) if offs[-1] else np.zeros((1, 2))).to(dev)
    d_o = torch.from_numpy(offs).to(dev)
    c1 = torch.zeros(K2, dtype=torch.int64, device=dev)
    c2 = torch.zeros(N * K2 * K2, dtype=torch.int64, device=dev)
    c3 = torch.zeros(N * 2 * N * K3 ** 3, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()  # the zeroed histograms (filled on PyTorch's stream) before the library reads them
    check(basis._lib.tp3_histogram_pictures(basis.ctx, len(pics), ctypes.c_void_p(d_p.data_ptr()), int(d_p.shape[0]),
                                            ctypes.c_void_p(d_o.data_ptr()), float(dq), N, K2, K3,
                                            ctypes.c_void_p(c1.data_ptr()), ctypes.c_void_p(c2.data_ptr()),
                                            ctypes.c_void_p(c3.data_ptr())), basis.ctx)
    basis.sync()
    n1 = c1.cpu().numpy()
    n2 = c2.cpu().numpy().reshape((N, K2, K2), order="F")
    n3 = c3.cpu().numpy().reshape((N, 2 * N, K3, K3, K3), order="F")
    if return_counts:
        return n1, n2, n3
    w1, w2, w3 = _weights(K2, K3)
    return n1 * w1, n2 * w2[None], n3 * w3[None, None]


def countTriplets(c3) -> float:
    """Total triplets of a weighted c3 histogram (src/datagen.jl:478-483)."""
    K3 = c3.shape[2]
    _, _, w3 = _weights(K3, K3)
    return float(np.sum(np.abs(c3) / w3[None, None]))


def intensity_max(basis, coeff: np.ndarray, dq: float, n_theta: int = 64, n_phi: int = 128) -> float:
    """Largest value of the SH intensity on its shells (a fine angular grid)."""
    import torch
    c = np.ascontiguousarray(coeff, dtype=np.complex128)
    d_c = torch.from_numpy(c.view(np.float64).copy()).cuda()
    out = ctypes.c_double()
    check(basis._lib.tp3_intensity_max(basis.ctx, ctypes.c_void_p(d_c.data_ptr()), c.shape[0],
                                       int(round(math.sqrt(c.shape[1]))), float(dq), n_theta, n_phi,
                                       ctypes.byref(out)), basis.ctx)
    return out.value


def generateHistogram(basis, coeff: np.ndarray, dq: float, qcut: float, K2: int, K3: int, N: int, pictures: int,
                      number_incident_photons: int = 1000, lambda_: float = 0.0, seed: int = 1,
                      batch: int = 4096, max_out: int = 1024, return_counts: bool = False):
    """Weighted (c1, c2, c3) of `pictures` sampled pictures of the intensity coeff[KMAX, LMAX^2]
    (shell k at |q| = k dq), binned with the histogram spacing qcut / K2 (src/datagen.jl:367:
    dq = qcut / K2) and the envelope width qcut / 3 (src/datagen.jl:397).  All on the GPU."""
    import torch
    c = np.ascontiguousarray(coeff, dtype=np.complex128)
    KMAX, LMAX = c.shape[0], int(round(math.sqrt(c.shape[1])))
    dev = torch.device("cuda")
    d_c = torch.from_numpy(c.view(np.float64).copy()).to(dev)
    Imax = intensity_max(basis, c, dq)
    dqh = qcut / K2
    c1 = torch.zeros(K2, dtype=torch.int64, device=dev)
    c2 = torch.zeros(N * K2 * K2, dtype=torch.int64, device=dev)
    c3 = torch.zeros(N * 2 * N * K3 ** 3, dtype=torch.int64, device=dev)
    nb = min(batch, pictures)
    ph = torch.empty((nb, max_out, 2), dtype=torch.float64, device=dev)
    cnt = torch.empty(nb, dtype=torch.int32, device=dev)
    done = 0
    torch.cuda.synchronize()  # zeroed histograms before the library adds to them
    while done < pictures:
        n = min(nb, pictures - done)
        check(basis._lib.tp3_sample_pictures(basis.ctx, n, done, ctypes.c_void_p(d_c.data_ptr()), KMAX, LMAX,
                                             float(dq), float(qcut), float(qcut / 3.0), number_incident_photons,
                                             float(lambda_), float(Imax), ctypes.c_uint64(seed), max_out,
                                             ctypes.c_void_p(ph.data_ptr()), ctypes.c_void_p(cnt.data_ptr())),
              basis.ctx)
        basis.sync()  # the sampled photons and counts before PyTorch compacts them
        counts = cnt[:n].to(torch.int64)
        mask = torch.arange(max_out, device=dev)[None, :] < counts[:, None]
        flat = ph[:n][mask].contiguous()
        offs = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        offs[1:] = torch.cumsum(counts, 0)
        if flat.numel() == 0:
            flat = torch.zeros((1, 2), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()  # the compacted photons and offsets before the library reads them
        check(basis._lib.tp3_histogram_pictures(basis.ctx, n, ctypes.c_void_p(flat.data_ptr()), int(flat.shape[0]),
                                                ctypes.c_void_p(offs.data_ptr()), float(dqh), N, K2, K3,
                                                ctypes.c_void_p(c1.data_ptr()), ctypes.c_void_p(c2.data_ptr()),
                                                ctypes.c_void_p(c3.data_ptr())), basis.ctx)
        done += n
    basis.sync()
    n1 = c1.cpu().numpy()
    n2 = c2.cpu().numpy().reshape((N, K2, K2), order="F")
    n3 = c3.cpu().numpy().reshape((N, 2 * N, K3, K3, K3), order="F")
    if return_counts:
        return n1, n2, n3
    w1, w2, w3 = _weights(K2, K3)
    return n1 * w1, n2 * w2[None], n3 * w3[None, None]
