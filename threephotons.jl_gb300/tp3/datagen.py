"""Histogram synthesis on the device (the role of src/datagen.jl's histogramming).

``generateHistogram`` (src/datagen.jl:363-429 without its file I/O) samples photon
pictures of an SH intensity on the GPU (tp3_sample_pictures_ex, the role of
pointsPerOrientation, src/datagen.jl:88-144, with the variable incident photon count
and the beamstop filter) plus, for a ``GaussianNoise``, the noise photons of the same
pictures (src/datagen.jl:403-405), and bins them there.
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

from dataclasses import dataclass

from . import _lib
from ._lib import TP3Error, check


@dataclass
class GaussianNoise:
    """Radially symmetric Gaussian noise (src/datagen.jl:26-31): gamma > 0 switches it on,
    sigma is its width in q, photons the incident photons of its draw per picture."""
    gamma: float = 0.0
    sigma: float = 1.0
    photons: int = 0


def noise_coefficients(KMAX: int, LMAX: int, dq: float, sigma: float) -> np.ndarray:
    """SH coefficients of the noise intensity (get_noise_volume, src/datagen.jl:295-304):
    only l = 0, c_00(k) = gaussian_distribution(k dq, 0, sigma) (src/utilities.jl:129-133)."""
    from .structure import seanindex0
    c = np.zeros((KMAX, LMAX * LMAX), dtype=np.complex128)
    q = dq * np.arange(1, KMAX + 1)
    c[:, seanindex0(0, 0, LMAX)] = np.exp(-q * q / (2.0 * sigma * sigma)) / math.sqrt(2.0 * math.pi * sigma * sigma)
    return c


def sample_pictures(basis, d_coeff_ptr: int, KMAX: int, LMAX: int, dq: float, qcut: float, envelope_sigma: float,
                    incident: int, Imax: float, seed: int, first: int, n: int, max_out: int, d_photons_ptr: int,
                    d_counts_ptr: int, incident_photon_variance: int = 0, beamstop_width: float = 0.0,
                    stream: int = 0, lambda_: float = 0.0) -> None:
    """n pictures (first .. first + n - 1) into device buffers photons [n][max_out][2],
    counts [n] (asynchronous on the context stream)."""
    check(basis._lib.tp3_sample_pictures_ex(basis.ctx, n, first, ctypes.c_void_p(d_coeff_ptr), KMAX, LMAX, float(dq),
                                            float(qcut), float(envelope_sigma), int(incident),
                                            int(incident_photon_variance), float(beamstop_width), int(stream),
                                            float(lambda_), float(Imax), ctypes.c_uint64(seed), max_out,
                                            ctypes.c_void_p(d_photons_ptr), ctypes.c_void_p(d_counts_ptr)),
          basis.ctx)


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
                      batch: int = 4096, max_out: int = 1024, return_counts: bool = False,
                      incident_photon_variance: int = 0, beamstop_width: float = 0.0, noise: GaussianNoise = None):
    """Weighted (c1, c2, c3) of `pictures` sampled pictures of the intensity coeff[KMAX, LMAX^2]
    (shell k at |q| = k dq), binned with the histogram spacing qcut / K2 (src/datagen.jl:367:
    dq = qcut / K2) and the envelope width qcut / 3 (src/datagen.jl:397); with the
    reference's variable incident photon count, beamstop filter and GaussianNoise photons
    (noise.photons incident photons of the noise intensity per picture, envelope width
    noise.sigma * 1.05, the same beamstop, src/datagen.jl:403-405).  All on the GPU."""
    import torch
    c = np.ascontiguousarray(coeff, dtype=np.complex128)
    KMAX, LMAX = c.shape[0], int(round(math.sqrt(c.shape[1])))
    dev = torch.device("cuda")
    d_c = torch.from_numpy(c.view(np.float64).copy()).to(dev)
    Imax = intensity_max(basis, c, dq)
    with_noise = noise is not None and noise.gamma > 0.0 and noise.photons > 0
    if with_noise:
        cn = noise_coefficients(KMAX, LMAX, dq, noise.sigma)
        d_cn = torch.from_numpy(cn.view(np.float64).copy()).to(dev)
        Imax_n = intensity_max(basis, cn, dq)
    dqh = qcut / K2
    c1 = torch.zeros(K2, dtype=torch.int64, device=dev)
    c2 = torch.zeros(N * K2 * K2, dtype=torch.int64, device=dev)
    c3 = torch.zeros(N * 2 * N * K3 ** 3, dtype=torch.int64, device=dev)
    nb = min(batch, pictures)
    nsl = 2 if with_noise else 1
    phs = [torch.empty((nb, max_out, 2), dtype=torch.float64, device=dev) for _ in range(nsl)]
    cnt = torch.empty((nsl, nb), dtype=torch.int32, device=dev)
    done = 0
    torch.cuda.synchronize()  # zeroed histograms before the library adds to them
    while done < pictures:
        n = min(nb, pictures - done)
        # molecule photons (stream 0) and noise photons (stream 1) of the same pictures
        sample_pictures(basis, d_c.data_ptr(), KMAX, LMAX, dq, qcut, qcut / 3.0, number_incident_photons, Imax,
                        seed, done, n, max_out, phs[0].data_ptr(), cnt[0].data_ptr(),
                        incident_photon_variance, beamstop_width, 0, lambda_)
        if with_noise:
            sample_pictures(basis, d_cn.data_ptr(), KMAX, LMAX, dq, qcut, noise.sigma * 1.05, noise.photons, Imax_n,
                            seed, done, n, max_out, phs[1].data_ptr(), cnt[1].data_ptr(),
                            0, beamstop_width, 1, lambda_)
        basis.sync()  # the sampled photons and counts before PyTorch compacts them
        counts = cnt[:, :n].to(torch.int64)
        ar = torch.arange(max_out, device=dev)[None, :]
        # per picture: its molecule photons, then its noise photons
        ph = torch.cat([x[:n] for x in phs], dim=1)
        mask = torch.cat([ar < counts[q][:, None] for q in range(nsl)], dim=1)
        flat = ph[mask].contiguous()
        counts = counts.sum(0)
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
