"""Histogram synthesis on the GPU end to end: photons sampled from a molecule's SH
intensity and binned all-to-all give a histogram whose slabs follow the model c3 and
against which the true structure scores better than shell-rotated ones."""
import math

import numpy as np
import pytest

import tp3

pytestmark = pytest.mark.gpu


def test_sampled_histogram_follows_model(config1):
    from tp3.datagen import generateHistogram, countTriplets
    from tp3.structure import loadHistograms, raw_to_5d
    from tp3.learned import rotated_starts
    p = config1["params"]
    L, LMAX, N, K = p["L"], p["LMAX"], p["N"], p["K"]
    coeff = config1["coeff"]                      # shells at |q| = k pi / rmax (rmax = 8)
    dq = math.pi / 8.0
    basis = tp3.calculate_basis(L, LMAX, N, K)
    c1, c2, c3 = generateHistogram(basis, coeff, dq, qcut=K * dq, K2=K, K3=K, N=N, pictures=20000,
                                   number_incident_photons=300, seed=11)
    ntrip = countTriplets(c3)
    assert ntrip > 1e7
    hist = loadHistograms(c3, K)
    model = raw_to_5d(basis.c3_raw(coeff[:K]).astype(np.float64), K, N)
    # slab shapes: correlation of the normalised histogram and model slabs, weighted by counts
    corr, wts = [], []
    for k1 in range(K):
        for k2 in range(k1 + 1):
            for k3 in range(k2 + 1):
                h = hist[:, :, k3, k2, k1].ravel()
                m = model[:, :, k3, k2, k1].ravel()
                corr.append(np.corrcoef(h, m)[0, 1])
                wts.append(c3[:, :, k3, k2, k1].sum())
    corr, wts = np.array(corr), np.array(wts)
    assert np.average(corr, weights=wts) > 0.9
    # the true structure scores better than per-shell rotated ones
    basis.set_histogram(hist)
    E_true = basis.energy_batch(coeff[None, :K])[0]
    E_rot = basis.energy_batch(rotated_starts(basis, coeff, 8, 3))
    assert E_true < E_rot.min()
    basis.close()


def _sample(basis, coeff, dq, qcut, sigma, incident, n, seed, variance=0, beamstop=0.0, stream=0, max_out=1024):
    import torch
    from tp3.datagen import sample_pictures, intensity_max
    c = np.ascontiguousarray(coeff, dtype=np.complex128)
    KMAX, LMAX = c.shape[0], int(round(math.sqrt(c.shape[1])))
    d_c = torch.from_numpy(c.view(np.float64).copy()).cuda()
    ph = torch.empty((n, max_out, 2), dtype=torch.float64, device="cuda")
    cnt = torch.empty(n, dtype=torch.int32, device="cuda")
    Imax = intensity_max(basis, c, dq)
    sample_pictures(basis, d_c.data_ptr(), KMAX, LMAX, dq, qcut, sigma, incident, Imax, seed, 0, n, max_out,
                    ph.data_ptr(), cnt.data_ptr(), variance, beamstop, stream)
    basis.sync()
    counts = cnt.cpu().numpy()
    assert counts.max() < max_out
    photons = ph.cpu().numpy()
    return counts, [photons[i, :counts[i]] for i in range(n)]


def test_picture_model_photon_variance_beamstop_and_noise():
    """The rest of generateHistogram's picture model (src/datagen.jl:88-113, 397-405) on the
    device: with a flat intensity every incident photon inside qcut is kept, so
    (a) incident_photon_variance gives per-picture counts of mean n and spread variance,
    (b) the beamstop keeps only photons with |x| and |y| above its width, in the Gaussian
        share (2 (1 - Phi(w / sigma)))^2,
    (c) GaussianNoise photons (stream 1, envelope 1.05 sigma) arrive at the rate the noise
        intensity predicts, and the molecule's stream is unchanged by them,
    (d) pictures of molecule plus noise photons bin on the device exactly as in the oracle."""
    from scipy.stats import norm
    from tp3.datagen import noise_coefficients, histogram_pictures
    from tp3.structure import seanindex0
    from oracle import histogram as oh
    basis = tp3.calculate_basis(2, 3, 4, 2)
    KMAX, LMAX, dq = 8, 3, 0.5
    qcut, sigma = KMAX * dq, 0.5
    flat = np.zeros((KMAX, LMAX * LMAX), dtype=np.complex128)
    flat[:, seanindex0(0, 0, LMAX)] = 1.0
    try:
        # (a) variable incident photon counts
        counts, _ = _sample(basis, flat, dq, qcut, sigma, 400, 4000, seed=5, variance=40)
        assert abs(counts.mean() - 400.0) < 5 * 40 / math.sqrt(4000)
        assert 36.0 < counts.std() < 44.0
        # (b) beamstop
        w = 0.1
        counts, pics = _sample(basis, flat, dq, qcut, sigma, 400, 2000, seed=6, beamstop=w)
        allp = np.concatenate(pics)
        assert np.all(np.abs(allp[:, 0]) > w) and np.all(np.abs(allp[:, 1]) > w)
        share = (2.0 * (1.0 - norm.cdf(w / sigma))) ** 2
        assert abs(counts.mean() / 400.0 - share) < 5 * math.sqrt(share * (1 - share) / 400 / 2000) + 1e-3
        # (c) noise photons: expected acceptance of the noise intensity
        sn = 1.0
        cn = noise_coefficients(KMAX, LMAX, dq, sn)
        c00 = cn[:, seanindex0(0, 0, LMAX)].real
        s = 1.05 * sn
        r = np.linspace(0.0, qcut, 200001)
        t = r / dq
        k0 = np.floor(t).astype(int)
        wgt = t - k0
        low, high = k0 < 1, k0 >= KMAX
        k0 = np.clip(k0, 1, KMAX)
        wgt[low | high] = 0.0
        k1 = np.minimum(k0 + 1, KMAX)
        I = (1 - wgt) * c00[k0 - 1] + wgt * c00[k1 - 1]
        ratio = I / c00.max() * np.exp(r * r / (2 * s * s))
        dens = r / (s * s) * np.exp(-r * r / (2 * s * s))
        f = dens * np.minimum(1.0, ratio)
        p_acc = float(np.sum(0.5 * (f[1:] + f[:-1]) * np.diff(r)))
        nph = 300
        counts_n, pics_n = _sample(basis, cn, dq, qcut, s, nph, 4000, seed=7, stream=1)
        expect = nph * p_acc
        assert abs(counts_n.mean() - expect) < 5 * math.sqrt(expect * (1 - p_acc) / 4000) + 0.05
        counts_a, pics_a = _sample(basis, flat, dq, qcut, sigma, 400, 50, seed=7, stream=0)
        counts_b, pics_b = _sample(basis, flat, dq, qcut, sigma, 400, 50, seed=7, stream=0)
        # the same photons (their order within a picture follows the device's slot claims)
        srt = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]
        assert np.array_equal(counts_a, counts_b)
        assert all(np.array_equal(srt(a), srt(b)) for a, b in zip(pics_a, pics_b))
        # (d) merged pictures bin exactly as in the oracle (the oracle bins all triplets in
        # Python, so each picture keeps 25 molecule and 15 noise photons)
        merged = [np.concatenate([a[:25], b[:15]]) for a, b in zip(pics_a[:20], pics_n[:20])]
        N, K2, K3, dqh = 8, KMAX, 6, dq
        c1 = np.zeros(K2); c2 = np.zeros((N, K2, K2)); c3 = np.zeros((N, 2 * N, K3, K3, K3))
        for pic in merged:
            oh.bin_picture(pic, dqh, N, K2, K3, c1, c2, c3)
        n1, n2, n3 = histogram_pictures(basis, merged, dqh, N, K2, K3, return_counts=True)
        np.testing.assert_array_equal(n1, c1)
        np.testing.assert_array_equal(n2, c2)
        np.testing.assert_array_equal(n3, c3)
    finally:
        basis.close()


def test_generate_histogram_with_noise_adds_noise_triplets(config1):
    """generateHistogram with GaussianNoise: the molecule's photons are drawn exactly as
    without noise (their stream is unchanged), so the noisy histogram counts are the
    clean ones plus the noise photons' contribution: more triplets, the same pictures."""
    from tp3.datagen import generateHistogram, countTriplets, GaussianNoise
    p = config1["params"]
    L, LMAX, N, K = p["L"], p["LMAX"], p["N"], p["K"]
    coeff = config1["coeff"]
    dq = math.pi / 8.0
    basis = tp3.calculate_basis(L, LMAX, N, K)
    try:
        kw = dict(qcut=K * dq, K2=K, K3=K, N=N, pictures=2000, number_incident_photons=300, seed=13,
                  return_counts=True, beamstop_width=0.05)
        n1, n2, n3 = generateHistogram(basis, coeff, dq, **kw)
        m1, m2, m3 = generateHistogram(basis, coeff, dq, noise=GaussianNoise(1.0, 1.5, 150), **kw)
        z1, z2, z3 = generateHistogram(basis, coeff, dq, noise=GaussianNoise(1.0, 1.5, 0), **kw)
        assert np.array_equal(z3, n3)          # no noise photons: identical histogram
        assert m1.sum() > n1.sum() and m3.sum() > n3.sum()
        assert np.all(m1 >= n1)                # every molecule photon is still there
    finally:
        basis.close()
