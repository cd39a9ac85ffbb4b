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
