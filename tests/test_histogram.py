"""Triplet histograms of photon pictures: the binning oracle's known answers on the CPU
(KAT-5: countTriplets of the weighted histogram is the number of binned triplets) and
the device binning against the oracle, count for count (GPU)."""
import math

import numpy as np
import pytest

from oracle import histogram as oh


def _pictures(n, seed, qcut=1.0, photons=(3, 40)):
    rng = np.random.default_rng(seed)
    pics = []
    for _ in range(n):
        m = int(rng.integers(*photons))
        r = qcut * np.sqrt(rng.uniform(0, 1, m))
        a = rng.uniform(0, 2 * math.pi, m)
        pics.append(np.stack([r * np.cos(a), r * np.sin(a)], axis=1))
    return pics


def test_kat5_count_triplets_matches_binned_triplets():
    N, K2, K3, dq = 8, 10, 7, 0.1
    c1 = np.zeros(K2); c2 = np.zeros((N, K2, K2)); c3 = np.zeros((N, 2 * N, K3, K3, K3))
    total = sum(oh.bin_picture(p, dq, N, K2, K3, c1, c2, c3) for p in _pictures(20, 1))
    assert total > 1000
    _, _, w3 = oh.weights(c1, c2, c3)
    assert oh.countTriplets(w3) == pytest.approx(total, rel=1e-12)
    assert c3.sum() == total


def test_angle_between_conventions():
    assert oh.angle_between([1.0, 0.0], [0.0, 1.0]) == 0.0          # exactly perpendicular: 0
    a = oh.angle_between([1.0, 0.0], [1.0, 1.0])
    assert a == pytest.approx(2 * math.pi - math.pi / 4)             # counter-clockwise: mirrored
    assert oh.angle_between([1.0, 1.0], [1.0, 0.0]) == pytest.approx(math.pi / 4)


@pytest.mark.gpu
def test_device_binning_matches_oracle():
    import tp3
    from tp3.datagen import histogram_pictures, countTriplets
    N, K2, K3, dq = 8, 10, 7, 0.1
    pics = _pictures(60, 2, photons=(0, 60))
    c1 = np.zeros(K2); c2 = np.zeros((N, K2, K2)); c3 = np.zeros((N, 2 * N, K3, K3, K3))
    total = sum(oh.bin_picture(p, dq, N, K2, K3, c1, c2, c3) for p in pics)
    basis = tp3.calculate_basis(2, 3, 4, 2)
    n1, n2, n3 = histogram_pictures(basis, pics, dq, N, K2, K3, return_counts=True)
    np.testing.assert_array_equal(n1, c1)
    np.testing.assert_array_equal(n2, c2)
    np.testing.assert_array_equal(n3, c3)
    w1, w2, w3 = histogram_pictures(basis, pics, dq, N, K2, K3)
    assert countTriplets(w3) == pytest.approx(total, rel=1e-12)
    basis.close()
