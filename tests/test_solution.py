"""Start structures from two-photon correlations: the inversion recovers every shell
Gram matrix G_l[k1, k2] = sum_m c_k1lm conj(c_k2lm) of a band-limited intensity, and the
recovered coefficients reproduce the model c2 (host-side linear algebra); the rotation fit
on the host and (GPU) on the device."""
import math

import numpy as np
import pytest

from tp3.solution import twoPhotons, retrieveSolution
from tp3.structure import seanindex0


def _band_limited(K, LMAX, L, seed):
    """Real-function coefficients with shell k carrying orders l <= min(L, 2k - 2) only
    (the orders retrieveSolution fits for that shell)."""
    rng = np.random.default_rng(seed)
    c = np.zeros((K, LMAX * LMAX), dtype=np.complex128)
    for k in range(1, K + 1):
        for l in range(0, min(L, 2 * k - 2) + 1, 2):
            for m in range(0, l + 1):
                v = rng.normal() + (1j * rng.normal() if m else 0.0)
                c[k - 1, seanindex0(l, m, LMAX)] = v / (1 + l)
                if m:
                    c[k - 1, seanindex0(l, -m, LMAX)] = (-1) ** m * np.conj(v) / (1 + l)
        c[k - 1, seanindex0(0, 0, LMAX)] = 5.0 + k   # positive mean intensity
    return c


def _gram(c, l, LMAX, K):
    idx = [seanindex0(l, m, LMAX) for m in range(-l, l + 1)]
    return (c[:K, idx] @ c[:K, idx].conj().T).real


def test_retrieve_solution_recovers_gram_matrices_and_c2():
    K, LMAX, L, N = 12, 9, 4, 32
    dq = 0.3
    c = _band_limited(K, LMAX, L, 3)
    c2 = twoPhotons(c, LMAX, L, N, K, dq)
    r = retrieveSolution(c2, L, LMAX, range(1, K + 1), K * dq)
    for l in range(0, L + 1, 2):
        np.testing.assert_allclose(_gram(r, l, LMAX, K), _gram(c, l, LMAX, K), atol=1e-9 * np.abs(_gram(c, 0, LMAX, K)).max())
    np.testing.assert_allclose(twoPhotons(r, LMAX, L, N, K, dq), c2, atol=1e-10 * np.abs(c2).max())
    # a real function again: c[l,-m] = (-1)^m conj(c[l,m])
    for l in range(0, L + 1, 2):
        for m in range(1, l + 1):
            np.testing.assert_allclose(r[:, seanindex0(l, -m, LMAX)], (-1) ** m * np.conj(r[:, seanindex0(l, m, LMAX)]),
                                       atol=1e-12)


def test_similarity_and_rotation_fit(config1):
    from tp3.postprocess import similarity, fitStructures_random, rotateStructure
    p = config1["params"]
    LMAX, K, L = p["LMAX"], p["K"], p["L"]
    c = config1["coeff"][:K]
    assert abs(similarity(c, c, LMAX, range(1, K + 1)) - 1) < 1e-12
    from tp3.postprocess import _rotation_matrix
    import tp3
    for l in (2, 5, 8):
        np.testing.assert_allclose(_rotation_matrix(0.7, -1.2, 2.1, l), tp3.rotationMatrix(0.7, -1.2, 2.1, l), atol=1e-13)
    rot = rotateStructure(c, 1.1, 0.4, -0.7, K, range(2, L + 1, 2), LMAX)
    s_rot = similarity(c, rot, LMAX, range(2, K + 1))
    assert s_rot < 0.99
    fitted, best, *_ = fitStructures_random(rot, c, LMAX, range(2, K + 1), L, 0.99, repetitions=8, seed=1)
    assert best > 0.995 and best > s_rot
    assert abs(similarity(c, fitted, LMAX, range(2, K + 1)) - best) < 1e-12


def test_fit_draws_follow_the_host_search_order():
    """The device search is fed the host search's random numbers in its order."""
    from tp3.postprocess import fit_draws
    d = fit_draws(3, 0.9, seed=4)
    rng = np.random.default_rng(4)
    S = (d.shape[1] - 3) // 3
    assert S > 0 and math.pi * 0.9 ** S <= math.pi / 180 < math.pi * 0.9 ** (S - 1)
    for r in range(3):
        np.testing.assert_array_equal(d[r, :3], [rng.random() for _ in range(3)])
        np.testing.assert_array_equal(d[r, 3:], [rng.normal() for _ in range(3 * S)])


@pytest.mark.gpu
def test_device_fit_matches_host_fit(config1):
    """tp3_fit_structures_random walks the same restarts as the host search: the same best
    rotation, the similarity to 1e-10, and the rotated structure (shells 1..max(K_range),
    orders 2:2:L) to 1e-10."""
    import tp3
    from tp3.postprocess import fitStructures_random, rotateStructure, similarity
    p = config1["params"]
    LMAX, K, L = p["LMAX"], p["K"], p["L"]
    c = config1["coeff"][:K]
    rot = rotateStructure(c, 1.1, 0.4, -0.7, K, range(2, L + 1, 2), LMAX)
    basis = tp3.calculate_basis(L, LMAX, p["N"], K)
    try:
        for K_range in (range(2, K + 1), range(1, K - 2)):
            h = fitStructures_random(rot, c, LMAX, K_range, L, 0.97, repetitions=6, seed=3)
            d = fitStructures_random(rot, c, LMAX, K_range, L, 0.97, repetitions=6, seed=3, basis=basis)
            assert abs(d[1] - h[1]) < 1e-10
            np.testing.assert_allclose(d[2:], h[2:], atol=1e-12)
            scale = np.abs(h[0]).max()
            assert np.abs(d[0] - h[0]).max() < 1e-10 * scale
            assert abs(similarity(c, d[0], LMAX, K_range) - d[1]) < 1e-10
    finally:
        basis.close()


@pytest.mark.gpu
def test_device_retrieve_solution_matches_host(config1):
    """tp3_retrieve_solution: the same least-squares Gram matrices, eigenpairs (signs fixed
    the same way) and negativity flip as the host inversion, so the same coefficients; at
    lambda = 0 and lambda = 1.2."""
    import tp3
    p = config1["params"]
    basis = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    try:
        for K, LMAX, L, N, lam in ((12, 9, 4, 24, 0.0), (16, 11, 6, 32, 1.2)):
            c = _band_limited(K, LMAX, L, seed=K)
            qmax = 8.0
            c2 = twoPhotons(c, LMAX, L, N, K, qmax / K, lam)
            h = retrieveSolution(c2, L, LMAX, range(1, K + 1), qmax, lam)
            d = retrieveSolution(c2, L, LMAX, range(1, K + 1), qmax, lam, basis=basis)
            np.testing.assert_allclose(d, h, atol=1e-9 * np.abs(h).max())
    finally:
        basis.close()

