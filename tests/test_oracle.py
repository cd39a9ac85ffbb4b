"""The oracle pinned against the golden vectors, and its known-answer properties.

No GPU.  Golden vectors: sympy's exact 3j and scipy's spherical harmonics (the
two GSL routines the reference calls, src/spherical_harmonics.jl:63-76), basis
sizes of calculate_basis (src/correlations.jl:87-131), and the committed
config-1 fixture.
"""
import math

import numpy as np
import pytest

from oracle import sh
from oracle.basis import enumerate_basis, lt_form_F, reference_tables
from oracle.c3 import (triple_products, c3_lt_form, c3_reference_form, energy_bayes, slab_energies,
                       load_histogram)


def test_wigner3j_matches_sympy(golden_sh):
    for l1, l2, l3, m1, m2, m3, v in golden_sh["wigner3j"]:
        assert sh.wigner3j(l1, l2, l3, m1, m2, m3) == pytest.approx(v, abs=1e-15, rel=1e-13)


def test_sphPlm_matches_scipy(golden_sh):
    for l, m, th, v in golden_sh["sphPlm"]:
        assert sh.sphPlm(l, m, th) == pytest.approx(v, abs=1e-13)


def test_seanindex_layout():
    # m >= 0 blocks first (m = 0: l = 0..LMAX-1, then m = 1, ...), then m < 0: bijection onto 1..LMAX^2
    LMAX = 7
    idx = sorted(sh.seanindex(l, m, LMAX) for l in range(LMAX) for m in range(-l, l + 1))
    assert idx == list(range(1, LMAX * LMAX + 1))
    assert sh.seanindex(0, 0, LMAX) == 1 and sh.seanindex(LMAX - 1, 0, LMAX) == LMAX
    assert sh.seanindex(1, 1, LMAX) == LMAX + 1


@pytest.mark.parametrize("L,expect", [(8, (4583, 65)), (12, (26263, 175))])
def test_basis_sizes(L, expect):
    b = enumerate_basis(L, L + 1, 4, 2)
    assert (b.basislen, b.n_lt) == expect


def test_basis_rejects_small_lmax():
    with pytest.raises(ValueError):
        enumerate_basis(8, 8, 16, 8)


def test_config1_golden(config1, config1_hist):
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    assert b.basislen == int(config1["basislen"])
    T = triple_products(b, config1["coeff"])
    c3 = c3_lt_form(lt_form_F(b), T)
    np.testing.assert_allclose(c3, config1["c3_fp64"], rtol=1e-12, atol=0)
    E = energy_bayes(c3, config1_hist, p["K"], p["N"])
    assert E == pytest.approx(float(config1["E_fp64"]), rel=1e-12)


def test_reference_form_equals_lt_form(config1):
    """The reference's B * PA with f32 tables vs the FP64 l-triple regrouping."""
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    B32, P32 = reference_tables(b)
    c3r = c3_reference_form(b, config1["coeff"], B32, P32)
    np.testing.assert_allclose(c3r, config1["c3_refform"], rtol=1e-12)
    rel = np.abs(c3r - config1["c3_fp64"]).sum() / np.abs(config1["c3_fp64"]).sum()
    assert rel < 1e-6


def test_kat1_monopole_only_is_flat():
    """KAT-1: only l = 0 coefficients -> c3 constant over (alpha, beta) in every slab."""
    L, LMAX, N, K = 4, 5, 8, 3
    b = enumerate_basis(L, LMAX, N, K)
    rng = np.random.default_rng(0)
    coeff = np.zeros((K, LMAX * LMAX), complex)
    coeff[:, 0] = rng.uniform(1, 2, K)
    c3 = c3_lt_form(lt_form_F(b), triple_products(b, coeff))
    assert np.allclose(c3, c3[:1, :], rtol=1e-12)


def _wigner_D_real(l, R):
    """Rotation of real-valued SH coefficients by the rotation matrix R, by sampling."""
    # least-squares fit of rotated real SH on random directions (exact for band-limited data)
    rng = np.random.default_rng(l)
    n = rng.normal(size=(4 * (2 * l + 1) + 8, 3))
    n /= np.linalg.norm(n, axis=1)[:, None]

    def Ylm_complex(dirs):
        th = np.arccos(np.clip(dirs[:, 2], -1, 1))
        ph = np.arctan2(dirs[:, 1], dirs[:, 0])
        return np.stack([np.array([sh.sphPlm(l, m, t) for t in th]) * np.exp(1j * m * ph)
                         for m in range(-l, l + 1)], axis=1)
    Y = Ylm_complex(n)
    Yr = Ylm_complex(n @ R)  # f(R^T x) evaluated through Y(R^T n)
    D, *_ = np.linalg.lstsq(Y, Yr, rcond=None)
    return D  # f'(n) = sum_m c_m Y_m(R^T n) = sum_m' (D^T c)_m' Y_m'(n)


def test_kat2_common_rotation_invariance(config1):
    """KAT-2: one SO(3) rotation applied to every shell leaves c3 unchanged."""
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    coeff = config1["coeff"][: p["K"]].copy()
    rng = np.random.default_rng(3)
    Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(Q) < 0:
        Q[:, 0] *= -1
    rot = coeff.copy()
    for l in range(0, p["L"] + 1, 2):
        D = _wigner_D_real(l, Q)
        idx = [sh.seanindex(l, m, p["LMAX"]) - 1 for m in range(-l, l + 1)]
        rot[:, idx] = coeff[:, idx] @ D
    F = lt_form_F(b)
    c0 = c3_lt_form(F, triple_products(b, coeff))
    c1 = c3_lt_form(F, triple_products(b, rot))
    assert np.abs(c1 - c0).max() / np.abs(c0).max() < 1e-9


def test_kat3_per_l_rotation_keeps_power(config1):
    """KAT-3: a per-l SO(2l+1) rotation (the reference move) changes c3 but keeps
    sum_m |c_klm|^2 per (k, l)."""
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    coeff = config1["coeff"][: p["K"]].copy()
    rng = np.random.default_rng(5)
    new = coeff.copy()
    for l in range(2, p["L"] + 1, 2):
        Q, _ = np.linalg.qr(rng.normal(size=(2 * l + 1, 2 * l + 1)))
        rot = sh.Umat(l).conj().T @ Q @ sh.Umat(l)
        idx = [sh.seanindex(l, m, p["LMAX"]) - 1 for m in range(-l, l + 1)]
        new[:, idx] = (rot @ coeff[:, idx].T).T
        np.testing.assert_allclose(np.sum(np.abs(new[:, idx]) ** 2, 1), np.sum(np.abs(coeff[:, idx]) ** 2, 1),
                                   rtol=1e-12)
    F = lt_form_F(b)
    c0 = c3_lt_form(F, triple_products(b, coeff))
    c1 = c3_lt_form(F, triple_products(b, new))
    assert np.abs(c1 - c0).max() / np.abs(c0).max() > 1e-3


def test_kat4_perfect_model_gives_entropy(config1):
    """KAT-4: q = p -> each slab term is tf * H(q^)."""
    p = config1["params"]
    c3 = config1["c3_fp64"]
    hist = np.zeros((p["N"], 2 * p["N"], p["K"], p["K"], p["K"]), order="F")
    i = 0
    for k1 in range(1, p["K"] + 1):
        for k2 in range(1, k1 + 1):
            for k3 in range(1, k2 + 1):
                hist[:, :, k3 - 1, k2 - 1, k1 - 1] = c3[:, i].reshape(p["N"], 2 * p["N"], order="F")
                i += 1
    terms = slab_energies(c3, hist, p["K"], p["N"])
    i = 0
    for k1 in range(1, p["K"] + 1):
        for k2 in range(1, k1 + 1):
            for k3 in range(1, k2 + 1):
                q = c3[:, i] / c3[:, i].sum()
                assert terms[i] == pytest.approx(-np.sum(q * np.log(q)) * sh.tripletFactor(k1, k2, k3), rel=1e-12)
                i += 1


def test_histogram_contract():
    """loadHistograms: doubling N x N, clamp, cut to K3, global L1 normalisation."""
    rng = np.random.default_rng(0)
    raw = rng.poisson(3.0, size=(4, 4, 5, 5, 5)).astype(float)
    h = load_histogram(raw, 3)
    assert h.shape == (4, 8, 3, 3, 3)
    assert h.min() > 0 and abs(h.sum() - 1.0) < 1e-12
    np.testing.assert_allclose(h[:, :4], h[:, 4:])


def test_oracle_pinned_to_reference_cuda_kernel(config1):
    """The reference's own GPU path (src/cuda_kernel.cu + SGEMM, src/cuda.jl:74-108), run on
    a GB300 on the same coefficients and tables (tests/golden/make_refcuda_golden.py),
    against the oracle: relative L1 within the reference's own CPU-vs-GPU tolerance
    (tests/test_cuda.jl:15)."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "config1_refcuda.npz"))
    ref = d["c3_refcuda"].astype(np.float64)
    for mine in (config1["c3_refform"], config1["c3_fp64"]):
        assert np.abs(ref - mine).sum() / np.abs(mine).sum() < 1e-5


def test_kat6_lambda_forms_agree(config1):
    """KAT-6: at lambda = 2.5 (tests/test_cuda.jl:2) the reference's B * PA form and the
    Fourier-pair form agree."""
    import math
    from oracle.c3 import c3_pair_form
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"], lam=2.5, dq=math.pi / 8)
    B32, P32 = reference_tables(b)
    c3r = c3_reference_form(b, config1["coeff"], B32, P32)
    c3q = c3_pair_form(b, config1["coeff"])
    assert np.abs(c3r - c3q).sum() / np.abs(c3q).sum() < 1e-6


def test_pair_form_vectorised_equals_loop_form(config1):
    """The chunked pair form used at the production shape equals the per-entry loop form."""
    import math
    from oracle.c3 import c3_pair_form, c3_pair_form_fast, triple_products
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"], lam=2.5, dq=math.pi / 8)
    c3q = c3_pair_form(b, config1["coeff"])
    c3v = c3_pair_form_fast(b, triple_products(b, config1["coeff"]), chunk=333)
    assert np.abs(c3q - c3v).max() / np.abs(c3q).max() < 1e-13
