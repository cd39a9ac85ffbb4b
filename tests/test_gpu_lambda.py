"""Ewald curvature (lambda != 0): the Legendre factors depend on the shells, as in the
reference's own GPU test (tests/test_cuda.jl:2, lambda = 2.5).  Both paths contract over
Fourier pairs (m2, m3): the plain FP32 path with a SIMT angular kernel, the tensor-core
paths by building H[ki][(m2, m3)] from FP32 triple products and contracting it with the
cosine table on tcgen05 (the unfolded N x 2N grid, 2N^2 / 256 halves per tile).  Parity
against the oracle's reference form and FP64 pair form, at config 1 and at the
production shape (L18 K26 N32)."""
import math

import numpy as np
import pytest

import tp3
from oracle.basis import enumerate_basis, reference_tables
from oracle.c3 import c3_reference_form, c3_pair_form, c3_pair_form_fast, energy_bayes

pytestmark = pytest.mark.gpu

LAM, DQ = 2.5, math.pi / 8
MODES = [tp3.TP3_MODE_PLAIN_FP32, tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3]


@pytest.fixture(scope="module")
def lam_setup(config1):
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"], lam=LAM, dq=DQ)
    B32, P32 = reference_tables(b)
    c3r = c3_reference_form(b, config1["coeff"], B32, P32)
    c364 = c3_pair_form(b, config1["coeff"])
    basis = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"], LAM, DQ)
    yield basis, c3r, c364, p
    basis.close()


@pytest.mark.parametrize("mode", MODES)
def test_lambda_c3(lam_setup, config1, mode):
    basis, c3r, c364, p = lam_setup
    basis.set_mode(mode)
    c3 = basis.c3_raw(config1["coeff"]).astype(np.float64)
    assert np.abs(c3 - c3r).sum() / np.abs(c3r).sum() <= 1e-5
    err = np.abs(c3 - c364) / np.abs(c364).max()
    assert err.max() < 1e-5


def test_lambda_tensor_core_is_the_default(lam_setup):
    basis, _, _, _ = lam_setup
    basis.set_mode(tp3.TP3_MODE_AUTO)
    assert basis.mode == tp3.TP3_MODE_TC_BF16X3


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("schedule", [tp3.TP3_ANGULAR_PERSISTENT, tp3.TP3_ANGULAR_TILE])
def test_lambda_energy(lam_setup, config1, config1_hist, mode, schedule):
    basis, c3r, c364, p = lam_setup
    basis.set_mode(mode)
    if mode != tp3.TP3_MODE_PLAIN_FP32:
        basis.set_angular(schedule)  # N = 16: 512 grid points, both schedules fit
        basis.set_coupling(6 if schedule == tp3.TP3_ANGULAR_TILE else 0)
    E = tp3.energy(tp3.SphericalHarmonicsVolume(config1["coeff"], 9, 8, 8.0), basis, config1_hist)
    basis.set_angular(tp3.TP3_ANGULAR_PERSISTENT)
    assert E == pytest.approx(energy_bayes(c3r, config1_hist, p["K"], p["N"]), rel=1e-6)
    assert E == pytest.approx(energy_bayes(c364, config1_hist, p["K"], p["N"]), rel=1e-6)


def test_lambda_batches_agree_across_modes(lam_setup, config1, config1_hist):
    basis, _, _, p = lam_setup
    basis.set_histogram(config1_hist)
    rng = np.random.default_rng(3)
    coeffs = np.stack([config1["coeff"] * (1 + 0.05 * rng.normal(size=config1["coeff"].shape)) for _ in range(40)])
    out = {}
    for mode in MODES:
        basis.set_mode(mode)
        out[mode] = basis.energy_batch(coeffs)
    for mode in MODES[1:]:
        np.testing.assert_allclose(out[mode], out[tp3.TP3_MODE_PLAIN_FP32], rtol=2e-6)


def test_lambda_out_of_range_rejected(config1):
    p = config1["params"]
    with pytest.raises(tp3.TP3Error):
        tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"], 100.0, 1.0)


def test_lambda_production_shape_against_fp64():
    """L18 K26 N32 LMAX25 at lambda = 2.5 (dq = 0.15): 2 048 grid points in 8 halves per
    tile.  c3 of both tensor-core modes against the FP64 pair form
    (relative L1 <= 1e-5), and the energy of a batch against the FP64 energy (1e-6)."""
    from oracle.refcpu import triple_products_fast
    from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms
    L, LMAX, N, K, lam, dq = 18, 25, 32, 26, 2.5, 0.15
    coeff = intensity_coefficients(synthetic_molecule(327, seed=20240601), LMAX, 38, 38.0, kcount=K)[:K]
    ob = enumerate_basis(L, LMAX, N, K, lam=lam, dq=dq)
    c364 = c3_pair_form_fast(ob, triple_products_fast(ob, coeff))
    hist = loadHistograms(poisson_histogram(c364, K, N, 1e9, seed=11), K)
    E64 = energy_bayes(c364, hist, K, N)
    basis = tp3.calculate_basis(L, LMAX, N, K, lam, dq)
    try:
        basis.set_histogram(hist)
        with pytest.raises(tp3.TP3Error):
            basis.set_angular(tp3.TP3_ANGULAR_TILE)  # 2 048 grid points do not fit one CTA's TMEM
        for mode in (tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3):
            basis.set_mode(mode)
            for form in (0, 6):
                basis.set_coupling(form)
                c3 = basis.c3_raw(coeff).astype(np.float64)
                rel = np.abs(c3 - c364).sum() / np.abs(c364).sum()
                assert rel < 1e-5, (mode, form, rel)
                E = basis.energy_batch(np.stack([coeff] * 3))
                np.testing.assert_allclose(E, E64, rtol=1e-6)
    finally:
        basis.close()
