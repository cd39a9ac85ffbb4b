"""The production shape (L=18, K=26, N=32, LMAX=25): c3 against the FP64 oracle and the
reference-form CPU restatement (f32 tables, f64 accumulation) in every mode and coupling
form, the energy against the FP64 energy, and a short device chain against the FP64
oracle chain."""
import math

import numpy as np
import pytest

import tp3
from tp3.chains import Chains
from oracle import chain as oc
from oracle.basis import enumerate_basis, lt_form_F
from oracle.c3 import energy_bayes
from oracle.refcpu import RefCPU, triple_products_fast

pytestmark = pytest.mark.gpu

L, LMAX, N, K = 18, 25, 32, 26


@pytest.fixture(scope="module")
def prod():
    from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms
    coeff = intensity_coefficients(synthetic_molecule(327, seed=20240601), LMAX, 38, 38.0, kcount=K)[:K]
    ob = enumerate_basis(L, LMAX, N, K)
    F = lt_form_F(ob)
    c3_64 = F @ triple_products_fast(ob, coeff).T
    hist = loadHistograms(poisson_histogram(c3_64, K, N, 1e9, seed=7), K)
    basis = tp3.calculate_basis(L, LMAX, N, K)
    basis.set_histogram(hist)
    yield basis, coeff, ob, F, c3_64, hist
    basis.close()


def _e64(ob, F, hist, c):
    return energy_bayes(F @ triple_products_fast(ob, c).T, hist, K, N)


def test_c3_and_energy_all_modes(prod):
    basis, coeff, ob, F, c3_64, hist = prod
    ref = RefCPU(L, LMAX, N, K).c3(coeff)
    assert np.abs(ref - c3_64).sum() / np.abs(c3_64).sum() < 1e-7
    E64 = energy_bayes(c3_64, hist, K, N)
    variants = [(tp3.TP3_MODE_PLAIN_FP32, None)] + [(m, f) for m in (tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3)
                                                    for f in (0, 1, 3, 4, 5, 6, 7, 8)]
    for mode, form in variants:
        basis.set_mode(mode)
        if form is not None:
            basis.set_coupling(form)
        c3 = basis.c3_raw(coeff).astype(np.float64)
        rel = np.abs(c3 - ref).sum() / np.abs(ref).sum()
        assert rel < 1e-5, (mode, form, rel)
        E = basis.energy_batch(coeff[None])[0]
        assert E == pytest.approx(E64, rel=1e-6), (mode, form)
    basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
    basis.set_coupling(0)


@pytest.mark.parametrize("mode", [tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3])
def test_angular_schedules_at_production_shape(prod, mode):
    """Both grid halves (512 unique points) and 26 tiles per proposal: the persistent and
    per-tile angular schedules give the FP64 energy for 64 perturbed proposals."""
    basis, coeff, ob, F, c3_64, hist = prod
    basis.set_mode(mode)
    basis.set_coupling(6)
    rng = np.random.default_rng(5)
    coeffs = np.stack([coeff * (1 + 0.02 * rng.normal(size=coeff.shape)) for _ in range(64)])
    basis.set_angular(tp3.TP3_ANGULAR_PERSISTENT)
    Ep = basis.energy_batch(coeffs)
    basis.set_angular(tp3.TP3_ANGULAR_TILE)
    Et = basis.energy_batch(coeffs)
    basis.set_angular(tp3.TP3_ANGULAR_PERSISTENT)
    basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
    basis.set_coupling(0)
    np.testing.assert_allclose(Ep, Et, rtol=5e-7)  # FP32 partial sums in another order
    for i in (0, 63):
        assert Ep[i] == pytest.approx(_e64(ob, F, hist, coeffs[i]), rel=1e-6)


def test_short_chain_matches_fp64_chain(prod):
    basis, coeff, ob, F, c3_64, hist = prod
    seed = 0xC0FFEE
    T0 = 5.0
    ch = Chains(basis, coeff[None], T0, math.pi / 4, 1.02, 0.99, seed, ncand=4, log_capacity=64)
    ch.run(3)
    rows = ch.log(0)[:8]
    _, _, _, _, ref = oc.run_chain(lambda c: _e64(ob, F, hist, c), coeff, L, LMAX, T0, math.pi / 4, 1.02, 0.99,
                                   seed, 0, len(rows))
    tol = 2e-7 * abs(ref[0][3])
    for d, r in zip(rows, ref):
        s = int(r[0]) - 1
        u = oc.u01(oc.philox4x32_10((s, 0, 2, 0), (seed & oc.M32, seed >> 32))[0])
        if d[1] != r[1]:
            assert abs(r[4]) <= tol or abs(r[4] + r[5] * math.log(u)) <= tol
            break
        assert d[2] == pytest.approx(r[2], rel=1e-6)
    ch.close()
