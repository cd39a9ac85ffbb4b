"""Ewald curvature (lambda != 0): the Legendre factors depend on the shells, as in the
reference's own GPU test (tests/test_cuda.jl:2, lambda = 2.5).  The plain path contracts
over Fourier pairs (m2, m3); parity against the oracle's reference form and FP64 form."""
import math

import numpy as np
import pytest

import tp3
from oracle.basis import enumerate_basis, reference_tables
from oracle.c3 import c3_reference_form, c3_pair_form, energy_bayes

pytestmark = pytest.mark.gpu

LAM, DQ = 2.5, math.pi / 8


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


def test_lambda_c3(lam_setup, config1):
    basis, c3r, c364, p = lam_setup
    assert basis.mode == tp3.TP3_MODE_PLAIN_FP32  # the tensor-core path needs lambda = 0
    c3 = basis.c3_raw(config1["coeff"]).astype(np.float64)
    assert np.abs(c3 - c3r).sum() / np.abs(c3r).sum() <= 1e-5
    err = np.abs(c3 - c364) / np.abs(c364).max()
    assert err.max() < 1e-5


def test_lambda_energy(lam_setup, config1, config1_hist):
    basis, c3r, c364, p = lam_setup
    E = tp3.energy(tp3.SphericalHarmonicsVolume(config1["coeff"], 9, 8, 8.0), basis, config1_hist)
    assert E == pytest.approx(energy_bayes(c3r, config1_hist, p["K"], p["N"]), rel=1e-6)


def test_lambda_out_of_range_rejected(config1):
    p = config1["params"]
    with pytest.raises(tp3.TP3Error):
        tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"], 100.0, 1.0)
