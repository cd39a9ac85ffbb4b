"""GPU parity of libtp3 against the oracle, called through the C ABI.

Tolerances:
  c3 relative L1 vs the reference-form restatement   <= 1e-5  (tests/test_cuda.jl:15)
  energy relative vs the reference-form restatement  <= 1e-6  (tests/test_cuda.jl:34)
  c3 max / RMS error vs the FP64 oracle are asserted below stated bounds.
"""
import numpy as np
import pytest

import tp3
from tp3 import _lib
from oracle.basis import enumerate_basis, lt_form_F
from oracle.c3 import triple_products, c3_lt_form, energy_bayes

pytestmark = pytest.mark.gpu

MODES = [tp3.TP3_MODE_PLAIN_FP32, tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3]


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


@pytest.fixture(scope="module")
def basis1(config1):
    p = config1["params"]
    b = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    yield b
    b.close()


@pytest.mark.parametrize("mode", MODES)
def test_triple_products_config1(basis1, config1, mode):
    """Stage (a) alone: T = sum_j w_j Re(c c c) per (shell triple, l-triple)."""
    basis1.set_mode(mode)
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    T64 = triple_products(b, config1["coeff"])
    T = basis1.triple_products(config1["coeff"]).astype(np.float64)
    scale = np.abs(T64).max(axis=1, keepdims=True)
    assert np.max(np.abs(T - T64) / scale) < 2e-5


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("kind", ["general", "real_function"])
def test_triple_products_random(basis1, config1, mode, kind):
    """Stage (a) on random coefficients: arbitrary complex ones (general path) and ones
    of a real function, c[l,-m] = (-1)^m conj(c[l,m]) (the symmetric path)."""
    basis1.set_mode(mode)
    p = config1["params"]
    LMAX = p["LMAX"]
    rng = np.random.default_rng(11)
    c = rng.normal(size=(p["K"], LMAX * LMAX)) + 1j * rng.normal(size=(p["K"], LMAX * LMAX))
    if kind == "real_function":
        from tp3.structure import seanindex0
        for l in range(LMAX):
            c[:, seanindex0(l, 0, LMAX)] = c[:, seanindex0(l, 0, LMAX)].real
            for m in range(1, l + 1):
                c[:, seanindex0(l, -m, LMAX)] = (-1) ** m * np.conj(c[:, seanindex0(l, m, LMAX)])
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    T64 = triple_products(b, c)
    T = basis1.triple_products(c).astype(np.float64)
    assert np.max(np.abs(T - T64)) / np.abs(T64).max() < 2e-5


@pytest.mark.parametrize("mode", MODES)
def test_c3_config1(basis1, config1, mode):
    basis1.set_mode(mode)
    vol = tp3.SphericalHarmonicsVolume(config1["coeff"], 9, 8, 8.0)
    c3 = tp3.FullCorrelation_parallized(vol, basis1, True, False, True)
    assert c3.shape == config1["c3_fp64"].shape
    assert rel_l1(c3, config1["c3_refform"]) <= 1e-5
    err = np.abs(c3 - config1["c3_fp64"]) / np.abs(config1["c3_fp64"]).max()
    assert err.max() < 1e-5 and np.sqrt(np.mean(err ** 2)) < 2e-6


@pytest.mark.parametrize("mode", MODES)
def test_c3_matches_reference_cuda_kernel(basis1, config1, mode):
    """libtp3's c3 vs the reference's own CUDA kernel + SGEMM output (golden fixture)."""
    import os
    basis1.set_mode(mode)
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "config1_refcuda.npz"))["c3_refcuda"]
    c3 = basis1.c3_raw(config1["coeff"]).astype(np.float64)
    assert rel_l1(c3, ref.astype(np.float64)) <= 1e-5


@pytest.mark.parametrize("mode", MODES)
def test_energy_config1(basis1, config1, config1_hist, mode):
    basis1.set_mode(mode)
    vol = tp3.SphericalHarmonicsVolume(config1["coeff"], 9, 8, 8.0)
    E = tp3.energy(vol, basis1, config1_hist)
    assert E == pytest.approx(float(config1["E_refform"]), rel=1e-6)
    assert E == pytest.approx(float(config1["E_fp64"]), rel=1e-6)


@pytest.mark.parametrize("mode", MODES)
def test_energy_batch_matches_single(basis1, config1, config1_hist, mode):
    basis1.set_mode(mode)
    basis1.set_histogram(config1_hist)
    rng = np.random.default_rng(7)
    coeffs = np.stack([config1["coeff"] * (1 + 0.05 * rng.normal(size=config1["coeff"].shape)) for _ in range(5)])
    Eb = basis1.energy_batch(coeffs)
    Es = np.array([basis1.energy_batch(c[None])[0] for c in coeffs])
    np.testing.assert_array_equal(Eb, Es)  # deterministic, order-independent per proposal
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    F = lt_form_F(b)
    for c, e in zip(coeffs, Eb):
        e64 = energy_bayes(c3_lt_form(F, triple_products(b, c)), config1_hist, p["K"], p["N"])
        assert e == pytest.approx(e64, rel=1e-6)


@pytest.mark.parametrize("mode", MODES)
def test_energy_batch_chunked(basis1, config1, config1_hist, mode):
    """Batches of >= 32 are packed and copied in chunks; each energy must not depend on it."""
    basis1.set_mode(mode)
    basis1.set_histogram(config1_hist)
    rng = np.random.default_rng(9)
    coeffs = np.stack([config1["coeff"] * (1 + 0.02 * rng.normal(size=config1["coeff"].shape)) for _ in range(37)])
    Eb = basis1.energy_batch(coeffs)
    Es = np.array([basis1.energy_batch(c[None])[0] for c in coeffs])
    np.testing.assert_array_equal(Eb, Es)


def test_energy_deterministic(basis1, config1, config1_hist):
    basis1.set_histogram(config1_hist)
    E1 = basis1.energy_batch(config1["coeff"][None])
    E2 = basis1.energy_batch(config1["coeff"][None])
    assert E1[0] == E2[0]


def test_errors_are_statuses(config1):
    p = config1["params"]
    b = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    with pytest.raises(tp3.TP3Error) as e:
        b.energy_batch(config1["coeff"][None])
    assert e.value.status == _lib.TP3_ERR_NO_HISTOGRAM
    bad = np.ones((p["N"], 2 * p["N"], p["K"], p["K"], p["K"]))
    bad[0, 0, 0, 0, 0] = np.nan
    with pytest.raises(tp3.TP3Error) as e:
        b.set_histogram(bad)
    assert e.value.status == _lib.TP3_ERR_BAD_HISTOGRAM
    zero = np.ones((p["N"], 2 * p["N"], p["K"], p["K"], p["K"]))
    zero[:, :, 1, 1, 2] = 0.0
    with pytest.raises(tp3.TP3Error) as e:
        b.set_histogram(zero)
    assert e.value.status == _lib.TP3_ERR_BAD_HISTOGRAM
    small = np.ones((p["N"], 2 * p["N"], p["K"] - 1, p["K"] - 1, p["K"] - 1))
    with pytest.raises(tp3.TP3Error) as e:
        b.set_histogram(small)
    assert e.value.status == _lib.TP3_ERR_ARG
    b.close()
    with pytest.raises(tp3.TP3Error):
        tp3.calculate_basis(8, 8, 16, 8)  # LMAX must exceed L


@pytest.mark.parametrize("form", [0, 1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("kind", ["general", "real_function"])
def test_coupling_forms_agree(basis1, config1, config1_hist, form, kind):
    """Every coupling form the autotuner may pick (one-kernel 512 threads, split, one-kernel
    256 threads x 2 CTAs per SM, warp-local 512 threads, warp-local 256 threads x 2 CTAs
    per SM, folded-row 8, 7 and 13 warps and 14 warps in pairs) gives the oracle's
    triple products and the same energy."""
    basis1.set_mode(tp3.TP3_MODE_TC_BF16X3)
    basis1.set_coupling(form)
    p = config1["params"]
    LMAX = p["LMAX"]
    rng = np.random.default_rng(form + 7)
    c = rng.normal(size=(p["K"], LMAX * LMAX)) + 1j * rng.normal(size=(p["K"], LMAX * LMAX))
    if kind == "real_function":
        from tp3.structure import seanindex0
        for l in range(LMAX):
            c[:, seanindex0(l, 0, LMAX)] = c[:, seanindex0(l, 0, LMAX)].real
            for m in range(1, l + 1):
                c[:, seanindex0(l, -m, LMAX)] = (-1) ** m * np.conj(c[:, seanindex0(l, m, LMAX)])
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    T64 = triple_products(b, c)
    T = basis1.triple_products(c).astype(np.float64)
    assert np.max(np.abs(T - T64)) / np.abs(T64).max() < 2e-5
    basis1.set_histogram(config1_hist)
    E = basis1.energy_batch(config1["coeff"][None, : p["K"]])[0]
    assert E == pytest.approx(float(config1["E_fp64"]), rel=1e-6)
    basis1.set_coupling(0)


@pytest.mark.parametrize("mode", [tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3])
@pytest.mark.parametrize("form", [0, 6])
def test_angular_schedules_agree(basis1, config1, config1_hist, mode, form):
    """The persistent angular schedule (one CTA per SM over (proposal, tile, half) units,
    two TMEM accumulators) and the one-CTA-per-tile schedule score alike: 400 proposals
    give every CTA more than two units, so both accumulators are reused.  Form 6 feeds
    the order-major T (MN-major A operand in BF16 mode), form 0 the K-major one."""
    basis1.set_mode(mode)
    basis1.set_coupling(form)
    basis1.set_histogram(config1_hist)
    rng = np.random.default_rng(11)
    coeffs = np.stack([config1["coeff"] * (1 + 0.03 * rng.normal(size=config1["coeff"].shape)) for _ in range(400)])
    basis1.set_angular(tp3.TP3_ANGULAR_PERSISTENT)
    Ep = basis1.energy_batch(coeffs)
    basis1.set_angular(tp3.TP3_ANGULAR_TILE)
    Et = basis1.energy_batch(coeffs)
    basis1.set_angular(tp3.TP3_ANGULAR_PERSISTENT)
    basis1.set_coupling(0)
    np.testing.assert_allclose(Ep, Et, rtol=5e-7)  # FP32 partial sums in another order
    p = config1["params"]
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    F = lt_form_F(b)
    for i in (0, 137, 399):
        e64 = energy_bayes(c3_lt_form(F, triple_products(b, coeffs[i])), config1_hist, p["K"], p["N"])
        assert Ep[i] == pytest.approx(e64, rel=1e-6)


def test_host_input_routes_agree(basis1, config1, config1_hist):
    """tp3_energy_batch reading the host array in place (where the device reads pageable
    host memory) and through host packing + a pinned copy give identical energies."""
    basis1.set_mode(tp3.TP3_MODE_TC_BF16X3)
    basis1.set_histogram(config1_hist)
    rng = np.random.default_rng(13)
    coeffs = np.stack([config1["coeff"] * (1 + 0.03 * rng.normal(size=config1["coeff"].shape)) for _ in range(70)])
    basis1.set_host_input(tp3.TP3_HOST_INPUT_STAGED)
    Es = basis1.energy_batch(coeffs)
    try:
        basis1.set_host_input(tp3.TP3_HOST_INPUT_DIRECT)
    except tp3.TP3Error:
        pytest.skip("this device does not read pageable host memory")
    Ed = basis1.energy_batch(coeffs)
    np.testing.assert_array_equal(Ed, Es)
    with pytest.raises(tp3.TP3Error):
        basis1.set_host_input(5)


def test_angular_schedule_argument_checked(basis1):
    with pytest.raises(tp3.TP3Error):
        basis1.set_angular(2)


def test_bounded_wait_reports_timeout_and_context_stays_usable(basis1, config1, config1_hist):
    """Failure detection without a fault: a device wait on a flag nothing sets runs out
    after ~5 ms, the status reaches the host as TP3_ERR_TIMEOUT at the next synchronising
    call, and the context then scores correctly again."""
    lib = tp3.load()
    basis1.set_histogram(config1_hist)
    assert lib.tp3_selftest_timeout(basis1.ctx, 10_000_000) == 0
    with pytest.raises(tp3.TP3Error) as ei:
        basis1.sync()
    assert ei.value.status == _lib.TP3_ERR_TIMEOUT
    p = config1["params"]
    E = basis1.energy_batch(config1["coeff"][None, : p["K"]])[0]
    assert E == pytest.approx(float(config1["E_fp64"]), rel=1e-6)


def test_stage_timing_and_fp32_peak(basis1, config1, config1_hist):
    """Per-stage CUDA-event timing counts one coupling and one angular launch per batch in
    a tensor-core mode, and the measured FP32 FMA peak is a plausible GB300 figure
    (nominal 152 SMs x 128 FMA/clock x 2.07 GHz = 80.5 TFLOP/s)."""
    p = config1["params"]
    basis1.set_histogram(config1_hist)
    basis1.set_mode(tp3.TP3_MODE_TC_BF16X3)
    basis1.set_coupling(0)
    batch = np.repeat(config1["coeff"][None, : p["K"]], 4, axis=0)
    basis1.energy_batch(batch)
    basis1.profile_enable(True)
    for _ in range(3):
        basis1.energy_batch(batch)
    n_a, ms_a = basis1.profile_read(0)
    n_c, ms_c = basis1.profile_read(1)
    basis1.profile_enable(False)
    assert n_a == 3 and n_c == 3 and ms_a > 0 and ms_c > 0
    peak = basis1.measure_fp32_peak()
    assert 40.0 < peak < 120.0, peak
