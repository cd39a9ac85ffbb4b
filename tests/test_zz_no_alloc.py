"""The allocation-free scoring entry point, checked against the context path.

tp3_bayes_energy_noalloc serves callers that may not allocate device memory when
they score: a Julia host whose CUDA.jl pool owns the device memory, runtimes with a
device-memory budget granted up front, loops that must not stall on cudaMalloc's
synchronisation.  Here its energy of a c3 produced by tp3_c3 must match tp3_energy
of the same coefficients within the energy tolerance used throughout (1e-6
relative), on two calls in a row with different inputs, so a call cannot lean on
what the previous one left in the shared scratch.  Checked at the small shape
(L8 K8 N16) and at the production shape (L18 K26 N32, 3 276 slabs of 2 048 grid
points, where the per-slab sums are longest).  This file sorts last so that a stop
at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import tp3

pytestmark = pytest.mark.gpu


def _qhat(hist, K, N):
    slabs = []
    for k1 in range(1, K + 1):
        for k2 in range(1, k1 + 1):
            for k3 in range(1, k2 + 1):
                q = hist[:, :, k3 - 1, k2 - 1, k1 - 1].reshape(-1, order="F")
                slabs.append(q / np.sum(np.abs(q)))
    return np.ascontiguousarray(np.stack(slabs), dtype=np.float32)


def _two_calls(basis, hist, base, K, N, seed):
    torch = pytest.importorskip("torch")
    lib = tp3.load()
    rng = np.random.default_rng(seed)
    sets = [base, base * (1 + 0.05 * rng.normal(size=base.shape))]
    q = torch.from_numpy(_qhat(hist, K, N)).cuda()
    d_E = torch.empty(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    energies = []
    for coeff in sets:  # two calls in a row, different inputs
        E_ctx = float(basis.energy_batch(coeff[None])[0])
        c3 = np.ascontiguousarray(basis.c3_raw(coeff).T)  # [klength][2N^2]
        d_c3 = torch.from_numpy(c3).cuda()
        d_E.fill_(np.nan)
        st = lib.tp3_bayes_energy_noalloc(ctypes.c_void_p(d_c3.data_ptr()), ctypes.c_void_p(q.data_ptr()), K, N,
                                          ctypes.c_void_p(d_E.data_ptr()), ctypes.c_void_p(stream))
        assert st == 0, lib.tp3_last_error(None)
        torch.cuda.synchronize()
        E = float(d_E.item())
        assert E == pytest.approx(E_ctx, rel=1e-6)
        energies.append(E)
    assert energies[0] != energies[1]
    # sizes beyond the static scratch are rejected before any launch
    assert lib.tp3_bayes_energy_noalloc(ctypes.c_void_p(d_c3.data_ptr()), ctypes.c_void_p(q.data_ptr()), 80, N,
                                        ctypes.c_void_p(d_E.data_ptr()), ctypes.c_void_p(stream)) == tp3._lib.TP3_ERR_ARG


def test_noalloc_energy_matches_context_path(config1, config1_hist):
    p = config1["params"]
    K, N, L, LMAX = p["K"], p["N"], p["L"], p["LMAX"]
    basis = tp3.calculate_basis(L, LMAX, N, K)
    try:
        basis.set_histogram(config1_hist)
        _two_calls(basis, config1_hist, config1["coeff"][:K], K, N, 23)
    finally:
        basis.close()


def test_noalloc_energy_matches_context_path_production_shape():
    from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms
    L, LMAX, N, K = 18, 25, 32, 26
    coeff = intensity_coefficients(synthetic_molecule(327, seed=20240601), LMAX, 38, 38.0, kcount=K)[:K]
    basis = tp3.calculate_basis(L, LMAX, N, K)
    try:
        basis.set_mode(tp3.TP3_MODE_PLAIN_FP32)
        hist = loadHistograms(poisson_histogram(basis.c3_raw(coeff).astype(np.float64), K, N, 1e9, seed=7), K)
        basis.set_histogram(hist)
        basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
        _two_calls(basis, hist, coeff, K, N, 29)
    finally:
        basis.close()
