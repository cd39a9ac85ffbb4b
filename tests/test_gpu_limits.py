"""The largest shapes the library supports, where the FP64 oracle is too slow to run:
config 4 (L=24, K=38, N=32), the largest order of the pair-block tables (L=30: 16 l3
values per block) and the most shells of the warp-local coupling and per-shell moves
(K=64).  Every tensor-core mode and coupling form that fits is checked against the
independent plain FP32 path (direct basis-table coupling, SIMT angular contraction):
triple products to 2e-5 of their largest magnitude, energies to 2e-6 relative; and the
energy of a structure turned as a whole (the same rotation for every shell) is unchanged."""
import numpy as np
import pytest

import tp3
from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms

pytestmark = pytest.mark.gpu

SHAPES = [(24, 25, 32, 38), (30, 31, 16, 8), (4, 5, 16, 64)]


@pytest.mark.parametrize("L,LMAX,N,K", SHAPES)
def test_largest_shapes_agree_with_plain_path(L, LMAX, N, K):
    import torch
    coeff = intensity_coefficients(synthetic_molecule(200, seed=3), LMAX, K, float(K))
    basis = tp3.calculate_basis(L, LMAX, N, K)
    try:
        basis.set_mode(tp3.TP3_MODE_PLAIN_FP32)
        T0 = basis.triple_products(coeff).astype(np.float64)
        vol = tp3.SphericalHarmonicsVolume(coeff, LMAX, K, float(K))
        c3 = tp3.FullCorrelation_parallized(vol, basis, True, False, True)
        basis.set_histogram(loadHistograms(poisson_histogram(c3, K, N, 1e9, seed=5), K))
        E0 = float(basis.energy_batch(coeff[None, :K])[0])
        scale = np.abs(T0).max()
        checked = 0
        for mode in (tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3):
            basis.set_mode(mode)
            for form in range(9):
                try:
                    basis.set_coupling(form)
                except tp3.TP3Error:
                    continue  # this form does not fit the shape
                T = basis.triple_products(coeff).astype(np.float64)
                err = np.abs(T - T0).max() / scale
                assert err < 2e-5, (mode, form, err)
                E = float(basis.energy_batch(coeff[None, :K])[0])
                assert E == pytest.approx(E0, rel=2e-6), (mode, form)
                checked += 1
        assert checked >= 2  # at least one form per mode (at K=38 only the split coupling fits)
        # a common rotation of every shell leaves the energy unchanged (tensor-core mode)
        basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
        dev = torch.device("cuda")
        d_c = torch.from_numpy(np.ascontiguousarray(coeff[:K]).view(np.float64).copy()).to(dev).reshape(1, -1)
        d_v = torch.tensor(np.repeat([[0.7, -0.4, 1.1]], K, axis=0), dtype=torch.float64, device=dev)
        d_r = torch.empty_like(d_c)
        basis.rotate_shells_device(1, d_c.data_ptr(), d_v.data_ptr(), d_r.data_ptr())
        d_E = torch.empty(1, dtype=torch.float64, device=dev)
        basis.energy_batch_device(1, d_r.data_ptr(), d_E.data_ptr())
        basis.sync()
        assert float(d_E[0]) == pytest.approx(E0, rel=2e-6)
    finally:
        basis.close()
