"""Structure -> SH coefficients (createSphericalHarmonicsStructure, src/structure.jl:125-134).

CPU: the oracle's restatement of the s2kit transform (src/sh/s2kit_interface.c:72-178) is
pinned to an independent spherical-harmonic implementation (scipy) and to the exactness of
the Driscoll-Healy weights; the product's analytic intensity coefficients equal that
transform of the reference's intensityShell samples.  GPU: tp3_structure_sh, both routes,
against the oracle (FP64 throughout, relative to each array's largest magnitude)."""
import math

import numpy as np
import pytest

import tp3
import tp3.structure as st
from oracle import sht

pytestmark = []


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_dh_weights_integrate_polynomials_exactly():
    for bw in (4, 9, 16):
        x = np.cos(sht.dh_angles(bw)[1])
        w = sht.dh_weights(bw)
        for p in range(2 * bw):
            exact = (1 - (-1) ** (p + 1)) / (p + 1)
            assert abs(w @ x ** p - exact) < 1e-13


def test_oracle_transform_matches_independent_harmonics():
    """forward() of Y_lm samples (scipy's orthonormal harmonics with the Condon-Shortley
    phase) is the unit coefficient at seanindex(l, m): the transform's normalisation,
    phase and order conventions are those of s2kit's."""
    sph = pytest.importorskip("scipy.special")
    if not hasattr(sph, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    bw = 8
    phi, th = sht.dh_angles(bw)
    T, P = np.meshgrid(th, phi, indexing="ij")
    for l in range(bw):
        for m in range(-l, l + 1):
            c = sht.forward(sph.sph_harm_y(l, m, T, P).reshape(-1), bw)
            e = np.zeros(bw * bw, dtype=complex)
            e[sht.seanindex0(l, m, bw)] = 1.0
            assert np.abs(c - e).max() < 1e-13, (l, m)


def test_oracle_inverse_forward_round_trip():
    bw = 11
    rng = np.random.default_rng(1)
    c = rng.normal(size=bw * bw) + 1j * rng.normal(size=bw * bw)
    assert np.abs(sht.forward(sht.inverse(c, bw), bw) - c).max() < 1e-12


def test_analytic_intensity_equals_intensity_shell_route():
    """The product's host intensity coefficients equal the s2kit-semantics transform of
    getIntensity_cartesian samples at q_k = k pi / rmax; the difference is the two grids'
    aliasing of orders >= LMAX, which grows with q."""
    atoms = st.synthetic_molecule(40, seed=3, radius=6.0)
    LMAX, KMAX, rmax = 12, 16, 40.0
    ci = st.intensity_coefficients(atoms, LMAX, KMAX, rmax, kcount=8)
    # measured: 6e-15, 6e-15, 3e-13, 2e-11, 6e-10, 1.2e-8, 1.7e-7, 1.9e-6
    bounds = {1: 1e-13, 2: 1e-13, 3: 3e-12, 4: 2e-10, 5: 6e-9, 6: 1.2e-7, 7: 1.7e-6, 8: 2e-5}
    for k, b in bounds.items():
        co = sht.forward(sht.intensity_samples(atoms, k * math.pi / rmax, LMAX) + 0j, LMAX)
        assert _rel(ci[k - 1], co) < b, k


@pytest.fixture(scope="module")
def mols():
    return [st.synthetic_molecule(30, seed=3), st.synthetic_molecule(45, seed=8)]


@pytest.mark.gpu
def test_device_intensity_route_matches_oracle(mols):
    LMAX, KMAX, rmax = 12, 10, 40.0
    out = st.structure_sh(mols, LMAX, KMAX, rmax, route="intensity")
    assert set(out) == {"intensity"}
    for i, m in enumerate(mols):
        ref = np.stack([sht.forward(sht.intensity_samples(m, k * math.pi / rmax, LMAX) + 0j, LMAX)
                        for k in range(1, KMAX + 1)])
        assert _rel(out["intensity"][i], ref) < 1e-12


@pytest.mark.gpu
def test_device_reference_route_matches_oracle(mols):
    """density -> transform -> spherical Bessel transform -> absoluteSquare, per stage."""
    LMAX, KMAX, rmax = 10, 24, 40.0
    out = st.structure_sh(mols, LMAX, KMAX, rmax, route="reference")
    for i, m in enumerate(mols):
        dens, amp, inten = sht.density_route(m, LMAX, KMAX, rmax)
        assert _rel(out["density"][i], dens) < 1e-12
        assert _rel(out["amplitude"][i], amp) < 1e-11
        assert _rel(out["intensity"][i], inten) < 1e-11


@pytest.mark.gpu
def test_create_structure_from_pdb(tmp_path, mols):
    path = str(tmp_path / "m.pdb")
    st.write_pdb(mols[1], path)
    d, f, I = st.createSphericalHarmonicsStructure(path, 8, 12, 30.0)
    assert (d.rmax, f.rmax, I.rmax) == (30.0, math.pi * 12 / 30.0, math.pi * 12 / 30.0)
    ref = st.structure_sh([st.loadPDB(path)], 8, 12, 30.0)["intensity"][0]
    np.testing.assert_array_equal(I.coeff, ref)
    # a real intensity: c(l, -m) = (-1)^m conj c(l, m)
    for l in range(8):
        for m in range(1, l + 1):
            a, b = I.coeff[:, st.seanindex0(l, m, 8)], I.coeff[:, st.seanindex0(l, -m, 8)]
            assert np.abs(b - (-1) ** m * np.conj(a)).max() <= 1e-12 * np.abs(I.coeff).max()


@pytest.mark.gpu
def test_structure_sh_rejects_bad_arguments(mols):
    with pytest.raises(tp3.TP3Error):
        st.structure_sh(mols, 49, 4, 10.0)           # LMAX above 48
    with pytest.raises(tp3.TP3Error):
        st.structure_sh(mols, 8, 1, 10.0)            # KMAX below 2
    with pytest.raises(tp3.TP3Error):
        st.structure_sh(mols, 8, 4, -1.0)            # rmax <= 0
