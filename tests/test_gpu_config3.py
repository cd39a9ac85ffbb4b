"""Ragged scoring at the batched production shape: chains with K in 16..26 and L in
12..18 at N=32, each with its own molecule and its own 1e9-triplet histogram, scored
together in one tp3_energy_batch_ragged_device launch on the L18 K26 N32 context, and
every energy compared with the FP64 oracle evaluated at that chain's own (L, K).
Each chain contributes its molecule, a perturbed real-function coefficient set and a
perturbed general complex set (the fast and the general coupling paths).

The oracle for a chain of basis (L, K) is the reference's c3 for that basis
(src/correlations.jl:87-193, lrange = 0:2:L, shell triples k1 >= k2 >= k3 of 1..K)
and its Bayes energy against the chain's histogram (src/correlations.jl:196-226).  At
this shape the ragged launch skips pair blocks of orders above the chain's L, shells
from its K on and angular tiles past its K(K+1)(K+2)/6 shell triples, so the check
covers exactly the skipping logic that small shapes do not reach."""
import dataclasses

import numpy as np
import pytest

import tp3
from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms
from oracle.basis import enumerate_basis, lt_form_F
from oracle.c3 import energy_bayes
from oracle.refcpu import triple_products_fast

pytestmark = pytest.mark.gpu

LMAX, N, LBIG, KBIG = 25, 32, 18, 26
# (L, K) of each chain: every L of {12, 14, 18} with K of {16, 21, 26}, plus one L = 16
SHAPES = [(12, 16), (14, 21), (18, 26), (12, 26), (18, 16), (14, 16), (18, 21), (16, 26), (12, 21)]


def _basis_for(cache, L, K):
    """Oracle basis of (L, K): the enumeration depends on L only; the shell triples on K."""
    if L not in cache:
        b = enumerate_basis(L, LMAX, N, KBIG)
        cache[L] = (b, lt_form_F(b))
    b, F = cache[L]
    kl = np.array([(k1, k2, k3) for k1 in range(1, K + 1) for k2 in range(1, k1 + 1) for k3 in range(1, k2 + 1)],
                  dtype=np.int64)
    return dataclasses.replace(b, K=K, klist=kl), F


@pytest.fixture(scope="module")
def world():
    cache = {}
    mols, hists, oracles = [], [], []
    for i, (L, K) in enumerate(SHAPES):
        atoms = synthetic_molecule(200 + 25 * i, seed=9100 + i)
        coeff = intensity_coefficients(atoms, LMAX, 38, 38.0, kcount=KBIG)[:KBIG]
        b, F = _basis_for(cache, L, K)
        c3 = F @ triple_products_fast(b, coeff[:K]).T
        hists.append(loadHistograms(poisson_histogram(c3, K, N, 1e9, seed=70 + i), K))
        mols.append(coeff)
        oracles.append((b, F))
    big = tp3.calculate_basis(LBIG, LMAX, N, KBIG)
    big.set_histograms(hists, [K for _, K in SHAPES])
    yield big, mols, hists, oracles
    big.close()


def _perturb(coeff, rng, real):
    """Element-wise perturbation of every coefficient; real=True restores the relation
    c[l,-m] = (-1)^m conj(c[l,m]) of a real intensity (the fast real-function path),
    real=False leaves a general complex set (the general path)."""
    from tp3.structure import seanindex0
    x = coeff * (1.0 + 0.2 * rng.normal(size=coeff.shape)) + 0.2j * np.abs(coeff) * rng.normal(size=coeff.shape)
    if real:
        for l in range(0, LMAX):
            i0 = seanindex0(l, 0, LMAX)
            x[:, i0] = x[:, i0].real
            for m in range(1, l + 1):
                x[:, seanindex0(l, -m, LMAX)] = (-1) ** m * np.conj(x[:, seanindex0(l, m, LMAX)])
    return x


@pytest.mark.parametrize("form", [3, 5])
@pytest.mark.parametrize("mode", [tp3.TP3_MODE_TC_BF16X3, tp3.TP3_MODE_TC_TF32X3])
def test_ragged_config3_energies_match_fp64_oracle(world, mode, form):
    import torch
    big, mols, hists, oracles = world
    big.set_mode(mode)
    big.set_coupling(form)
    rng = np.random.default_rng(5 + mode)
    props, lkh, ref = [], [], []
    for h, ((L, K), coeff) in enumerate(zip(SHAPES, mols)):
        for j in range(3):
            c = coeff.copy() if j == 0 else _perturb(coeff, rng, real=(j == 1))
            props.append(c)
            lkh.append((L, K, h))
            b, F = oracles[h]
            # the oracle sees only the chain's own orders (<= L) and shells (< K)
            ref.append(energy_bayes(F @ triple_products_fast(b, c[:K]).T, hists[h], K, N))
    n = len(props)
    dev = torch.device("cuda")
    d_c = torch.from_numpy(np.ascontiguousarray(np.stack(props)).view(np.float64).copy()).to(dev)
    d_l = torch.tensor(lkh, dtype=torch.int32, device=dev)
    d_E = torch.empty(n, dtype=torch.float64, device=dev)
    big.energy_batch_ragged_device(n, d_c.data_ptr(), d_l.data_ptr(), d_E.data_ptr())
    big.sync()
    E = d_E.cpu().numpy()
    rel = np.abs(E - np.array(ref)) / np.abs(np.array(ref))
    assert rel.max() <= 1e-6, list(zip(lkh, rel))
    # the perturbed proposals move the energy by far more than the tolerance (the Bayes
    # energy is stationary at the histogram's own structure, so it moves at second order)
    for h in range(len(SHAPES)):
        assert abs(ref[3 * h + 1] - ref[3 * h]) > 1e-5 * abs(ref[3 * h])
        assert abs(ref[3 * h + 2] - ref[3 * h]) > 1e-5 * abs(ref[3 * h])
