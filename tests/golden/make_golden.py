"""Generate the committed golden fixtures of the c3 + Bayes path.

    python tests/golden/make_golden.py

Writes, beside this script:
  sh_values.json   Wigner 3j symbols from sympy's exact implementation and
                   orthonormal Legendre values from scipy.special.sph_harm_y,
                   the two GSL routines the reference calls
                   (src/spherical_harmonics.jl:63-76), as independent pins of the
                   oracle's and the library's special functions.
  config1.npz      the small determination case (L=8, LMAX=9, K=8, N=16):
                   intensity coefficients of a seeded 327-atom synthetic molecule,
                   a 1e8-triplet Poisson histogram (counts), the FP64 c3 of the
                   oracle (l-triple form), the c3 of the reference-form restatement
                   (f32 B / h_P tables, f64 accumulation, src/correlations.jl:157-193)
                   and the Bayes energies of both.
"""
from __future__ import annotations

import json
import math
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "threephotons.jl_gb300"))

CONFIG1 = dict(L=8, LMAX=9, K=8, N=16, KMAX=8, rmax=8.0, atoms=327, mol_seed=1, hist_seed=2, triplets=1e8)


def sh_values():
    from sympy.physics.wigner import wigner_3j
    from scipy.special import sph_harm_y
    rng = random.Random(12345)
    threej = []
    while len(threej) < 400:
        l1, l2 = rng.randint(0, 24), rng.randint(0, 24)
        l3 = rng.randint(abs(l1 - l2), min(l1 + l2, 30))
        m1, m2 = rng.randint(-l1, l1), rng.randint(-l2, l2)
        m3 = -m1 - m2
        if abs(m3) > l3:
            continue
        threej.append([l1, l2, l3, m1, m2, m3, float(wigner_3j(l1, l2, l3, m1, m2, m3))])
    # structural and accidental zeros
    for args in [(3, 2, 3, 0, 0, 0), (1, 1, 1, 0, 0, 0), (2, 2, 3, 0, 0, 0), (4, 2, 4, 2, 0, -2)]:
        threej.append([*args, float(wigner_3j(*args))])
    plm = []
    for l in range(0, 25):
        for m in range(-l, l + 1):
            for th in (0.2, 1.1, math.pi / 2, 2.9):
                plm.append([l, m, th, float(sph_harm_y(l, m, th, 0.0).real)])
    return {"wigner3j": threej, "sphPlm": plm}


def config1():
    from oracle.basis import enumerate_basis, reference_tables, lt_form_F
    from oracle.c3 import triple_products, c3_reference_form, c3_lt_form, energy_bayes
    from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms
    c = CONFIG1
    atoms = synthetic_molecule(c["atoms"], seed=c["mol_seed"])
    coeff = intensity_coefficients(atoms, c["LMAX"], c["KMAX"], c["rmax"])
    b = enumerate_basis(c["L"], c["LMAX"], c["N"], c["K"])
    T = triple_products(b, coeff)
    F = lt_form_F(b)
    c3_64 = c3_lt_form(F, T)
    B32, P32 = reference_tables(b)
    c3_ref = c3_reference_form(b, coeff, B32, P32)
    counts = poisson_histogram(c3_64, c["K"], c["N"], c["triplets"], seed=c["hist_seed"])
    hist = loadHistograms(counts, c["K"])
    E64 = energy_bayes(c3_64, hist, c["K"], c["N"])
    Eref = energy_bayes(c3_ref, hist, c["K"], c["N"])
    return dict(coeff=coeff, counts=counts.astype(np.int64), c3_fp64=c3_64, c3_refform=c3_ref,
                E_fp64=E64, E_refform=Eref, basislen=b.basislen, n_lt=b.n_lt)


def main():
    with open(os.path.join(HERE, "sh_values.json"), "w") as f:
        json.dump(sh_values(), f)
    d = config1()
    np.savez_compressed(os.path.join(HERE, "config1.npz"), **d, params=json.dumps(CONFIG1))
    print("basislen", d["basislen"], "n_lt", d["n_lt"], "E_fp64", d["E_fp64"], "E_refform", d["E_refform"])


if __name__ == "__main__":
    main()
