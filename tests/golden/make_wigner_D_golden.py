"""Generate tests/golden/wigner_D.json: Wigner rotation matrices of the reference's
rotationMatrix convention (src/spherical_harmonics.jl:572-592),

    D[m, s] = exp(-i s gamma - i m phi) d^l_{ms}(theta),

with d^l from sympy.physics.wigner.wigner_d_small (an independent implementation of
the published formula; its matrix is the transpose of the reference's d_work order)
evaluated at 40 digits from the exact binary value of each angle.

    python tests/golden/make_wigner_D_golden.py
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = [(0, 0.3, 0.2, -0.1), (2, 0.7, 1.1, -0.4), (7, 2.2, -2.9, 0.6), (18, 1.3, 0.5, 2.8), (24, 0.05, -1.7, 3.0)]


def main():
    from sympy import Rational
    from sympy.physics.wigner import wigner_d_small
    out = []
    for l, th, ph, ga in CASES:
        d = np.array(wigner_d_small(l, Rational(th)).evalf(40).tolist(), dtype=float).T  # [m, s]
        ms = np.arange(-l, l + 1)
        D = np.exp(-1j * ms[None, :] * ga - 1j * ms[:, None] * ph) * d
        out.append({"l": l, "theta": th, "phi": ph, "gamma": ga, "re": D.real.tolist(), "im": D.imag.tolist()})
    with open(os.path.join(HERE, "wigner_D.json"), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    main()
