"""Device-resident annealing chains vs the sequential FP64 oracle chain.

Seeded plain chains reproduce the reference method's accept/reject sequence
except at steps whose decision lies within the energy tolerance (|dE| or
|dE + T log u| below 1e-6 |E| + 1e-9).
"""
import math

import numpy as np
import pytest

import tp3
from tp3.chains import Chains, calculate_temperature
from oracle import chain as oc
from oracle.basis import enumerate_basis, lt_form_F
from oracle.c3 import triple_products, c3_lt_form, energy_bayes

pytestmark = pytest.mark.gpu

SEED = 0x5EED1234ABCD


@pytest.fixture(scope="module")
def setup(config1, config1_hist):
    p = config1["params"]
    basis = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    basis.set_histogram(config1_hist)
    ob = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    F = lt_form_F(ob)

    def e64(c):
        return energy_bayes(c3_lt_form(F, triple_products(ob, c)), config1_hist, p["K"], p["N"])

    coeff = config1["coeff"][: p["K"]]
    stepsizes = {l: (math.pi / 4) * (l - 1) for l in range(2, p["L"] + 1, 2)}
    T0 = calculate_temperature(coeff, basis, config1_hist, stepsizes, 0.3, iterations=20)
    yield basis, e64, coeff, T0, p
    basis.close()


# decision tolerance: the energy difference of two structures is trusted to 2e-7 |E|
DE_TOL = 2e-7


def _compare(dev_rows, ref_rows, E0, chain):
    """Decisions must agree at every step whose dE lies farther than the tolerance from
    the decision boundaries (0 and -T log u); the comparison ends at the first step
    where a boundary case was decided differently, since that changes the rest of the
    trajectory.  Returns the number of steps compared."""
    tol = DE_TOL * abs(E0)
    n = min(len(dev_rows), len(ref_rows))
    compared = 0
    for i in range(n):
        d, r = dev_rows[i], ref_rows[i]
        s = int(r[0]) - 1
        dE, T = r[4], r[5]
        u = oc.u01(oc.philox4x32_10((s, chain, 2, 0), (SEED & oc.M32, SEED >> 32))[0])
        ambiguous = abs(dE) <= tol or abs(dE + T * math.log(u)) <= tol
        if d[1] != r[1]:
            assert ambiguous, f"decision differs at step {i + 1}: dev {d} ref {r}"
            return compared
        assert d[0] == r[0]
        assert d[2] == pytest.approx(r[2], rel=2e-6)
        assert abs(d[4] - r[4]) <= tol
        compared += 1
    return compared


@pytest.mark.parametrize("mode", [tp3.TP3_MODE_PLAIN_FP32, tp3.TP3_MODE_TC_BF16X3])
def test_chain_matches_oracle(setup, mode):
    basis, e64, coeff, T0, p = setup
    basis.set_mode(mode)
    ch = Chains(basis, np.stack([coeff, coeff]), T0, math.pi / 4, 1.02, 0.99, SEED, ncand=4, log_capacity=64)
    assert ch.graph_captured
    ch.run(6)
    st = ch.state()
    for c in range(2):
        rows = ch.log(c)
        nsteps = int(st["steps"][c])
        assert len(rows) == nsteps >= 6
        _, E, T, sigma, ref = oc.run_chain(e64, coeff, p["L"], p["LMAX"], T0, math.pi / 4, 1.02, 0.99, SEED, c,
                                           nsteps)
        compared = _compare(rows, ref, ref[0][3], c)
        assert compared >= min(6, nsteps)
        if compared == nsteps:
            assert st["E"][c] == pytest.approx(E, rel=1e-6)
            assert st["T"][c] == pytest.approx(T, rel=1e-12)
            assert st["sigma"][c][-1] == pytest.approx(sigma[p["L"]], rel=1e-12)
    ch.close()


def test_candidates_per_launch_do_not_change_the_trajectory(setup):
    basis, e64, coeff, T0, p = setup
    basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
    a = Chains(basis, coeff[None], T0, math.pi / 4, 1.02, 0.99, SEED, ncand=1, log_capacity=64)
    a.run(12)
    b = Chains(basis, coeff[None], T0, math.pi / 4, 1.02, 0.99, SEED, ncand=5, log_capacity=64)
    b.run(12)
    ra, rb = a.log(0), b.log(0)
    n = min(len(ra), len(rb))
    assert n >= 12
    np.testing.assert_array_equal(ra[:n], rb[:n])
    a.close(); b.close()


def test_snapshot_restore_is_bit_exact(setup):
    basis, e64, coeff, T0, p = setup
    basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
    ch = Chains(basis, np.stack([coeff, coeff, coeff]), T0, math.pi / 4, 1.02, 0.99, SEED + 1, ncand=3)
    ch.run(2)
    blob = ch.snapshot()
    ch.run(3)
    s1, c1 = ch.state(), ch.coeff()
    ch.restore(blob)
    ch.run(3)
    s2, c2 = ch.state(), ch.coeff()
    for k in s1:
        np.testing.assert_array_equal(s1[k], s2[k])
    np.testing.assert_array_equal(c1, c2)
    with pytest.raises(tp3.TP3Error):
        ch.restore(blob[:-8])
    ch.close()


@pytest.mark.parametrize("mode", [tp3.TP3_MODE_PLAIN_FP32, tp3.TP3_MODE_TC_BF16X3])
def test_config1_protocol_1000_steps(setup, config1_hist, mode):
    """The small determination case as run by the reference: one chain from the true
    structure with every shell turned by a uniform random rotation, 1000
    rotate_all_at_once steps with the Bayes measure; the GPU chain (FP32 evaluation)
    follows the FP64 oracle chain's accept/reject sequence up to the first decision that
    lies within the energy tolerance of a boundary."""
    from tp3.learned import rotated_starts
    basis, e64, coeff, T0, p = setup
    basis.set_mode(mode)
    start = rotated_starts(basis, coeff, 1, 2024)[0]
    ch = Chains(basis, start[None], T0, math.pi / 4, 1.02, 0.99, SEED + 7, ncand=4, log_capacity=1100)
    while ch.state()["steps"][0] < 1000:
        ch.run(8)
    rows = ch.log(0)[:1000]
    _, _, _, _, ref = oc.run_chain(e64, start, p["L"], p["LMAX"], T0, math.pi / 4, 1.02, 0.99, SEED + 7, 0, 1000)
    compared = _compare(rows, ref, ref[0][3], 0)
    print(f"\n[config 1] mode {mode}: {compared} of 1000 steps follow the FP64 chain "
          f"(accepted {int((ref[:compared, 1] != 0).sum())}); E {ref[0][3]:.4f} -> {ref[compared - 1][3]:.4f}")
    assert compared >= 50   # disagreements before that would have failed inside _compare
    ch.close()
