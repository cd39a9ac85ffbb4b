"""The evaluation-variant autotuner: every variant it times scores correctly, the
fastest becomes the context's mode, and TP3_MODE_AUTO contexts of the same shape
reuse the choice."""
import numpy as np
import pytest

import tp3

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_timed_variant_and_keeps_parity(config1, config1_hist):
    p = config1["params"]
    basis = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    basis.set_histogram(config1_hist)
    rep = basis.autotune(16)
    assert len(rep) >= 1 and rep[0][0] == tp3.TP3_MODE_PLAIN_FP32
    assert all(ms > 0 for _, _, _, ms in rep)
    # every variant is timed with the persistent angular schedule; the fastest
    # tensor-core one is timed again with one CTA per tile (the last row)
    tc_rows = [r for r in rep if r[0] != tp3.TP3_MODE_PLAIN_FP32]
    if tc_rows:
        assert rep[-1][2] == tp3.TP3_ANGULAR_TILE
        assert all(r[2] == tp3.TP3_ANGULAR_PERSISTENT for r in rep[:-1])
    best = min(rep, key=lambda r: r[3])
    assert basis.mode == best[0]
    E = basis.energy_batch(config1["coeff"][None, : p["K"]])[0]
    assert E == pytest.approx(float(config1["E_fp64"]), rel=1e-6)
    # a new AUTO context of the same shape takes the tuned mode
    other = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    assert other.mode == best[0]
    other.close()
    basis.close()
