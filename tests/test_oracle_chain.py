"""The oracle chain's random stream and move, without a GPU."""
import math

import numpy as np
import pytest

from oracle import chain as oc
from oracle.sh import seanindex


def test_philox_known_answer():
    # Random123's published known-answer vector for philox4x32-10: zero counter, zero key
    assert oc.philox4x32_10((0, 0, 0, 0), (0, 0)) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]


def test_plane_is_orthonormal():
    for l in (2, 8, 18):
        p, q = oc.plane(7, 3, 1, l)
        assert abs(p @ p - 1) < 1e-14 and abs(q @ q - 1) < 1e-14 and abs(p @ q) < 1e-14


def test_normals_are_standard():
    z = np.array([v for i in range(4000) for v in oc.normals4(1, i, 0, 1, 5)])
    assert abs(z.mean()) < 0.03 and abs(z.std() - 1) < 0.03


def test_move_keeps_shell_power(config1):
    """get_MC_step rotates each l-block of every shell by a unitary matrix."""
    p = config1["params"]
    c = config1["coeff"][: p["K"]]
    sigma = {l: 0.5 * (l - 1) for l in range(2, p["L"] + 1, 2)}
    new = oc.propose(c, p["L"], p["LMAX"], sigma, 5, 0, 0)
    for l in range(0, p["L"] + 1, 2):
        idx = [seanindex(l, m, p["LMAX"]) - 1 for m in range(-l, l + 1)]
        np.testing.assert_allclose(np.sum(np.abs(new[:, idx]) ** 2, 1), np.sum(np.abs(c[:, idx]) ** 2, 1), rtol=1e-12)
    assert np.abs(new - c).max() > 1e-3 * np.abs(c).max()
    # l = 0 and l > L are untouched
    idx0 = seanindex(0, 0, p["LMAX"]) - 1
    np.testing.assert_array_equal(new[:, idx0], c[:, idx0])
