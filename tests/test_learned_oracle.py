"""CPU checks of the oracle's learned-proposal mathematics (the restatement the device
moves are tested against): the two-sided drift density and its Metropolis-Hastings ratio,
the per-launch gradient estimator, and the drift's size."""
import math

import numpy as np
import pytest

from oracle import chain as oc
from oracle import mlp as om


def _params(rng, K, sigma):
    u = rng.normal(size=(K, 3))
    s_hat = rng.normal(size=(K, 3)) * 0.3
    return oc.shell_params(u, s_hat, sigma)


def test_two_sided_density_is_symmetric():
    rng = np.random.default_rng(0)
    K, sigma = 6, 0.05
    m, s = _params(rng, K, sigma)
    for _ in range(5):
        v = rng.normal(size=(K, 3)) * 0.1
        assert oc.net_logdens(v, m, s) == pytest.approx(oc.net_logdens(-v, m, s), abs=1e-12)


def test_ratio_is_one_for_unchanged_network_outputs():
    """With the network's parameters equal at x and x' (history-only drift) the mixture
    density is symmetric, so the Metropolis-Hastings correction vanishes."""
    rng = np.random.default_rng(1)
    K, sigma = 5, 0.08
    m, s = _params(rng, K, sigma)
    for p_net in (0.8, 1.0):
        v = rng.normal(size=(K, 3)) * 0.2
        assert oc.mixture_log_ratio(v, m, s, m, s, sigma, p_net) == pytest.approx(0.0, abs=1e-12)


def test_drift_size_is_sqrt_gamma_sigma():
    rng = np.random.default_rng(2)
    K, sigma = 26, 0.013
    u = rng.normal(size=(K, 3)) * 3.0
    m, _ = oc.shell_params(u, np.zeros((K, 3)), sigma)
    want = sigma * math.sqrt(om.DRIFT_GAMMA) * np.linalg.norm(u) / math.sqrt(np.sum(u * u) + om.DRIFT_EPS ** 2)
    assert np.linalg.norm(m) == pytest.approx(want, rel=1e-12)
    assert np.linalg.norm(m) == pytest.approx(4.0 * sigma, rel=1e-3)


def test_gradient_estimator_recovers_a_linear_gradient():
    """dE = sigma g . z + c over many candidates of one state: the estimate is sigma g / T
    (Gaussian smoothing, exact in expectation for a linear energy); candidates with a
    non-finite energy are left out."""
    rng = np.random.default_rng(3)
    K, B, sigma, T = 4, 20000, 0.05, 0.7
    g = rng.normal(size=(K, 3)) * 10.0
    z = rng.normal(size=(B, K, 3))
    dE = sigma * np.einsum("kd,bkd->b", g, z) + 3.0
    dE[:50] = np.nan
    e = oc.gradient_estimate(dE, T, z)
    ref = sigma * g / T
    assert np.linalg.norm(e - ref) / np.linalg.norm(ref) < 0.05
    assert np.all(oc.gradient_estimate(np.full(4, np.inf), T, z[:4]) == 0.0)


def test_loss_gradient_with_regression_only():
    """The regression term alone (NLL weights zero): the drift outputs' gradient is
    -lambda r v per row and nothing reaches the log-scale outputs' last-layer weights."""
    rng = np.random.default_rng(4)
    n_in, H, R, K = 5, 32, 8, 4
    p = om.init_params(n_in, H, 2).astype(np.float64)
    X = rng.normal(size=(R, n_in))
    v = rng.normal(size=(R, 3))
    w = np.zeros(R)
    tw = np.stack([rng.normal(size=R // K), np.full(R // K, 0.5)], axis=1)
    loss, g = om.loss_grad(p, X, v, w, n_in, H, tw, K)
    assert loss > 0.0
    # last layer W4 is 6 x H, stored row-major before b4: rows 3..5 (log-scales) get no gradient
    gW4 = g[-6 * H - 6:-6].reshape(6, H)
    assert np.all(gW4[3:] == 0.0) and np.any(gW4[:3] != 0.0)
