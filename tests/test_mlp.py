"""Learned-proposal network: the oracle's own consistency on the CPU, and the
library's tcgen05 forward/backward kernels against the oracle (GPU)."""
import math

import numpy as np
import pytest

from oracle import mlp as om


def _bf16_inputs(rng, R, n_in, pad):
    X = np.zeros((R, pad))
    X[:, :n_in] = om.bf16(rng.normal(size=(R, n_in)) * 0.5)
    return X


def test_oracle_gradient_matches_finite_differences():
    """Without the BF16 roundings the oracle's backward is the exact gradient."""
    rng = np.random.default_rng(0)
    n_in, H, R, K = 7, 32, 16, 4
    p = om.init_params(n_in, H, 1).astype(np.float64)
    p[-6 * H - 6:] *= 10.0  # drift outputs of order one
    X = rng.normal(size=(R, n_in))
    v = rng.normal(size=(R, 3)) * 0.3
    w = rng.uniform(0, 1, size=R)
    tw = np.stack([rng.normal(size=R // K), rng.uniform(0.1, 1.0, size=R // K)], axis=1)
    ident = lambda x: np.asarray(x, dtype=np.float64)  # noqa: E731
    orig = om.bf16, om.f32
    om.bf16 = om.f32 = ident
    try:
        _, g = om.loss_grad(p, X, v, w, n_in, H, tw, K)
        for idx in list(rng.choice(p.size, 40, replace=False)) + list(range(p.size - 6 * H - 6, p.size, 37)):
            h = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[idx] += h
            pm[idx] -= h
            fd = (om.loss_grad(pp, X, v, w, n_in, H, tw, K)[0] - om.loss_grad(pm, X, v, w, n_in, H, tw, K)[0]) / (2 * h)
            assert fd == pytest.approx(g[idx], rel=1e-5, abs=1e-8)
    finally:
        om.bf16, om.f32 = orig


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1e-3], dtype=np.float32)
    got = om.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -7 and got[3] == -2.5
    assert abs(got[4] - 1e-3) / 1e-3 < 2 ** -8


def _net(n_in, H, R, seed=3):
    import tp3
    from tp3.learned import ProposalMLP
    basis = tp3.calculate_basis(2, 3, 4, 2)
    net = ProposalMLP(basis, n_in, hidden=H, max_rows=R, seed=seed)
    return basis, net


@pytest.mark.gpu
@pytest.mark.parametrize("n_in,H,R,K", [(394, 512, 512, 26), (45, 64, 256, 8)])
def test_device_forward_and_gradient_match_oracle(n_in, H, R, K):
    import torch
    rng = np.random.default_rng(n_in)
    basis, net = _net(n_in, H, R)
    pad = net.stride
    p = om.init_params(n_in, H, 7)
    net.set_params(p)
    X = _bf16_inputs(rng, R, n_in, pad)
    v = (rng.normal(size=(R, 3)) * 0.2).astype(np.float32)
    w = rng.uniform(0, 2, size=R).astype(np.float32)
    w[-5:] = 0.0
    nc = R // K
    tw = np.stack([rng.normal(size=nc) * 3.0, np.full(nc, 1.0 / nc)], axis=1).astype(np.float32)
    dev = torch.device("cuda")
    dX = torch.tensor(X, dtype=torch.bfloat16, device=dev)
    dv = torch.tensor(v, device=dev)
    dw = torch.tensor(w, device=dev)
    dt = torch.tensor(tw, device=dev)
    out = torch.empty((R, 6), dtype=torch.float32, device=dev)
    net.forward_device(R, dX.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    O, _ = om.forward(p.astype(np.float64), X, n_in, H)
    mu, s = om.head(O)
    got = out.cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(got[:, :3], mu, atol=2e-3)
    np.testing.assert_allclose(got[:, 3:], s, atol=2e-3)
    loss, g = net.loss_grad(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), dt.data_ptr(), K)
    lref, gref = om.loss_grad(p.astype(np.float64), X, v.astype(np.float64), w.astype(np.float64), n_in, H,
                              tw.astype(np.float64), K)
    assert loss == pytest.approx(lref, rel=1e-4)
    # per parameter block: relative error of the gradient
    sizes = [H * n_in, H, H * H, H, H * H, H, 6 * H, 6]
    o = 0
    for sz in sizes:
        a, b = g[o:o + sz].astype(np.float64), gref[o:o + sz]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b) + 1e-6, (o, sz)
        o += sz
    basis.close()


@pytest.mark.gpu
def test_device_training_fits_a_state_dependent_drift():
    """Adam on the device learns per-row drifts u*(x) from candidates' targets
    t = sum_k u*(x_k) . v_k + noise (the regression the proposal is trained with), and
    the log-scales from the steps' spread: the loss falls well below its untrained value
    and the learned u correlates strongly with u* (cosine > 0.7)."""
    import torch
    n_in, H, R, K = 64, 128, 4096, 2  # 2048 candidates: one equation per 6 unknown drifts
    rng = np.random.default_rng(5)
    basis, net = _net(n_in, H, R)
    X = _bf16_inputs(rng, R, n_in, net.stride)
    A = rng.normal(size=(n_in, 3)) * 0.1
    ustar = np.tanh(X[:, :n_in] @ A)
    v = rng.normal(size=(R, 3)).astype(np.float32)
    nc = R // K
    t = (ustar * v).reshape(nc, K * 3).sum(axis=1) + rng.normal(size=nc) * 0.05
    tw = np.stack([t, np.full(nc, 1.0 / nc)], axis=1).astype(np.float32)
    w = np.full(R, 1.0 / R, dtype=np.float32)
    dev = torch.device("cuda")
    dX = torch.tensor(X, dtype=torch.bfloat16, device=dev)
    dv, dw, dt = torch.tensor(v, device=dev), torch.tensor(w, device=dev), torch.tensor(tw, device=dev)
    l0 = net.train_step(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), 1e-3, dt.data_ptr(), K, want_loss=True)
    for _ in range(800):
        net.train_step(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), 1e-3, dt.data_ptr(), K)
    l1, _ = net.loss_grad(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), dt.data_ptr(), K, want_grad=False)
    assert math.isfinite(l1) and l1 < l0 - 1.0, (l0, l1)
    out = torch.empty((R, 6), dtype=torch.float32, device=dev)
    net.forward_device(R, dX.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    u = out.cpu().numpy()[:, :3].astype(np.float64)
    cos = float(np.sum(u * ustar) / (np.linalg.norm(u) * np.linalg.norm(ustar)))
    assert cos > 0.7, cos
    basis.close()


@pytest.mark.gpu
def test_network_at_chain_batch_size():
    """Forward and training step at the learned annealer's batch (64 chains x 16 candidates
    x 26 shells = 26 624 rows, 394 features, 3 x 512): finite outputs, loss falls."""
    import torch
    n_in, H, R, K = 394, 512, 26624, 26
    rng = np.random.default_rng(9)
    basis, net = _net(n_in, H, R)
    X = np.zeros((R, net.stride), dtype=np.float32)
    X[:, :n_in] = rng.normal(size=(R, n_in)).astype(np.float32) * 0.5
    dev = torch.device("cuda")
    dX = torch.tensor(X, dtype=torch.bfloat16, device=dev)
    dv = torch.tensor(rng.normal(size=(R, 3)).astype(np.float32) * 0.1, device=dev)
    dw = torch.full((R,), 1.0 / R, dtype=torch.float32, device=dev)
    nc = R // K
    dt = torch.tensor(np.stack([rng.normal(size=nc), np.full(nc, 1.0 / nc)], axis=1).astype(np.float32), device=dev)
    out = torch.empty((R, 6), dtype=torch.float32, device=dev)
    for _ in range(3):
        net.forward_device(R, dX.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    l0 = net.train_step(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), 1e-3, dt.data_ptr(), K, want_loss=True)
    for _ in range(20):
        net.train_step(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), 1e-3, dt.data_ptr(), K)
    l1, _ = net.loss_grad(R, dX.data_ptr(), dv.data_ptr(), dw.data_ptr(), dt.data_ptr(), K, want_grad=False)
    assert math.isfinite(l1) and l1 < l0
    basis.close()
