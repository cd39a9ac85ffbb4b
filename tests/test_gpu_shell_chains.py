"""Per-shell SO(3) chain moves and the learned (network) proposal on the device
against the oracle: the isotropic chain's trajectory, the per-launch gradient
estimates that feed the network, the network proposal with a constant head reducing
to the isotropic one, and the logged features, two-sided drift steps and
Metropolis-Hastings ratios of a random network recomputed on the CPU."""
import math

import numpy as np
import pytest

import tp3
from tp3.chains import Chains
from tp3.learned import ProposalMLP, n_in_for
from oracle import chain as oc
from oracle import mlp as om
from oracle.basis import enumerate_basis, lt_form_F
from oracle.c3 import triple_products, c3_lt_form, energy_bayes

pytestmark = pytest.mark.gpu

SEED = 0x5EEDC0FFEE12
DE_TOL = 2e-7


@pytest.fixture(scope="module")
def setup(config1, config1_hist):
    p = config1["params"]
    basis = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    basis.set_histogram(config1_hist)
    ob = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    F = lt_form_F(ob)

    def e64(c):
        return energy_bayes(c3_lt_form(F, triple_products(ob, c)), config1_hist, p["K"], p["N"])

    coeff = np.ascontiguousarray(config1["coeff"][: p["K"]])
    # start: the true structure with every shell turned by its own rotation
    rng = np.random.default_rng(4)
    start = oc.rotate_shells(coeff, rng.normal(size=(p["K"], 3)) * 0.6, p["L"], p["LMAX"])
    yield basis, e64, start, p
    basis.close()


def _agree(dev_rows, ref_rows, E0, chain):
    tol = DE_TOL * abs(E0)
    compared = 0
    for d, r in zip(dev_rows, ref_rows):
        s = int(r[0]) - 1
        dE, T = r[4], r[5]
        u = oc.u01(oc.philox4x32_10((s, chain, 2, 0), (SEED & oc.M32, SEED >> 32))[0])
        ambiguous = abs(dE) <= tol or abs(dE + T * math.log(u)) <= tol
        if d[1] != r[1]:
            assert ambiguous, f"decision differs at step {s + 1}: dev {d} ref {r}"
            break
        assert d[2] == pytest.approx(r[2], rel=2e-6)
        compared += 1
    return compared


def test_isotropic_shell_chain_matches_oracle(setup):
    basis, e64, start, p = setup
    nch, B, launches = 2, 4, 4
    T0, sigma0, f, decay = 2.0, 0.25, 1.05, 0.995
    ch = Chains(basis, np.repeat(start[None], nch, axis=0), T0, 0.1, f, decay, SEED, ncand=B, log_capacity=64)
    ch.set_move(tp3.TP3_MOVE_SHELL_SO3, sigma0)
    ch.run(launches)
    assert all(ch.state()["steps"] > 0)
    for c in range(nch):
        rows = ch.log(c)
        _, _, _, _, ref = oc.run_shell_chain(e64, start, p["L"], p["LMAX"], T0, sigma0, f, decay, SEED, c, launches, B)
        assert _agree(rows, ref, ref[0][3], c) >= min(len(rows), 3)
    ch.close()


def _constant_head_params(net, s_const):
    P = np.zeros(net.n_params, dtype=np.float32)
    P[-3:] = math.atanh((s_const - om.S_MID) / om.S_HALF)  # b4[3:6]: s = s_const, u = 0
    return P


def test_constant_network_proposes_isotropic_steps(setup):
    """A network with u = 0 and constant log-scales proposes the isotropic step (its own
    launch-keyed normals times sigma_i) and its Metropolis-Hastings ratio is exactly one."""
    basis, e64, start, p = setup
    nch, B = 4, 4
    L, K = p["L"], p["K"]
    net = ProposalMLP(basis, n_in_for(L), hidden=64, max_rows=((nch * B * K + 127) // 128) * 128, seed=1)
    net.set_params(_constant_head_params(net, math.log(0.2)))
    sigma0 = 0.2
    ch = Chains(basis, np.repeat(start[None], nch, axis=0), 2.0, 0.1, 1.05, 0.995, SEED, ncand=B)
    ch.set_move(tp3.TP3_MOVE_LEARNED, sigma0, 1.0, net)
    ch.enable_move_log(4)
    ch.run(1)
    stride = (n_in_for(L) + 31) // 32 * 32
    _, V, M = _gather(ch, list(range(nch * B)), K, stride)
    assert np.all(M[:, 3] == 1.0) and np.all(M[:, 4] == 0.0)
    for c in range(nch):
        for i in range(B):
            z, _ = oc.shell_noise(SEED, 0, c, i, K)
            j = c * B + i
            np.testing.assert_allclose(V[j * K:(j + 1) * K], z, rtol=1e-6, atol=1e-6)
    ch.close()
    net.close()


def _gather(ch, positions, K, stride):
    import torch
    dev = torch.device("cuda")
    n = len(positions)
    idx = torch.tensor(positions, dtype=torch.int64, device=dev)
    X = torch.empty((n * K, stride), dtype=torch.bfloat16, device=dev)
    V = torch.empty((n * K, 3), dtype=torch.float32, device=dev)
    M = torch.empty((n, 7), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    ch.move_log_gather(n, idx.data_ptr(), X.data_ptr(), V.data_ptr(), M.data_ptr())
    torch.cuda.synchronize()
    return X.float().cpu().numpy().astype(np.float64), V.cpu().numpy().astype(np.float64), M.cpu().numpy()


def test_gradient_history_matches_oracle(setup):
    """Each launch's per-shell gradient estimate (from its candidates' energy changes and
    whitened steps) enters the next launch's feature rows: recomputed on the CPU from the
    logged candidates of the first launch."""
    basis, e64, start, p = setup
    nch, B = 2, 8
    L, LMAX, K = p["L"], p["LMAX"], p["K"]
    T0, decay = 2.0, 0.995
    ch = Chains(basis, np.repeat(start[None], nch, axis=0), T0, 0.1, 1.05, decay, SEED, ncand=B)
    ch.set_move(tp3.TP3_MOVE_SHELL_SO3, 0.3)
    ch.enable_move_log(4)
    ch.run(2)
    stride = (n_in_for(L) + 31) // 32 * 32
    nf = (L + 1) ** 2
    X1, V1, M1 = _gather(ch, list(range(nch * B)), K, stride)
    X2, _, _ = _gather(ch, [nch * B + c * B for c in range(nch)], K, stride)
    for c in range(nch):
        dE = M1[c * B:(c + 1) * B, 0]
        w = V1[c * B * K:(c + 1) * B * K].reshape(B, K, 3)  # isotropic steps: w = v / sigma
        e = oc.gradient_estimate(dE, T0 * decay, w)
        assert np.abs(e).max() > 1e-3  # a real signal, not a zero history
        got = X2[c * K:(c + 1) * K, nf + 9:nf + 12]  # newest launch first
        ref = 0.5 * np.clip(e, -8, 8)
        np.testing.assert_allclose(got, ref, rtol=2 ** -7, atol=1e-4)
        # older launches: zeros (two launches run, the first saw an empty history)
        assert np.all(X2[c * K:(c + 1) * K, nf + 12:nf + 33] == 0.0)
    ch.close()


def test_learned_moves_match_oracle(setup):
    import torch
    basis, e64, start, p = setup
    nch, B = 2, 8
    L, LMAX, K = p["L"], p["LMAX"], p["K"]
    n_in = n_in_for(L)
    net = ProposalMLP(basis, n_in, hidden=128, max_rows=((nch * B * K + 127) // 128) * 128, seed=2)
    params = om.init_params(n_in, 128, 11)
    # moderate steps (s^ near 0, drifts of a few sigma): the reverse density stays well
    # conditioned, so one-ulp BF16 differences between the device's and the oracle's
    # features of x' move the ratio by far less than the tolerance
    nW4 = 6 * 128
    params[-6 - nW4:-6] *= 0.3
    params[-6:-3] = 0.0
    params[-3:] = math.atanh((0.0 - om.S_MID) / om.S_HALF)
    net.set_params(params)
    T0, sigma0, decay, p_net = 2.0, 0.3, 0.995, 0.8
    ch = Chains(basis, np.repeat(start[None], nch, axis=0), T0, 0.1, 1.05, decay, SEED, ncand=B)
    ch.set_move(tp3.TP3_MOVE_LEARNED, sigma0, p_net, net)
    ch.enable_move_log(4)
    # plant a gradient history (the snapshot's last block: [nch][8][K][3] float32)
    blob = bytearray(ch.snapshot())
    ng = nch * 8 * K * 3
    ghist = np.random.default_rng(8).normal(size=(nch, 8, K, 3)).astype(np.float32)
    blob[len(blob) - 4 * ng:] = ghist.tobytes()
    ch.restore(bytes(blob))
    ch.run(1)
    n = ch.move_log_count()
    assert n == nch * B
    stride = (n_in + 31) // 32 * 32
    X, V, M = _gather(ch, list(range(n)), K, stride)
    hist = np.zeros(8)
    P64 = params.astype(np.float64)
    E0 = e64(start)
    dev = torch.device("cuda")

    def dev_head(feats):  # the device network on given feature rows
        d_x = torch.tensor(feats, dtype=torch.bfloat16, device=dev)
        out = torch.empty((feats.shape[0], 6), dtype=torch.float32, device=dev)
        net.forward_device(feats.shape[0], d_x.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        o = out.cpu().numpy().astype(np.float64)
        return o[:, :3], o[:, 3:]

    n_net = 0
    for c in range(nch):
        for i in range(B):
            j = c * B + i
            T = T0
            for _ in range(i + 1):
                T *= decay
            feats = om.shell_features(start, L, LMAX, hist, T, stride, ghist[c])
            Xd = X[j * K:(j + 1) * K]
            # features agree to one BF16 rounding
            assert np.all(np.abs(Xd - feats) <= 2 ** -7 * np.abs(feats) + 1e-30)
            comp = 1.0 if oc.component_uniform(SEED, i, c) < p_net else 0.0
            z, a = oc.shell_noise(SEED, 0, c, i, K)
            assert M[j, 3] == comp
            n_net += int(comp)
            v = V[j * K:(j + 1) * K]
            # network vs oracle network (FP64 accumulation, same BF16 roundings)
            u_o, s_o = om.head(om.forward(P64, feats, n_in, 128)[0])
            uh, sh = dev_head(Xd)  # the rows the chain used
            np.testing.assert_allclose(uh, u_o, atol=3e-3)
            np.testing.assert_allclose(sh, s_o, atol=3e-3)
            sig_i = sigma0
            for _ in range(i):  # candidate i assumes i rejections: sigma / f^i
                sig_i /= 1.05
            assert M[j, 5] == pytest.approx(sig_i, rel=1e-6)
            v = v * M[j, 5]  # the log holds v / sigma_i
            m, s = oc.shell_params(uh, sh, sig_i)
            if comp:
                vref = a * m + np.exp(s) * z
            else:
                vref = sig_i * z
            np.testing.assert_allclose(v, vref, rtol=1e-5, atol=1e-6)
            # Metropolis-Hastings ratio of the mixture, reverse density at x'
            x2 = oc.rotate_shells(start, v, L, LMAX)
            m2, s2 = oc.shell_params(*dev_head(om.shell_features(x2, L, LMAX, hist, T, stride, ghist[c])), sig_i)
            lr = oc.mixture_log_ratio(v, m, s, m2, s2, sig_i, p_net)
            assert M[j, 4] == pytest.approx(lr, abs=0.05 + 0.01 * abs(lr))
            assert M[j, 0] == pytest.approx(e64(x2) - E0, abs=5e-7 * abs(E0))
    assert 0 < n_net < nch * B
    ch.close()
    net.close()


def test_drift_moves_match_oracle(setup):
    """The network-free drift move: with a planted gradient history, every logged step is
    v = a sigma f(u) u + sigma z (drift-drawn) or sigma z (isotropic) with u the chain's
    newest gradient estimate and isotropic scales; the proposal is symmetric, so the
    logged Metropolis-Hastings log ratio is exactly 0; energy changes match the FP64
    oracle."""
    basis, e64, start, p = setup
    nch, B = 2, 8
    L, LMAX, K = p["L"], p["LMAX"], p["K"]
    T0, sigma0, decay, p_net = 2.0, 0.3, 0.995, 0.8
    ch = Chains(basis, np.repeat(start[None], nch, axis=0), T0, 0.1, 1.05, decay, SEED, ncand=B)
    ch.set_move(tp3.TP3_MOVE_DRIFT, sigma0, p_net)
    ch.enable_move_log(4)
    blob = bytearray(ch.snapshot())
    ng = nch * 8 * K * 3
    ghist = np.random.default_rng(9).normal(size=(nch, 8, K, 3)).astype(np.float32)
    blob[len(blob) - 4 * ng:] = ghist.tobytes()
    ch.restore(bytes(blob))
    ch.run(1)
    n = ch.move_log_count()
    assert n == nch * B
    stride = (n_in_for(L) + 31) // 32 * 32
    _, V, M = _gather(ch, list(range(n)), K, stride)
    E0 = e64(start)
    n_drift = 0
    for c in range(nch):
        u = ghist[c, 0].astype(np.float64)
        for i in range(B):
            j = c * B + i
            comp = 1.0 if oc.component_uniform(SEED, i, c) < p_net else 0.0
            assert M[j, 3] == comp
            n_drift += int(comp)
            z, a = oc.shell_noise(SEED, 0, c, i, K)
            sig_i = sigma0 / 1.05 ** i
            v = V[j * K:(j + 1) * K] * M[j, 5]
            m, s = oc.shell_params(u, np.zeros((K, 3)), sig_i)
            vref = a * m + np.exp(s) * z if comp else sig_i * z
            np.testing.assert_allclose(v, vref, rtol=1e-5, atol=1e-6)
            assert M[j, 4] == 0.0
            x2 = oc.rotate_shells(start, v, L, LMAX)
            assert M[j, 0] == pytest.approx(e64(x2) - E0, abs=5e-7 * abs(E0))
    assert 0 < n_drift < nch * B
    ch.close()


def test_learned_proposal_gain_is_measured(config1, config1_hist, capsys):
    """The full learned-proposal protocol at the small configuration: the plain
    annealer's logged moves train the network on the device (held-out loss falls), and
    the learned annealer reaches the plain annealer's final median energy in fewer
    launches (the wall-clock ratio is reported: at this size the network's forward
    passes cost about as much as the scoring)."""
    from tp3.learned import learned_vs_plain
    p = config1["params"]
    basis = tp3.calculate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    basis.set_histogram(config1_hist)
    res = learned_vs_plain(basis, config1["coeff"], nchains=16, ncand=8, collect_launches=200, train_steps=200,
                           batch_candidates=256, eval_launches=120, seed=7)
    basis.close()
    assert res["collect"]["moves"] == 16 * 8 * 200
    assert res["train"]["heldout_nll_after"] < res["train"]["heldout_nll_before"]
    assert math.isfinite(res["learned"]["median_E"]) and math.isfinite(res["plain"]["final_median_E"])
    assert 0.05 < res["learned"]["accept_rate"] < 0.95
    assert res["learned"]["reached"] and res["learned"]["launches"] < res["plain"]["launches"]
    with capsys.disabled():
        print(f"\n[learned proposal, L8 K8 N16] plain: {res['plain']['launches']} launches "
              f"{res['plain']['seconds']:.3f} s -> median E {res['plain']['final_median_E']:.4f}; learned: "
              f"{res['learned']['launches']} launches {res['learned']['seconds_to_target']:.3f} s -> "
              f"{res['learned']['median_E']:.4f} (reached={res['learned']['reached']}, "
              f"time ratio={res['time_ratio']})")


def test_learned_proposal_gain_at_production_shape(capsys):
    """A shortened run of the benchmark's protocol at L18 K26 N32 (64 chains x 16
    candidates: 300 logged launches, 600 Adam steps, 150 evaluation launches): the
    learned annealer reaches the plain annealer's final median energy in at most half its
    wall-clock (the spec bar).  The network-free drift annealer (drift along the
    newest gradient estimate, same mixture) runs the same protocol beside it; its ratio
    is reported so the network's own contribution is measured, not assumed."""
    import os
    import sys
    from tp3.learned import learned_vs_plain
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    base = bench.molecule_coefficients()
    basis = tp3.calculate_basis(bench.L, bench.LMAX, bench.N, bench.K)
    try:
        basis.set_histogram(bench.build_histogram(basis, base))
        basis.set_mode(tp3.TP3_MODE_TC_BF16X3)
        res = learned_vs_plain(basis, base, collect_launches=300, train_steps=600, eval_launches=150, seed=31)
    finally:
        basis.close()
    assert res["learned"]["reached"]
    assert res["time_ratio"] <= 0.5, res["time_ratio"]
    assert "drift" in res and math.isfinite(res["drift"]["median_E"])
    with capsys.disabled():
        d = res["drift"]
        print(f"\n[learned proposal, L18 K26 N32, shortened] plain {res['plain']['seconds']:.2f} s -> "
              f"{res['plain']['final_median_E']:.3f}; learned {res['learned']['seconds_to_target']:.2f} s "
              f"({res['learned']['launches']} launches), time ratio {res['time_ratio']:.3f}; drift-only "
              f"{d['seconds_to_target']:.2f} s ({d['launches']} launches, reached={d['reached']}), "
              f"time ratio {res['time_ratio_drift']}")
