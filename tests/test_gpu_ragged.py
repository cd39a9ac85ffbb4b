"""Ragged batches: proposals and chains of different (L, K), each with its own
histogram, scored in one launch on the largest shape, against separate contexts of
each shape (and the FP64 oracle)."""
import math

import numpy as np
import pytest

import tp3
from tp3.chains import Chains
from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms
from oracle import chain as oc
from oracle.basis import enumerate_basis, lt_form_F
from oracle.c3 import triple_products, c3_lt_form, energy_bayes

pytestmark = pytest.mark.gpu

LMAX, N, LBIG, KBIG = 9, 16, 8, 8
SHAPES = [(8, 8), (6, 7), (4, 5), (8, 6)]


@pytest.fixture(scope="module")
def world():
    mols = [intensity_coefficients(synthetic_molecule(200 + 40 * i, seed=31 + i), LMAX, 8, 8.0)
            for i in range(len(SHAPES))]
    ctxs, hists = [], []
    for (L, K), coeff in zip(SHAPES, mols):
        b = tp3.calculate_basis(L, LMAX, N, K)
        b.set_mode(tp3.TP3_MODE_TC_BF16X3)
        c3 = b.c3_raw(coeff[:K]).astype(np.float64)
        h = loadHistograms(poisson_histogram(c3, K, N, 1e8, seed=5), K)
        b.set_histogram(h)
        ctxs.append(b)
        hists.append(h)
    big = tp3.calculate_basis(LBIG, LMAX, N, KBIG)
    big.set_mode(tp3.TP3_MODE_TC_BF16X3)
    big.set_histograms(hists, [K for _, K in SHAPES])
    yield big, ctxs, hists, mols
    for b in ctxs:
        b.close()
    big.close()


def test_ragged_energies_match_per_shape_contexts(world):
    import torch
    big, ctxs, hists, mols = world
    rng = np.random.default_rng(3)
    props, lkh, ref = [], [], []
    for h, ((L, K), coeff) in enumerate(zip(SHAPES, mols)):
        for _ in range(3):
            c = coeff[:KBIG] * (1.0 + 0.05 * rng.normal(size=(KBIG, 1)))
            props.append(c)
            lkh.append((L, K, h))
            ref.append(ctxs[h].energy_batch(c[None, :K])[0])
    n = len(props)
    dev = torch.device("cuda")
    d_c = torch.from_numpy(np.ascontiguousarray(np.stack(props)).view(np.float64).copy()).to(dev)
    d_l = torch.tensor(lkh, dtype=torch.int32, device=dev)
    d_E = torch.empty(n, dtype=torch.float64, device=dev)
    big.energy_batch_ragged_device(n, d_c.data_ptr(), d_l.data_ptr(), d_E.data_ptr())
    big.sync()
    np.testing.assert_allclose(d_E.cpu().numpy(), np.array(ref), rtol=1e-6)
    # one against the FP64 oracle at its own shape
    L, K = SHAPES[2]
    ob = enumerate_basis(L, LMAX, N, K)
    e64 = energy_bayes(c3_lt_form(lt_form_F(ob), triple_products(ob, props[6][:K])), hists[2], K, N)
    assert float(d_E[6]) == pytest.approx(e64, rel=1e-6)


def test_ragged_limits_are_checked(world):
    import torch
    big = world[0]
    dev = torch.device("cuda")
    d_c = torch.zeros((1, KBIG, LMAX * LMAX, 2), dtype=torch.float64, device=dev)
    d_l = torch.tensor([[LBIG, KBIG, 99]], dtype=torch.int32, device=dev)  # no such histogram
    d_E = torch.empty(1, dtype=torch.float64, device=dev)
    big.energy_batch_ragged_device(1, d_c.data_ptr(), d_l.data_ptr(), d_E.data_ptr())
    with pytest.raises(tp3.TP3Error) as ei:
        big.sync()
    assert ei.value.status == tp3._lib.TP3_ERR_ARG


def test_ragged_chains_follow_per_shape_chains(world):
    big, ctxs, hists, mols = world
    nch, B, launches, seed = len(SHAPES), 4, 5, 777
    starts = np.stack([m[:KBIG] for m in mols])
    T0 = 0.5
    rag = Chains(big, starts, T0, math.pi / 8, 1.02, 0.99, seed, ncand=B, log_capacity=64,
                 shapes=[(L, K, h) for h, (L, K) in enumerate(SHAPES)])
    rag.run(launches)
    for c, (L, K) in enumerate(SHAPES):
        # the same chain index in a chain set of its own shape draws the same random numbers
        sep = Chains(ctxs[c], np.repeat(starts[c:c + 1, :K], nch, axis=0), T0, math.pi / 8, 1.02, 0.99, seed,
                     ncand=B, log_capacity=64)
        sep.run(launches)
        a, b = rag.log(c), sep.log(c)
        n = min(len(a), len(b))
        assert n >= launches
        agree = 0
        for i in range(n):
            if a[i, 1] != b[i, 1]:
                # only a decision within the energy tolerance of a boundary may differ
                tol = 2e-7 * abs(b[0, 3])
                s = int(b[i, 0]) - 1
                u = oc.u01(oc.philox4x32_10((s, c, 2, 0), (seed & oc.M32, seed >> 32))[0])
                dE, T = b[i, 4], b[i, 5]
                assert abs(dE) <= tol or abs(dE + T * math.log(u)) <= tol, (c, i, a[i], b[i])
                break
            assert a[i, 2] == pytest.approx(b[i, 2], rel=2e-6)
            agree += 1
        assert agree >= min(n, 3)
        sep.close()
    rag.close()


def test_learned_moves_on_ragged_chains_match_oracle(world):
    """Learned moves on chains of different (L, K) in one context: each chain's feature
    rows carry its own orders only, its steps rotate its own orders, and the logged
    features, two-sided steps, Metropolis-Hastings ratios and energy changes match the
    oracle (per-shape contexts score the moved structures)."""
    import torch
    from tp3.learned import ProposalMLP, n_in_for
    from oracle import mlp as om
    big, ctxs, hists, mols = world
    nch, B, seed = len(SHAPES), 4, 4242
    n_in = n_in_for(LBIG)
    stride = (n_in + 31) // 32 * 32
    net = ProposalMLP(big, n_in, hidden=64, max_rows=((nch * B * KBIG + 127) // 128) * 128, seed=3)
    params = om.init_params(n_in, 64, 5)
    params[-6 - 6 * 64:-6] *= 0.3
    params[-6:-3] = 0.0
    params[-3:] = math.atanh((0.0 - om.S_MID) / om.S_HALF)
    net.set_params(params)
    starts = np.stack([m[:KBIG] for m in mols])
    T0, sigma0, decay, p_net = 0.5, 0.3, 0.99, 0.8
    ch = Chains(big, starts, T0, math.pi / 8, 1.05, decay, seed, ncand=B,
                shapes=[(L, K, h) for h, (L, K) in enumerate(SHAPES)])
    ch.set_move(tp3.TP3_MOVE_LEARNED, sigma0, p_net, net)
    ch.enable_move_log(2)
    ch.run(1)
    n = ch.move_log_count()
    assert n == nch * B
    dev = torch.device("cuda")
    idx = torch.arange(n, dtype=torch.int64, device=dev)
    X = torch.empty((n * KBIG, stride), dtype=torch.bfloat16, device=dev)
    V = torch.empty((n * KBIG, 3), dtype=torch.float32, device=dev)
    M = torch.empty((n, 7), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    ch.move_log_gather(n, idx.data_ptr(), X.data_ptr(), V.data_ptr(), M.data_ptr())
    torch.cuda.synchronize()
    X, V, M = X.float().cpu().numpy().astype(np.float64), V.cpu().numpy().astype(np.float64), M.cpu().numpy()

    def dev_head(feats):
        d_x = torch.tensor(feats, dtype=torch.bfloat16, device=dev)
        out = torch.empty((feats.shape[0], 6), dtype=torch.float32, device=dev)
        net.forward_device(feats.shape[0], d_x.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        o = out.cpu().numpy().astype(np.float64)
        return o[:, :3], o[:, 3:]

    hist0, ghist0 = np.zeros(8), np.zeros((8, KBIG, 3))
    nf = (LBIG + 1) ** 2
    for c, (L, K) in enumerate(SHAPES):
        start = starts[c]
        E0 = ctxs[c].energy_batch(start[None, :K])[0]
        for i in range(B):
            j = c * B + i
            T = T0 * decay ** (i + 1)
            feats = om.shell_features(start, LBIG, LMAX, hist0, T, stride, ghist0, L_used=L)
            Xd = X[j * KBIG:(j + 1) * KBIG]
            assert np.all(np.abs(Xd - feats) <= 2 ** -7 * np.abs(feats) + 1e-30)
            assert np.all(Xd[:, (L + 1) ** 2:nf] == 0.0)  # orders above the chain's L
            comp = 1.0 if oc.component_uniform(seed, i, c) < p_net else 0.0
            assert M[j, 3] == comp
            z, a = oc.shell_noise(seed, 0, c, i, KBIG)
            sig_i = sigma0 / 1.05 ** i
            v = V[j * KBIG:(j + 1) * KBIG] * M[j, 5]
            m, s = oc.shell_params(*dev_head(Xd), sig_i)
            vref = a * m + np.exp(s) * z if comp else sig_i * z
            np.testing.assert_allclose(v, vref, rtol=1e-5, atol=1e-6)
            x2 = oc.rotate_shells(start, v, L, LMAX)
            m2, s2 = oc.shell_params(*dev_head(om.shell_features(x2, LBIG, LMAX, hist0, T, stride, ghist0,
                                                                 L_used=L)), sig_i)
            lr = oc.mixture_log_ratio(v, m, s, m2, s2, sig_i, p_net)
            assert M[j, 4] == pytest.approx(lr, abs=0.05 + 0.01 * abs(lr))
            E2 = ctxs[c].energy_batch(x2[None, :K])[0]
            assert M[j, 0] == pytest.approx(E2 - E0, abs=2e-6 * abs(E0))
    ch.close()
    net.close()
