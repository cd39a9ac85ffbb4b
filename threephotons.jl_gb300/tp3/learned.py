"""Learned proposal for the annealer: the network handle over libtp3.

No counterpart in the reference.  ``ProposalMLP`` owns a device network
(tp3_mlp_*): 3 hidden ReLU layers, BF16 weights and activations, FP32
accumulation, trained by the library's own tcgen05 forward/backward kernels with
Adam.  Every method takes device pointers (torch tensors' ``data_ptr()``);
nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import TP3Error, check, load


def n_in_for(L: int) -> int:
    """Feature width per shell: (L+1)^2 real SH coefficients, 8 history values, log T,
    8 launches x 3 gradient estimates."""
    return (L + 1) * (L + 1) + 9 + 24


def n_in_pad(n_in: int) -> int:
    return (n_in + 31) // 32 * 32


class ProposalMLP:
    def __init__(self, basis, n_in: int, hidden: int = 512, max_rows: int = 32768, seed: int = 0):
        self._lib = load()
        self._basis = basis
        self.n_in, self.hidden, self.max_rows = n_in, hidden, max_rows
        self.stride = n_in_pad(n_in)
        h = ctypes.c_void_p()
        check(self._lib.tp3_mlp_create(basis.ctx, n_in, hidden, max_rows, ctypes.c_uint64(seed), ctypes.byref(h)),
              basis.ctx)
        self._h = h
        basis._adopt(self)
        n = ctypes.c_int64()
        check(self._lib.tp3_mlp_num_params(h, ctypes.byref(n)))
        self.n_params = n.value

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            # a network lives on its context: when the context is already gone (both
            # collected together at interpreter exit) the handle is dropped, not freed
            if getattr(self._basis, "_ctx", None):
                self._lib.tp3_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        check(self._lib.tp3_mlp_get_params(self._h, out.ctypes.data, self.n_params), self._basis.ctx)
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise TP3Error(_lib.TP3_ERR_ARG, f"expected {self.n_params} parameters")
        check(self._lib.tp3_mlp_set_params(self._h, p.ctypes.data, self.n_params), self._basis.ctx)

    def forward_device(self, rows: int, d_x: int, d_out: int) -> None:
        """(u, s) per row into d_out (rows x 6 float32)."""
        check(self._lib.tp3_mlp_forward_device(self._h, rows, ctypes.c_void_p(d_x), ctypes.c_void_p(d_out)),
              self._basis.ctx)

    def loss_grad(self, rows: int, d_x: int, d_v: int, d_w: int, d_t: int = 0, shells: int = 1,
                  want_grad: bool = True):
        """Loss (regression of the targets d_t = (t, lambda) per candidate of `shells` rows
        on the steps, plus the weighted NLL of the steps under the log-scales) and its
        gradient (host float32) when want_grad."""
        loss = ctypes.c_double()
        g = np.empty(self.n_params, dtype=np.float32) if want_grad else None
        check(self._lib.tp3_mlp_loss_grad(self._h, rows, ctypes.c_void_p(d_x), ctypes.c_void_p(d_v),
                                          ctypes.c_void_p(d_w), ctypes.c_void_p(d_t or None), shells,
                                          ctypes.byref(loss), g.ctypes.data if g is not None else None),
              self._basis.ctx)
        return loss.value, g

    def train_step(self, rows: int, d_x: int, d_v: int, d_w: int, lr: float, d_t: int = 0, shells: int = 1,
                   want_loss: bool = False):
        loss = ctypes.c_double()
        check(self._lib.tp3_mlp_train_step(self._h, rows, ctypes.c_void_p(d_x), ctypes.c_void_p(d_v),
                                           ctypes.c_void_p(d_w), ctypes.c_void_p(d_t or None), shells,
                                           ctypes.c_float(lr), ctypes.byref(loss) if want_loss else None),
              self._basis.ctx)
        return loss.value if want_loss else None


# ---------------------------------------------------------------------------
# Training on logged moves and the annealing comparison
# ---------------------------------------------------------------------------

def move_weights(meta):
    """NLL weight of a logged candidate (torch tensor [n, 7] -> [n]): accepted moves,
    counted more the more they lowered the energy (1 + min(-dE/T, 5) for dE < 0)."""
    import torch
    dE, T, acc = meta[:, 0], meta[:, 1], meta[:, 2]
    gain = torch.clamp(-dE / T, min=0.0, max=5.0)
    return acc * (1.0 + gain)


TARGET_CLIP = 30.0


def move_targets(meta):
    """Regression target of a logged candidate: its energy change relative to the
    launch's mean, over T (meta column 6), clipped to +-TARGET_CLIP so that the rare
    far-uphill candidates do not dominate the squared loss."""
    import torch
    return torch.clamp(meta[:, 6], min=-TARGET_CLIP, max=TARGET_CLIP)


def train_on_log(net: ProposalMLP, chains, steps: int, batch_candidates: int, lr: float = 1e-3, seed: int = 0,
                 holdout: float = 0.05, log_every: int = 0):
    """Adam steps on the training loss of logged candidates, batches of whole candidates
    (K rows each) drawn uniformly from the move log: the mean squared residual of the
    energy-change targets regressed on the steps through the drift heads u, plus the
    weighted NLL of the steps under the log-scale heads.  Returns (train losses,
    held-out loss before, held-out loss after); held-out candidates are never trained on."""
    import torch
    dev = torch.device("cuda")
    K = chains.basis.K
    total = chains.move_log_count()
    if total < 2:
        raise TP3Error(_lib.TP3_ERR_ARG, "move log is empty")
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(total, generator=g)
    nh = max(1, int(total * holdout))
    hold, train = perm[:nh], perm[nh:]
    nb = min(batch_candidates, train.numel())
    rows = (nb * K + 127) // 128 * 128
    if rows > net.max_rows:
        raise TP3Error(_lib.TP3_ERR_ARG, "batch exceeds the network's max_rows")
    X = torch.zeros((rows, net.stride), dtype=torch.bfloat16, device=dev)
    V = torch.zeros((rows, 3), dtype=torch.float32, device=dev)
    W = torch.zeros(rows, dtype=torch.float32, device=dev)
    Tg = torch.zeros((rows // K, 2), dtype=torch.float32, device=dev)
    M = torch.zeros((nb, 7), dtype=torch.float32, device=dev)

    def fill(idx_cpu):
        n = idx_cpu.numel()
        idx = idx_cpu.to(dev, dtype=torch.int64)
        torch.cuda.synchronize()   # indices (PyTorch's stream) before the gather reads them
        chains.move_log_gather(n, idx.data_ptr(), X.data_ptr(), V.data_ptr(), M.data_ptr())
        chains.basis.sync()        # gathered rows before PyTorch computes the weights
        w = move_weights(M[:n])
        W.zero_()
        W[: n * K] = (w / torch.clamp(w.sum(), min=1e-12)).repeat_interleave(K)
        Tg.zero_()
        Tg[:n, 0] = move_targets(M[:n])
        Tg[:n, 1] = 1.0 / n
        if n * K < rows:
            X[n * K:].zero_()
            V[n * K:].zero_()
        torch.cuda.synchronize()   # weights and padding before the library trains on them

    def heldout_loss():
        tot, wsum = 0.0, 0
        for a in range(0, nh, nb):
            part = hold[a:a + nb]
            fill(part)
            l, _ = net.loss_grad(rows, X.data_ptr(), V.data_ptr(), W.data_ptr(), Tg.data_ptr(), K, want_grad=False)
            tot += l * part.numel()
            wsum += part.numel()
        return tot / max(wsum, 1)

    before = heldout_loss()
    losses = []
    for it in range(steps):
        pick = train[torch.randint(0, train.numel(), (nb,), generator=g)]
        fill(pick)
        want = log_every and (it % log_every == 0 or it == steps - 1)
        l = net.train_step(rows, X.data_ptr(), V.data_ptr(), W.data_ptr(), lr, Tg.data_ptr(), K, want_loss=bool(want))
        if want:
            losses.append((it, l))
    after = heldout_loss()
    return losses, before, after


def time_to_energy(chains, target: float, max_launches: int, chunk: int = 10):
    """Run launches in chunks until the median chain energy is <= target; returns
    (seconds of device time, launches, median energy reached, energy trace)."""
    import time
    import torch
    trace = []
    t0 = time.perf_counter()
    done = 0
    med = float("inf")
    while done < max_launches:
        n = min(chunk, max_launches - done)
        chains.run(n)
        done += n
        st = chains.state()
        med = float(np.median(st["E"]))
        trace.append((done, time.perf_counter() - t0, med))
        if med <= target:
            break
    torch.cuda.synchronize()
    return time.perf_counter() - t0, done, med, trace


def haar_axis_angles(rng: np.random.Generator, shape) -> np.ndarray:
    """Axis-angle vectors (shape + (3,)) of Haar-uniform rotations (uniform unit quaternions)."""
    q = rng.normal(size=tuple(shape) + (4,))
    q /= np.linalg.norm(q, axis=-1, keepdims=True)
    q *= np.where(q[..., :1] < 0, -1.0, 1.0)
    w = np.clip(q[..., 0], -1.0, 1.0)
    ang = 2.0 * np.arccos(w)
    s = np.sqrt(np.maximum(1.0 - w * w, 1e-300))
    return q[..., 1:] / s[..., None] * ang[..., None]


def rotated_starts(basis, base: np.ndarray, nchains: int, seed: int) -> np.ndarray:
    """nchains copies of base[:K] with every shell turned by its own Haar-random rotation
    (on the device, tp3_rotate_shells_device)."""
    import torch
    K, ncoef = basis.K, basis.LMAX ** 2
    rng = np.random.default_rng(seed)
    v = haar_axis_angles(rng, (nchains, K))
    dev = torch.device("cuda")
    c = np.repeat(np.ascontiguousarray(base[:K], dtype=np.complex128)[None], nchains, axis=0)
    d_c = torch.from_numpy(c.view(np.float64).copy()).to(dev)
    d_v = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
    basis.rotate_shells_device(nchains, d_c.data_ptr(), d_v.data_ptr(), d_c.data_ptr())
    basis.sync()
    return d_c.cpu().numpy().view(np.complex128).reshape(nchains, K, ncoef)


def learned_vs_plain(basis, base: np.ndarray, nchains: int = 64, ncand: int = 16, collect_launches: int = 977,
                     train_steps: int = 1500, batch_candidates: int = 1024, eval_launches: int = 300,
                     sigma0: float = 0.2, stepsizefactor: float = 1.02, temperature_decay: float = 0.9995,
                     temperature_factor: float = 0.1, p_net: float = 0.8, hidden: int = 512, lr: float = 1e-3,
                     seed: int = 2024, chunk: int = 10, drift: bool = True) -> dict:
    """The learned-proposal experiment on the basis's histogram (set beforehand):
    1. the plain annealer (isotropic per-shell steps) logs its moves from Haar-rotated
       starts (collect_launches x nchains x ncand candidates);
    2. the network is trained on the device on those moves (regression of their energy
       changes on the steps through the drift heads, NLL of the steps under the log-scales);
    3. from fresh starts (another seed), the plain annealer runs eval_launches launches;
       its final median energy is the target;
    4. the learned annealer (mixture p_net network / isotropic, MH-corrected) runs from
       the same starts with the same schedule until its median energy reaches the target;
    5. (drift=True) the network-free drift annealer (the same mixture with the drift along
       the newest gradient estimate, TP3_MOVE_DRIFT) does the same: the ablation that
       shows what the trained network adds over its strongest input.
    Times are wall clock around graph replays (chunks of `chunk` launches)."""
    import time
    from .chains import Chains
    K, L = basis.K, basis.L
    out = {"nchains": nchains, "candidates_per_launch": ncand, "sigma0": sigma0, "stepsizefactor": stepsizefactor,
           "temperature_decay": temperature_decay, "p_net": p_net, "hidden": hidden}
    # temperature: temperature_factor x std of the start energies
    starts_c = rotated_starts(basis, base, nchains, seed)
    E0 = basis.energy_batch(starts_c)
    T0 = temperature_factor * float(np.std(E0))
    out["T0"] = T0
    # 1. collect
    t = time.perf_counter()
    col = Chains(basis, starts_c, T0, 0.1, stepsizefactor, temperature_decay, seed + 1, ncand=ncand)
    col.set_move(1, sigma0)
    col.enable_move_log(collect_launches)
    col.run(collect_launches)
    n_moves = col.move_log_count()
    out["collect"] = {"launches": collect_launches, "moves": n_moves, "seconds": time.perf_counter() - t,
                      "median_E_end": float(np.median(col.state()["E"]))}
    # 2. train
    t = time.perf_counter()
    rows = max(((nchains * ncand * K + 127) // 128) * 128, ((batch_candidates * K + 127) // 128) * 128)
    net = ProposalMLP(basis, n_in_for(L), hidden=hidden, max_rows=rows, seed=seed + 2)
    losses, before, after = train_on_log(net, col, train_steps, batch_candidates, lr=lr, seed=seed + 3,
                                         log_every=max(1, train_steps // 10))
    col.close()
    out["train"] = {"steps": train_steps, "batch_candidates": batch_candidates, "lr": lr,
                    "heldout_nll_before": before, "heldout_nll_after": after, "seconds": time.perf_counter() - t,
                    "loss_trace": losses}
    # 3. plain
    ev_starts = rotated_starts(basis, base, nchains, seed + 10)
    plain = Chains(basis, ev_starts, T0, 0.1, stepsizefactor, temperature_decay, seed + 11, ncand=ncand)
    plain.set_move(1, sigma0)
    plain.run(1)
    sec_p, n_p, med_p, trace_p = time_to_energy(plain, -float("inf"), eval_launches - 1, chunk)
    stp = plain.state()
    plain.close()
    target = med_p
    # 4. learned
    lrn = Chains(basis, ev_starts, T0, 0.1, stepsizefactor, temperature_decay, seed + 11, ncand=ncand)
    lrn.set_move(2, sigma0, p_net, net)
    lrn.run(1)
    sec_l, n_l, med_l, trace_l = time_to_energy(lrn, target, eval_launches - 1, chunk)
    stl = lrn.state()
    lrn.close()
    net.close()
    if drift:
        # 5. drift-only ablation: same starts, schedule, seed and mixture weight
        dr = Chains(basis, ev_starts, T0, 0.1, stepsizefactor, temperature_decay, seed + 11, ncand=ncand)
        dr.set_move(3, sigma0, p_net)
        dr.run(1)
        sec_d, n_d, med_d, trace_d = time_to_energy(dr, target, eval_launches - 1, chunk)
        std = dr.state()
        dr.close()
        out["drift"] = {"seconds_to_target": sec_d, "launches": n_d + 1, "median_E": med_d,
                        "reached": bool(med_d <= target),
                        "accept_rate": float(std["accepted"].sum() / max(std["steps"].sum(), 1)), "trace": trace_d}
        out["time_ratio_drift"] = sec_d / sec_p if med_d <= target else None
    out["plain"] = {"seconds": sec_p, "launches": n_p + 1, "final_median_E": med_p,
                    "accept_rate": float(stp["accepted"].sum() / max(stp["steps"].sum(), 1)), "trace": trace_p}
    out["learned"] = {"seconds_to_target": sec_l, "launches": n_l + 1, "median_E": med_l,
                      "reached": bool(med_l <= target),
                      "accept_rate": float(stl["accepted"].sum() / max(stl["steps"].sum(), 1)), "trace": trace_l}
    out["time_ratio"] = sec_l / sec_p if med_l <= target else None
    return out
