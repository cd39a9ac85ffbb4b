"""Sequential FP64 annealing chain (oracle).

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).

Restates rotate_all_at_once / evaluate_step (src/determination.jl:281-338,
491-515) with the move get_MC_step (src/determination.jl:232-241): per even l in
2..L the complex rotation rtc[l] * (C^T R(beta) C) * ctr[l], beta ~ N(0, sigma_l),
applied to every shell, built here as a dense (2l+1) x (2l+1) matrix product.

The random numbers follow the stream the device chains use, so both walk the same
trajectory: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) with key = seed and
counter = (step, chain, purpose, index); purpose 0 draws the angle of order l
(index l), purpose 1 the plane (index 64 l + j, four normals per call, Box-Muller
on (x + 0.5) 2^-32), purpose 2 the Metropolis uniform.
"""
from __future__ import annotations

import math

import numpy as np

from .sh import Umat, seanindex

M32 = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    """Philox4x32 with 10 rounds (Random123's philox4x32_R, R = 10)."""
    c = [int(x) & M32 for x in ctr]
    k0, k1 = int(key[0]) & M32, int(key[1]) & M32
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        hi0, lo0 = p0 >> 32, p0 & M32
        hi1, lo1 = p1 >> 32, p1 & M32
        c = [(hi1 ^ c[1] ^ k0) & M32, lo1, (hi0 ^ c[3] ^ k1) & M32, lo0]
        k0 = (k0 + 0x9E3779B9) & M32
        k1 = (k1 + 0xBB67AE85) & M32
    return c


def _key(seed: int):
    return (seed & M32, (seed >> 32) & M32)


def u01(x: int) -> float:
    return (x + 0.5) * 2.0 ** -32


def normals4(seed: int, step: int, chain: int, purpose: int, index: int):
    c = philox4x32_10((step & M32, chain, purpose, index), _key(seed))
    out = []
    for h in range(2):
        r = math.sqrt(-2.0 * math.log(u01(c[2 * h])))
        a = 2.0 * math.pi * u01(c[2 * h + 1])
        out += [r * math.cos(a), r * math.sin(a)]
    return out


def plane(seed: int, step: int, chain: int, l: int):
    d = 2 * l + 1
    z = []
    j = 0
    while len(z) < 2 * d:
        z += normals4(seed, step, chain, 1, 64 * l + j)
        j += 1
    p = np.array(z[:d])
    q = np.array(z[d:2 * d])
    p /= math.sqrt(p @ p)
    q -= (p @ q) * p
    q /= math.sqrt(q @ q)
    return p, q


def propose(coeff: np.ndarray, L: int, LMAX: int, sigma: dict, seed: int, step: int, chain: int) -> np.ndarray:
    """One get_MC_step with the device stream's random numbers (dense matrices)."""
    out = coeff.copy()
    for l in range(2, L + 1, 2):
        p, q = plane(seed, step, chain, l)
        beta = normals4(seed, step, chain, 0, l)[0] * sigma[l]
        d = 2 * l + 1
        M = (np.eye(d) + (math.cos(beta) - 1.0) * (np.outer(p, p) + np.outer(q, q))
             + math.sin(beta) * (np.outer(q, p) - np.outer(p, q)))
        U = Umat(l)
        rot = U.conj().T @ M @ U
        idx = [seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)]
        out[:, idx] = (rot @ coeff[:, idx].T).T
    return out


class SequentialChain:
    """The chain of run_chain advanced one step at a time (rotate_all_at_once /
    evaluate_step, src/determination.jl:281-338, 491-515): peek() proposes the next
    candidate and evaluates its energy change and natural Metropolis decision; commit(acc)
    takes a decision, so a comparison can make the oracle follow a device chain through a
    decision that lies within the energy tolerance of its boundary."""

    def __init__(self, energy_fn, coeff0: np.ndarray, L: int, LMAX: int, T0: float, initial_stepsize: float,
                 stepsizefactor: float, temperature_decay: float, seed: int, chain: int):
        self.energy_fn, self.L, self.LMAX = energy_fn, L, LMAX
        self.f, self.decay, self.seed, self.chain = stepsizefactor, temperature_decay, seed, chain
        self.state = coeff0.copy()
        self.E = energy_fn(self.state)
        self.T = T0
        self.sigma = {l: initial_stepsize * (l - 1) for l in range(2, L + 1, 2)}
        self.s = 0
        self._pending = None

    def peek(self) -> dict:
        T = self.T * self.decay
        cand = propose(self.state, self.L, self.LMAX, self.sigma, self.seed, self.s, self.chain)
        En = self.energy_fn(cand)
        dE = En - self.E
        ap = math.exp(-dE / T) if -dE / T < 700 else float("inf")
        u = u01(philox4x32_10((self.s & M32, self.chain, 2, 0), _key(self.seed))[0])
        acc = dE < 0.0 or (dE > 0.0 and u < ap)
        self._pending = dict(cand=cand, En=En, dE=dE, T=T, ap=ap, u=u, acc=acc)
        return self._pending

    def commit(self, acc: bool) -> list:
        p = self._pending
        self._pending = None
        self.T = p["T"]
        sign = 0.0
        if acc:
            sign = 1.0 if p["dE"] < 0.0 else -1.0
            for l in self.sigma:
                self.sigma[l] *= self.f
            self.E = p["En"]
            self.state = p["cand"]
        else:
            for l in self.sigma:
                self.sigma[l] /= self.f
        self.s += 1
        return [self.s, sign, p["En"], self.E, p["dE"], p["T"], p["ap"],
                self.sigma[max(self.sigma)] if self.sigma else 0.0]


def run_chain(energy_fn, coeff0: np.ndarray, L: int, LMAX: int, T0: float, initial_stepsize: float,
              stepsizefactor: float, temperature_decay: float, seed: int, chain: int, nsteps: int):
    """Sequential chain; returns (final coeff, E, T, sigma, log rows [step, sign, E_new, E, dE, T, ap, sigma_L])."""
    state = coeff0.copy()
    E = energy_fn(state)
    T = T0
    sigma = {l: initial_stepsize * (l - 1) for l in range(2, L + 1, 2)}
    rows = []
    for s in range(nsteps):
        T *= temperature_decay
        cand = propose(state, L, LMAX, sigma, seed, s, chain)
        En = energy_fn(cand)
        dE = En - E
        ap = math.exp(-dE / T) if -dE / T < 700 else float("inf")
        u = u01(philox4x32_10((s & M32, chain, 2, 0), _key(seed))[0])
        acc = dE < 0.0 or (dE > 0.0 and u < ap)
        sign = 0.0
        if acc:
            sign = 1.0 if dE < 0.0 else -1.0
            for l in sigma:
                sigma[l] *= stepsizefactor
            E = En
            state = cand
        else:
            for l in sigma:
                sigma[l] /= stepsizefactor
        rows.append([s + 1, sign, En, E, dE, T, ap, sigma[max(sigma)] if sigma else 0.0])
    return state, E, T, sigma, np.array(rows)


# ---------------------------------------------------------------------------
# Per-shell SO(3) moves (no reference counterpart: the learned-proposal experiment).
# Stream: purpose 3 index 0 (counter step) = component uniform; the step noise of
# candidate i of a launch = purpose 5 + 16 i, index k (counter launch) = the three
# normals of shell k; index 64 = the network step's side.
# ---------------------------------------------------------------------------

def rodrigues(v) -> np.ndarray:
    v = np.asarray(v, dtype=np.float64)
    a = float(np.linalg.norm(v))
    if a == 0.0:
        return np.eye(3)
    u = v / a
    Kx = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
    return math.cos(a) * np.eye(3) + math.sin(a) * Kx + 2.0 * math.sin(0.5 * a) ** 2 * np.outer(u, u)


def rotate_shells(coeff: np.ndarray, v: np.ndarray, L: int, LMAX: int) -> np.ndarray:
    """Shell k's even orders l = 2..L rotated by exp([v_k]x) (action on functions)."""
    from .sh import wigner_D_sampled
    out = coeff.copy()
    for k in range(coeff.shape[0]):
        R = rodrigues(v[k])
        for l in range(2, L + 1, 2):
            idx = [seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)]
            out[k, idx] = wigner_D_sampled(l, R) @ coeff[k, idx]
    return out


def component_uniform(seed: int, step: int, chain: int) -> float:
    """The uniform that picks the network (u < p_net) or the isotropic step."""
    return u01(philox4x32_10((step & M32, chain, 3, 0), _key(seed))[0])


def shell_noise(seed: int, launch: int, chain: int, i: int, K: int):
    """Unit normals z[K][3] of candidate i of a launch and the network step's side a = +-1."""
    z = np.array([normals4(seed, launch, chain, 5 + 16 * i, k)[:3] for k in range(K)])
    c = philox4x32_10((launch & M32, chain, 5 + 16 * i, 64), _key(seed))
    return z, (-1.0 if u01(c[0]) < 0.5 else 1.0)


def rot_logdens(v, mu, s) -> float:
    """log density of the rotation exp([v]x) under N(mu, diag(exp(2 s))) up to the Haar
    factor common to a move and its reverse (preimages |v| + 2 pi n, n = -1, 0, 1)."""
    v, mu, s = (np.asarray(x, dtype=np.float64) for x in (v, mu, s))
    th = float(np.linalg.norm(v))
    terms = []
    for n in ((-1, 0, 1) if th > 0 else (0,)):
        f = (th + 2 * math.pi * n) / th if th > 0 else 1.0
        z = (v * f - mu) * np.exp(-s)
        terms.append(-0.5 * float(z @ z) - float(s.sum()) - 1.5 * math.log(2 * math.pi)
                     + 2.0 * math.log(abs(f) if f != 0 else 1e-300))
    m = max(terms)
    return m + math.log(sum(math.exp(t - m) for t in terms))


def drift_factor(u_hat) -> float:
    """sqrt(gamma) / sqrt(sum over the candidate's shells of |u|^2 + eps^2)."""
    from .mlp import DRIFT_GAMMA, DRIFT_EPS
    u = np.asarray(u_hat, dtype=np.float64)
    return math.sqrt(DRIFT_GAMMA) / math.sqrt(float(np.sum(u * u)) + DRIFT_EPS ** 2)


def shell_params(u_hat, s_hat, sigma: float):
    """Per-shell step parameters from the network head relative to the isotropic step
    size: drift m = sigma f u^ (f = drift_factor), s = log sigma + s^ - mean over shells
    of s^."""
    u_hat, s_hat = np.asarray(u_hat, dtype=np.float64), np.asarray(s_hat, dtype=np.float64)
    return sigma * drift_factor(u_hat) * u_hat, math.log(sigma) + s_hat - s_hat.mean(axis=0, keepdims=True)


def net_logdens(v, m, s) -> float:
    """log q_net(v) = log((prod_k q(v_k; +m_k, s_k) + prod_k q(v_k; -m_k, s_k)) / 2)."""
    K = v.shape[0]
    lp = sum(rot_logdens(v[k], m[k], s[k]) for k in range(K))
    lm = sum(rot_logdens(v[k], -m[k], s[k]) for k in range(K))
    return float(np.logaddexp(lp, lm) - math.log(2.0))


def mixture_log_ratio(v, m, s, m2, s2, sigma: float, p_net: float) -> float:
    """log q(x|x') - log q(x'|x) of the mixture p q_net + (1 - p) q_iso over all shells;
    (m, s) the network's step parameters at x, (m2, s2) at x'."""
    K = v.shape[0]
    ls = np.full(3, math.log(sigma))
    fnet = net_logdens(v, m, s)
    rnet = net_logdens(-v, m2, s2)
    fiso = sum(rot_logdens(v[k], np.zeros(3), ls) for k in range(K))
    lp = math.log(p_net)
    lq = math.log1p(-p_net) if p_net < 1 else -math.inf
    return float(np.logaddexp(lp + rnet, lq + fiso) - np.logaddexp(lp + fnet, lq + fiso))


def gradient_estimate(dE, T1: float, w) -> np.ndarray:
    """The launch's per-shell gradient estimate from its B candidates (all drawn at the
    same state): e = (1/n) sum_i ((dE_i - mean dE) / T1) w_i over the n candidates with a
    finite dE; w [B][K][3] the whitened step noise (z for an isotropic step)."""
    dE = np.asarray(dE, dtype=np.float64)
    w = np.asarray(w, dtype=np.float64)
    ok = np.isfinite(dE)
    if not ok.any():
        return np.zeros(w.shape[1:])
    d = dE[ok] - dE[ok].mean()
    return np.tensordot(d, w[ok], axes=(0, 0)) / (ok.sum() * T1)


def run_shell_chain(energy_fn, coeff0: np.ndarray, L: int, LMAX: int, T0: float, sigma0: float,
                    stepsizefactor: float, temperature_decay: float, seed: int, chain: int, nlaunches: int,
                    ncand: int):
    """Chain with the isotropic per-shell move, run as launches of ncand speculative
    candidates (candidate i of a launch assumes i rejections: sigma / f^i, T decay^(i+1),
    noise of its own launch-keyed stream); a launch takes its first accepted candidate
    or ncand rejections.  Rows as run_chain, one per step up to the taken one."""
    state = coeff0.copy()
    E = energy_fn(state)
    T, sigma = T0, sigma0
    rows = []
    K = coeff0.shape[0]
    step = 0
    for launch in range(nlaunches):
        for i in range(ncand):
            T *= temperature_decay
            z, _ = shell_noise(seed, launch, chain, i, K)
            cand = rotate_shells(state, sigma * z, L, LMAX)
            En = energy_fn(cand)
            dE = En - E
            ap = math.exp(-dE / T) if -dE / T < 700 else float("inf")
            u = u01(philox4x32_10((step & M32, chain, 2, 0), _key(seed))[0])
            acc = dE < 0.0 or (dE > 0.0 and u < ap)
            sign = 0.0
            if acc:
                sign = 1.0 if dE < 0.0 else -1.0
                sigma *= stepsizefactor
                E = En
                state = cand
            else:
                sigma /= stepsizefactor
            step += 1
            rows.append([step, sign, En, E, dE, T, ap, sigma])
            if acc:
                break
    return state, E, T, sigma, np.array(rows)
