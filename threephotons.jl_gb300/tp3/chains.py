"""Device-resident annealing chains over libtp3 (tp3_chains_*).

Mirrors the reference's annealing driver (src/determination.jl): ``Chains`` runs
many independent rotate_all_at_once chains with the get_MC_step move on the GPU;
``calculate_temperature`` is src/determination.jl:244-261 (std of the energies of
50 proposals times initial_temperature_factor), with the proposals scored on the
GPU in one batch.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import TP3Error, check, load
from .api import BasisTypeGB300, Umat
from .structure import seanindex0

MINSTEPSIZE = 1.5 * math.pi / 180.0  # src/determination.jl:1


def get_MC_step(coeff: np.ndarray, basis: BasisTypeGB300, stepsizes: dict, rng: np.random.Generator) -> np.ndarray:
    """Host version of get_MC_step (src/determination.jl:232-241) with numpy randomness."""
    out = np.array(coeff, dtype=np.complex128, copy=True)
    for l in range(2, basis.L + 1, 2):
        d = 2 * l + 1
        beta = rng.normal() * stepsizes[l]
        while True:
            Q, R = np.linalg.qr(rng.normal(size=(d, d)))
            Q = Q * np.sign(np.diag(R))
            if np.linalg.det(Q) > 0:
                break
        Rm = np.eye(d)
        Rm[0, 0] = math.cos(beta); Rm[0, 1] = -math.sin(beta)
        Rm[1, 0] = math.sin(beta); Rm[1, 1] = math.cos(beta)
        rot = basis.rtc[l] @ (Q.T @ Rm @ Q) @ basis.ctr[l]
        idx = [seanindex0(l, m, basis.LMAX) for m in range(-l, l + 1)]
        out[:, idx] = (rot @ coeff[:, idx].T).T
    return out


def calculate_temperature(coeff: np.ndarray, basis: BasisTypeGB300, c3ref, stepsizes: dict,
                          initial_temperature_factor: float, iterations: int = 50, seed: int = 0) -> float:
    """std(energies of `iterations` proposals) * factor (src/determination.jl:244-261)."""
    if initial_temperature_factor <= 0.0:
        return 0.0
    basis._ensure_histogram(c3ref)
    rng = np.random.default_rng(seed)
    props = np.stack([get_MC_step(coeff[: basis.K], basis, stepsizes, rng) for _ in range(iterations)])
    E = basis.energy_batch(props)
    return float(np.std(E, ddof=1) * initial_temperature_factor)


class Chains:
    """n chains x B speculative candidates per launch on one basis (context)."""

    def __init__(self, basis: BasisTypeGB300, coeff0: np.ndarray, T0, initial_stepsize: float,
                 stepsizefactor: float, temperature_decay: float, seed: int, ncand: int = 16,
                 log_capacity: int = 0, shapes=None):
        """shapes (ragged chains): per chain (L, K, histogram index) of basis.set_histograms."""
        self.basis = basis
        self._lib = load()
        c = np.ascontiguousarray(np.asarray(coeff0)[:, : basis.K], dtype=np.complex128)
        if c.ndim != 3 or c.shape[2] != basis.LMAX ** 2:
            raise TP3Error(_lib.TP3_ERR_ARG, "coeff0 must be [nchains, K, LMAX^2]")
        self.n = c.shape[0]
        self.ncand = ncand
        self.log_capacity = log_capacity
        T = np.ascontiguousarray(np.broadcast_to(np.asarray(T0, dtype=np.float64), (self.n,)))
        self._h = ctypes.c_void_p()
        if shapes is None:
            check(self._lib.tp3_chains_create(basis.ctx, self.n, ncand, c.ctypes.data, T.ctypes.data,
                                              float(initial_stepsize), float(stepsizefactor),
                                              float(temperature_decay), ctypes.c_uint64(seed), log_capacity,
                                              ctypes.byref(self._h)), basis.ctx)
        else:
            lkh = np.ascontiguousarray(shapes, dtype=np.int32).reshape(self.n, 3)
            check(self._lib.tp3_chains_create_ragged(basis.ctx, self.n, ncand, c.ctypes.data, T.ctypes.data,
                                                     float(initial_stepsize), float(stepsizefactor),
                                                     float(temperature_decay), ctypes.c_uint64(seed), log_capacity,
                                                     lkh.ctypes.data, ctypes.byref(self._h)), basis.ctx)
        basis._adopt(self)

    def run(self, launches: int) -> None:
        check(self._lib.tp3_chains_run(self._h, launches), self.basis.ctx)

    def state(self):
        n, nl = self.n, self.basis.L // 2 + 1
        E = np.empty(n); T = np.empty(n); sig = np.empty((n, nl))
        steps = np.empty(n, dtype=np.int64); acc = np.empty(n, dtype=np.int64)
        check(self._lib.tp3_chains_state(self._h, E.ctypes.data, T.ctypes.data, sig.ctypes.data,
                                         steps.ctypes.data, acc.ctypes.data), self.basis.ctx)
        return {"E": E, "T": T, "sigma": sig, "steps": steps, "accepted": acc}

    def coeff(self) -> np.ndarray:
        out = np.empty((self.n, self.basis.K, self.basis.LMAX ** 2), dtype=np.complex128)
        check(self._lib.tp3_chains_coeff(self._h, out.ctypes.data), self.basis.ctx)
        return out

    def log(self, chain: int) -> np.ndarray:
        rows = np.empty((max(self.log_capacity, 1), 8))
        n = ctypes.c_int64()
        check(self._lib.tp3_chains_log(self._h, chain, rows.ctypes.data, ctypes.byref(n)), self.basis.ctx)
        return rows[: n.value].copy()

    def snapshot(self) -> bytes:
        size = ctypes.c_size_t()
        check(self._lib.tp3_chains_snapshot(self._h, None, 0, ctypes.byref(size)), self.basis.ctx)
        buf = ctypes.create_string_buffer(size.value)
        check(self._lib.tp3_chains_snapshot(self._h, buf, size.value, ctypes.byref(size)), self.basis.ctx)
        return buf.raw

    def restore(self, blob: bytes) -> None:
        check(self._lib.tp3_chains_restore(self._h, blob, len(blob)), self.basis.ctx)

    def set_move(self, kind: int, sigma0: float = 0.1, p_net: float = 0.0, net=None) -> None:
        """Move kind: 0 reference get_MC_step, 1 per-shell isotropic SO(3) step with
        sigma0 (radians), 2 mixture of the network's step (probability p_net) and the
        isotropic one, Metropolis-Hastings corrected, 3 the same mixture with the drift
        along the newest gradient estimate instead of a network (symmetric proposal)."""
        check(self._lib.tp3_chains_set_move(self._h, kind, float(sigma0), float(p_net),
                                            net.handle if net is not None else None), self.basis.ctx)

    def enable_move_log(self, launches: int) -> None:
        check(self._lib.tp3_chains_enable_move_log(self._h, launches), self.basis.ctx)

    def move_log_count(self) -> int:
        n = ctypes.c_int64()
        check(self._lib.tp3_chains_move_log_count(self._h, ctypes.byref(n)), self.basis.ctx)
        return n.value

    def move_log_gather(self, n: int, d_idx: int, d_x: int, d_v: int, d_meta: int) -> None:
        """Device pointers: idx int64[n]; x bf16[n*K][stride]; v float[n*K][3] (steps / sigma_i);
        meta float[n][7] (dE, T, accepted, drawn-from-network, log MH ratio, sigma_i,
        (dE - mean dE over the launch's candidates) / T)."""
        check(self._lib.tp3_chains_move_log_gather(self._h, n, ctypes.c_void_p(d_idx), ctypes.c_void_p(d_x),
                                                   ctypes.c_void_p(d_v), ctypes.c_void_p(d_meta)), self.basis.ctx)

    @property
    def graph_captured(self) -> bool:
        v = ctypes.c_int()
        check(self._lib.tp3_chains_graph(self._h, ctypes.byref(v)), self.basis.ctx)
        return bool(v.value)

    def close(self) -> None:
        if self._h:
            # chains live on their context: when it is already gone (both collected
            # together at interpreter exit) the handle is dropped, not freed
            if getattr(self.basis, "_ctx", None):
                self._lib.tp3_chains_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
