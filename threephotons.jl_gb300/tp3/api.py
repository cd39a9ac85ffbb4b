"""Host-side mirror of the reference's hot-path API over libtp3.

Same names, argument meaning and error behaviour as the Julia functions the
annealing loop calls:

    CUDA_init()                                   src/cuda.jl:10-22
    calculate_basis / complexBasis_choice          src/correlations.jl:87-153, src/cuda.jl:57-71
    FullCorrelation_parallized(intensity, basis,
        minimal=True, normalize=False, return_raw=False)   src/cuda.jl:74-108
    energy(intensity, basis, c3ref, K3_range, measure="Bayes", negativity_factor=0.0)
                                                  src/correlations.jl:196-226
    get_MC_step / random_rotation(_step)           src/determination.jl:232-241, src/utilities.jl:165-190
    rotationMatrix / rotateStructure               src/spherical_harmonics.jl:588-603

Every number that is part of c3 or the energy is computed by libtp3 on the GPU.
Errors raise ``TP3Error``; a missing library raises ImportError.  Nothing here
falls back to a CPU computation.
"""
from __future__ import annotations

import ctypes
import math
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import TP3Error, check, load


@dataclass
class SphericalHarmonicsVolume:
    """Shell-wise SH coefficients (src/spherical_harmonics.jl:9-31).

    coeff: complex128 [KMAX, LMAX^2], row k-1 = shell k, columns in seanindex order."""
    coeff: np.ndarray
    LMAX: int
    KMAX: int
    rmax: float

    def copy(self) -> "SphericalHarmonicsVolume":
        return SphericalHarmonicsVolume(self.coeff.copy(), self.LMAX, self.KMAX, self.rmax)


def dq(volume: SphericalHarmonicsVolume) -> float:
    """Shell spacing (spherical_harmonics.jl:95)."""
    return volume.rmax / volume.KMAX


def CUDA_init() -> None:
    """Load libtp3 and check that a CUDA device is usable (no CPU fallback)."""
    lib = load()
    ctx = ctypes.c_void_p()
    st = lib.tp3_ctx_create(0, 1, 2, 1, 0.0, 0.0, ctypes.byref(ctx))
    check(st)
    lib.tp3_ctx_destroy(ctx)


def Umat(l: int) -> np.ndarray:
    """Complex -> real SH transformation of order l (spherical_harmonics.jl:445-457)."""
    d = 2 * l + 1
    U = np.zeros((d, d), dtype=np.complex128)
    s = 1.0 / math.sqrt(2.0)
    for iu, u in enumerate(range(-l, l + 1)):
        for im, m in enumerate(range(-l, l + 1)):
            v = 0j
            if m == 0 and u == 0:
                v += 1.0
            if u > 0 and m == u:
                v += s
            if u < 0 and m == u:
                v += s * 1j * (-1) ** m
            if u < 0 and m == -u:
                v += -1j * s
            if u > 0 and m == -u:
                v += s * (-1) ** m
            U[iu, im] = v
    return U


def rotationMatrix(theta: float, phi: float, gamma: float, l: int) -> np.ndarray:
    """Wigner D of order l (spherical_harmonics.jl:588-592): D[m, s] = e^{-i s gamma - i m phi} d_ms(theta),
    m, s = -l..l (libtp3, FP64 on the host)."""
    d = 2 * l + 1
    out = np.empty(2 * d * d, dtype=np.float64)
    check(load().tp3_wigner_D(l, theta, phi, gamma, out.ctypes.data))
    return out.view(np.complex128).reshape(d, d, order="F")


def rotateStructure(volume: SphericalHarmonicsVolume, theta: float, phi: float, gamma: float, K: int,
                    lrange) -> SphericalHarmonicsVolume:
    """Rotate every shell 1..K by rotationMatrix for each l in lrange (spherical_harmonics.jl:595-603)."""
    from .structure import seanindex0
    new = volume.copy()
    for l in lrange:
        D = rotationMatrix(theta, phi, gamma, l)
        idx = [seanindex0(l, m, volume.LMAX) for m in range(-l, l + 1)]
        new.coeff[:K, idx] = volume.coeff[:K, idx] @ D.T
    return new


class BasisTypeGB300:
    """Device-resident basis (role of BasisTypeCuda, src/cuda.jl:24-42).

    Exposes the fields the annealing code reads (L, N, K, LMAX, lrange, ctr, rtc,
    lambda_, dq) and owns one libtp3 context."""

    def __init__(self, L: int, LMAX: int, N: int, K: int, lambda_: float = 0.0, dq: float = 0.0,
                 mode: int = _lib.TP3_MODE_AUTO):
        self.L, self.LMAX, self.N, self.K = L, LMAX, N, K
        self.lambda_, self.dq = float(lambda_), float(dq)
        self.lrange = list(range(0, L + 1, 2))
        self.ctr = {l: Umat(l) for l in self.lrange}
        self.rtc = {l: self.ctr[l].conj().T for l in self.lrange}
        self._lib = load()
        self._dependents = weakref.WeakSet()
        self._ctx = ctypes.c_void_p()
        check(self._lib.tp3_ctx_create(L, LMAX, N, K, self.lambda_, self.dq, ctypes.byref(self._ctx)))
        info = (ctypes.c_int64 * 8)()
        check(self._lib.tp3_basis_info(L, LMAX, N, K, self.lambda_, self.dq, info))
        self.basislen, self.n_lt, self.klength = int(info[0]), int(info[1]), int(info[2])
        self.nnz_pi2 = int(info[7])
        self.nc = int(info[6])
        self.set_mode(mode)
        self._hist_key = None
        self._hist_ref = None

    # -- context plumbing -------------------------------------------------------
    @property
    def ctx(self):
        return self._ctx

    def set_mode(self, mode: int) -> None:
        check(self._lib.tp3_set_mode(self._ctx, mode), self._ctx)

    @property
    def mode(self) -> int:
        m = ctypes.c_int()
        check(self._lib.tp3_get_mode(self._ctx, ctypes.byref(m)), self._ctx)
        return m.value

    def set_stream(self, stream_ptr) -> None:
        """Launch on this cudaStream_t handle; None restores the context's own stream."""
        check(self._lib.tp3_set_stream(self._ctx, None if stream_ptr is None else ctypes.c_void_p(stream_ptr)),
              self._ctx)

    def reserve(self, n: int) -> None:
        check(self._lib.tp3_reserve(self._ctx, n), self._ctx)

    def set_coupling(self, form: int) -> None:
        """Tensor-core coupling form: 0 one-kernel, 1 split, 2 one-kernel on 256 threads, 3 warp-local,
        4 warp-local on 256 threads (two CTAs per SM), 5 / 6 / 7 folded-row at 8 / 7 / 13 warps,
        8 folded-row at 14 warps in pairs (two warps per unit, 7 D buffers)."""
        check(self._lib.tp3_set_coupling(self._ctx, form), self._ctx)

    def autotune(self, n: int = 64) -> list:
        """Time every evaluation variant on n synthetic proposals, keep the fastest (also
        for later TP3_MODE_AUTO contexts of this shape); returns
        [(mode, coupling form, angular schedule, ms/proposal)] with coupling form 0 one-kernel,
        1 split, 2 one-kernel on 256 threads (two CTAs per SM), 3 warp-local one-kernel,
        4 warp-local on 256 threads (two CTAs per SM), 5 / 6 / 7 folded-row at 8 / 7 / 13
        warps, 8 folded-row at 14 warps in pairs, and angular schedule TP3_ANGULAR_PERSISTENT or TP3_ANGULAR_TILE (the
        fastest tensor-core variant is timed with both)."""
        cap = ctypes.c_int(24)
        rep = np.zeros(4 * 24)
        check(self._lib.tp3_autotune(self._ctx, n, rep.ctypes.data, ctypes.byref(cap)), self._ctx)
        return [(int(rep[4 * i]), int(rep[4 * i + 1]), int(rep[4 * i + 2]), float(rep[4 * i + 3]))
                for i in range(min(cap.value, 24))]

    def set_host_input(self, mode: int) -> None:
        """How energy_batch reaches host coefficients: TP3_HOST_INPUT_DIRECT (kernels read
        the array in place; the default where the device reads pageable host memory) or
        TP3_HOST_INPUT_STAGED (host packing + one pinned copy)."""
        check(self._lib.tp3_set_host_input(self._ctx, mode), self._ctx)

    def set_angular(self, schedule: int) -> None:
        """Angular-stage schedule of the tensor-core path: TP3_ANGULAR_PERSISTENT
        (default) or TP3_ANGULAR_TILE."""
        check(self._lib.tp3_set_angular(self._ctx, schedule), self._ctx)

    def _adopt(self, obj) -> None:
        """Register an object holding library handles on this context (chains, networks);
        close() releases it first, so no handle outlives its context."""
        self._dependents.add(obj)

    def close(self) -> None:
        for d in list(getattr(self, "_dependents", ())):
            d.close()
        if self._ctx:
            self._lib.tp3_ctx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- inputs -----------------------------------------------------------------
    def pack(self, coeff: np.ndarray) -> np.ndarray:
        """First K shells as a contiguous complex128 [K, LMAX^2] block."""
        c = np.asarray(coeff)
        if c.ndim != 2 or c.shape[0] < self.K or c.shape[1] != self.LMAX * self.LMAX:
            raise TP3Error(_lib.TP3_ERR_ARG, f"coefficients must be [>= {self.K}, {self.LMAX ** 2}], got {c.shape}")
        return np.ascontiguousarray(c[: self.K], dtype=np.complex128)

    def set_histogram(self, c3ref: np.ndarray) -> None:
        c = np.asarray(c3ref, dtype=np.float64)
        if c.ndim != 5 or c.shape[0] != self.N or c.shape[1] != 2 * self.N:
            raise TP3Error(_lib.TP3_ERR_ARG, f"c3ref must be N x 2N x K3 x K3 x K3, got {c.shape}")
        K3 = c.shape[2]
        if c.shape[3] != K3 or c.shape[4] != K3:
            raise TP3Error(_lib.TP3_ERR_ARG, "c3ref shell axes differ")
        cf = np.asfortranarray(c)
        check(self._lib.tp3_set_histogram(self._ctx, cf.ctypes.data, K3), self._ctx)
        self._hist_key = (id(c3ref), c.shape)
        self._hist_ref = c3ref

    def _ensure_histogram(self, c3ref) -> None:
        if self._hist_ref is not c3ref or self._hist_key != (id(c3ref), np.shape(c3ref)):
            self.set_histogram(c3ref)

    # -- compute ----------------------------------------------------------------
    def c3_raw(self, coeff: np.ndarray) -> np.ndarray:
        """G x klength float32 (column-major semantics of the reference's raw output)."""
        cc = self.pack(coeff)
        out = np.empty((self.klength, 2 * self.N * self.N), dtype=np.float32)
        check(self._lib.tp3_c3(self._ctx, cc.ctypes.data, out.ctypes.data), self._ctx)
        return out.T  # [G, klength]

    def triple_products(self, coeff: np.ndarray) -> np.ndarray:
        """T[ki, lt] (klength x n_lt, float32) from the current mode's coupling kernel."""
        cc = self.pack(coeff)
        out = np.empty((self.klength, self.n_lt), dtype=np.float32)
        check(self._lib.tp3_triple_products(self._ctx, cc.ctypes.data, out.ctypes.data), self._ctx)
        return out

    def sync(self) -> None:
        check(self._lib.tp3_sync(self._ctx), self._ctx)

    def energy_batch(self, coeffs: np.ndarray) -> np.ndarray:
        """Energies of a batch of coefficient sets, complex128 [n, >=K, LMAX^2]."""
        c = np.asarray(coeffs)
        if c.ndim != 3:
            raise TP3Error(_lib.TP3_ERR_ARG, "batch must be [n, K, LMAX^2]")
        cc = np.ascontiguousarray(c[:, : self.K], dtype=np.complex128)
        n = cc.shape[0]
        E = np.empty(n, dtype=np.float64)
        check(self._lib.tp3_energy_batch(self._ctx, n, cc.ctypes.data, E.ctypes.data), self._ctx)
        return E

    def energy_batch_device(self, n: int, d_coeffs_ptr: int, d_E_ptr: int) -> None:
        check(self._lib.tp3_energy_batch_device(self._ctx, n, ctypes.c_void_p(d_coeffs_ptr),
                                                ctypes.c_void_p(d_E_ptr)), self._ctx)

    def set_histograms(self, hists, Ks) -> None:
        """Histogram set of ragged batches: hists[h] as for set_histogram (N x 2N x K3 x K3 x K3,
        K3 >= Ks[h]), scored on its first Ks[h] shells."""
        arrs = [np.asfortranarray(h, dtype=np.float64) for h in hists]
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        K3 = np.array([a.shape[2] for a in arrs], dtype=np.int32)
        Kh = np.ascontiguousarray(Ks, dtype=np.int32)
        check(self._lib.tp3_set_histograms(self._ctx, len(arrs), ptrs, K3.ctypes.data, Kh.ctypes.data), self._ctx)
        self._hist_set = arrs  # keep alive until uploaded (the call copies)

    def energy_batch_ragged_device(self, n: int, d_coeffs_ptr: int, d_lkh_ptr: int, d_E_ptr: int) -> None:
        check(self._lib.tp3_energy_batch_ragged_device(self._ctx, n, ctypes.c_void_p(d_coeffs_ptr),
                                                       ctypes.c_void_p(d_lkh_ptr), ctypes.c_void_p(d_E_ptr)),
              self._ctx)

    def c3_batch_device(self, n: int, d_coeffs_ptr: int, d_c3_ptr: int) -> None:
        check(self._lib.tp3_c3_batch_device(self._ctx, n, ctypes.c_void_p(d_coeffs_ptr), ctypes.c_void_p(d_c3_ptr)),
              self._ctx)

    def rotate_shells_device(self, n: int, d_coeffs_ptr: int, d_axis_angle_ptr: int, d_out_ptr: int) -> None:
        """Rotate shell k of each of n device coefficient sets by exp([v]x), v = axis_angle[set][k] (FP64)."""
        check(self._lib.tp3_rotate_shells_device(self._ctx, n, ctypes.c_void_p(d_coeffs_ptr),
                                                 ctypes.c_void_p(d_axis_angle_ptr), ctypes.c_void_p(d_out_ptr)),
              self._ctx)

    def profile_enable(self, on: bool) -> None:
        check(self._lib.tp3_profile_enable(self._ctx, int(on)), self._ctx)

    def profile_read(self, stage: int = 0):
        """(launches, summed ms) of stage 0 (angular + Bayes) or 1 (coupling) since the last read."""
        n = ctypes.c_int64()
        ms = ctypes.c_double()
        check(self._lib.tp3_profile_read_stage(self._ctx, int(stage), ctypes.byref(n), ctypes.byref(ms)), self._ctx)
        return n.value, ms.value

    def measure_fp32_peak(self) -> float:
        """Measured FP32 FMA peak of the device in TFLOP/s (the coupling stage's roofline)."""
        v = ctypes.c_double()
        check(self._lib.tp3_measure_fp32_peak(self._ctx, ctypes.byref(v)), self._ctx)
        return v.value


def calculate_basis(L: int, LMAX: int, N: int, K: int, lambda_: float = 0.0, dq: float = 0.0,
                    forIntensity: bool = True) -> BasisTypeGB300:
    """Basis factory (correlations.jl:87; rebound as complexBasis_choice in cuda.jl:71)."""
    if not forIntensity:
        raise TP3Error(_lib.TP3_ERR_UNSUPPORTED, "only the intensity basis (lrange = 0:2:L) is on the hot path")
    return BasisTypeGB300(L, LMAX, N, K, lambda_, dq)


complexBasis_choice = calculate_basis


def FullCorrelation_parallized(intensity: SphericalHarmonicsVolume, basis: BasisTypeGB300, minimal: bool = True,
                               normalize: bool = False, return_raw: bool = False) -> np.ndarray:
    """c3 of one structure (src/cuda.jl:74-108)."""
    res = basis.c3_raw(intensity.coeff).astype(np.float64)
    if return_raw:
        return res
    N, K = basis.N, basis.K
    t = np.zeros((N, 2 * N, K, K, K), dtype=np.float64, order="F")
    i = 0
    for k1 in range(1, K + 1):
        for k2 in range(1, k1 + 1):
            for k3 in range(1, k2 + 1):
                t[:, :, k3 - 1, k2 - 1, k1 - 1] = res[:, i].reshape(N, 2 * N, order="F")
                i += 1
    return t / np.sum(np.abs(t)) if normalize else t


def energy(intensity: SphericalHarmonicsVolume, basis: BasisTypeGB300, c3ref: np.ndarray, K3_range=None,
           measure: str = "Bayes", negativity_factor: float = 0.0) -> float:
    """Bayes energy (src/correlations.jl:196-226).  K3_range must be 1:K as in the
    reference's determination runs (the reference indexes c3 columns from 1)."""
    if K3_range is not None and list(K3_range) != list(range(1, basis.K + 1)):
        raise TP3Error(_lib.TP3_ERR_ARG, "K3_range must be 1:K")
    if measure != "Bayes":
        return 0.0  # the reference returns res = 0.0 for any other measure
    basis._ensure_histogram(c3ref)
    return float(basis.energy_batch(np.asarray(intensity.coeff)[None])[0])
