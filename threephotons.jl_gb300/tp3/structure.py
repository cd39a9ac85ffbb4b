"""Inputs of the hot path: molecule -> intensity SH coefficients -> triplet histogram.

Host-side FP64 code (runs once per run, not per proposal).

* ``synthetic_molecule`` / ``write_pdb`` / ``loadPDB``: the PDB column layout the
  reference parser reads (src/structure.jl:30-55: serial in columns 9-11, x/y/z in
  31-38/39-46/47-54, B-factor in 62-66, element in column 78), centred on the mean
  position (structure.jl:58-70).
* ``structure_sh`` / ``createSphericalHarmonicsStructure``: the reference's route on the
  GPU (tp3_structure_sh): density shells -> s2kit-semantics transform -> spherical Bessel
  transform -> absoluteSquare, for many molecules in one call.
* ``intensity_coefficients``: SH coefficients of the intensity shells
  I(q) = |sum_j B_j exp(-R_j^2 q^2 / 2) exp(i q.r_j)|^2 (getIntensity_cartesian,
  structure.jl:80-94, atom factors structure.jl:8-16) at q_k = k pi / rmax, the
  shell spacing createSphericalHarmonicsStructure produces (forward() sets the
  Fourier-space rmax to qmax = pi KMAX / rmax, spherical_harmonics.jl:92-96, 336).
  The intensity is evaluated analytically on a Gauss-Legendre x uniform-phi grid and
  projected onto Y_lm = sphPlm(l,m,theta) e^{i m phi}: the coefficients of the
  reference's intensityShell route (s2kit transform of getIntensity_cartesian samples)
  up to the two grids' aliasing of orders >= LMAX.  createSphericalHarmonicsStructure's
  own route band-limits the density at LMAX before its Hankel transform, so its
  intensity differs from this one; ``structure_sh`` reproduces that route.
  The hot path's triple products are invariant under the (-1)^m and conjugation
  conventions of the coefficients, so the coefficient convention does not change c3.
* ``poisson_histogram`` / ``loadHistograms``: the target histogram (model c3 scaled
  to a triplet total and Poisson-sampled) and the c3ref contract of loadHistograms
  (datagen.jl:432-475): double N x N to N x 2N, clamp at 1e-30, cut to K3, normalise.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# (R, B) per element, structure.jl:8-16
ATOM_FACTORS = {
    "C": (0.7, 6.0), "N": (0.65, 7.0), "S": (1.0, 16.0), "O": (0.6, 8.0),
    "P": (0.65, 15.0), "H": (0.3, 1.0), "D": (0.3, 1.0),
}
_DEFAULT_FACTOR = (0.7, 6.0)


@dataclass
class Atom:
    index: int
    pos: np.ndarray
    element: str
    bfactor: float = 0.0


def synthetic_molecule(n_atoms: int = 327, seed: int = 0, radius: float = 13.0,
                       min_sep: float = 1.2, fractions=(0.60, 0.20, 0.18, 0.02)) -> list:
    """Seeded random molecule: C/N/O/S mix, uniform in a ball, >= min_sep apart."""
    rng = np.random.default_rng(seed)
    counts = np.floor(np.asarray(fractions) * n_atoms).astype(int)
    counts[0] += n_atoms - counts.sum()
    elements = []
    for e, c in zip("CNOS", counts):
        elements += [e] * int(c)
    rng.shuffle(elements)
    pos = []
    tries = 0
    while len(pos) < n_atoms:
        tries += 1
        if tries > 1000 * n_atoms:
            raise RuntimeError("could not place atoms; lower the count or separation")
        p = rng.uniform(-radius, radius, 3)
        if p @ p > radius * radius:
            continue
        if pos:
            d = np.asarray(pos) - p
            if np.min(np.einsum("ij,ij->i", d, d)) < min_sep * min_sep:
                continue
        pos.append(p)
    return [Atom(i + 1, np.asarray(p), e) for i, (p, e) in enumerate(zip(pos, elements))]


def write_pdb(atoms: list, path: str) -> None:
    """Write ATOM records in the fixed columns loadPDB reads (structure.jl:30-55)."""
    with open(path, "w") as f:
        for a in atoms:
            line = [" "] * 80
            def put(col, text):  # 1-based first column
                for i, ch in enumerate(text):
                    line[col - 1 + i] = ch
            put(1, "ATOM")
            put(9, f"{a.index % 1000:3d}")
            put(13, f" {a.element:<3s}")
            put(18, "GLY")
            put(31, f"{a.pos[0]:8.3f}")
            put(39, f"{a.pos[1]:8.3f}")
            put(47, f"{a.pos[2]:8.3f}")
            put(55, f"{1.0:6.2f}")
            put(62, f"{a.bfactor:5.2f}")
            put(78, a.element[0])
            f.write("".join(line).rstrip() + "\n")


def loadPDB(path: str, center: bool = True) -> list:
    """Parse ATOM records (structure.jl:30-55) and centre them (structure.jl:58-70)."""
    atoms = []
    with open(path) as f:
        for line in f:
            if len(line) > 4 and line[:4] == "ATOM":
                idx = int(line[8:11])
                x, y, z = float(line[30:38]), float(line[38:46]), float(line[46:54])
                bfac = float(line[61:66])
                t = line[77:78]
                atoms.append(Atom(idx, np.array([x, y, z]), t, bfac))
    if center and atoms:
        c = np.mean([a.pos for a in atoms], axis=0)
        for a in atoms:
            a.pos = a.pos - c
    return atoms


def _sph_plm_table(lmax_excl: int, x: np.ndarray) -> np.ndarray:
    """Orthonormal associated Legendre values with Condon-Shortley phase.

    Returns P[l, m, i] for 0 <= m <= l < lmax_excl at the cosines x[i]."""
    n = lmax_excl
    P = np.zeros((n, n, x.size))
    somx2 = np.sqrt(np.maximum(0.0, (1.0 - x) * (1.0 + x)))
    pmm = np.full(x.size, 1.0 / math.sqrt(4.0 * math.pi))
    for m in range(n):
        if m > 0:
            pmm = pmm * (-somx2) * math.sqrt((2.0 * m + 1.0) / (2.0 * m))
        P[m, m] = pmm
        if m + 1 < n:
            P[m + 1, m] = x * math.sqrt(2.0 * m + 3.0) * pmm
        for l in range(m + 2, n):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            P[l, m] = a * (x * P[l - 1, m] - b * P[l - 2, m])
    return P


def seanindex0(l: int, m: int, LMAX: int) -> int:
    """0-based seanindex (spherical_harmonics.jl:163-170 minus one)."""
    bigL = LMAX - 1
    if m >= 0:
        return m * (bigL + 1) - (m * (m - 1)) // 2 + (l - m)
    return (bigL * (bigL + 3)) // 2 + 1 + ((bigL + m) * (bigL + m + 1)) // 2 + (l - abs(m))


def intensity_coefficients(atoms: list, LMAX: int, KMAX: int, rmax: float, n_theta: int = 0,
                           n_phi: int = 0, kcount: int = 0) -> np.ndarray:
    """Intensity SH coefficients, complex128 [KMAX, LMAX^2] in seanindex order (only the
    first kcount shells computed when kcount > 0, the rest zero)."""
    n_theta = n_theta or 2 * LMAX
    n_phi = n_phi or 4 * LMAX
    xg, wg = np.polynomial.legendre.leggauss(n_theta)
    theta = np.arccos(xg)
    phi = (np.arange(n_phi) + 0.5) * (2 * math.pi / n_phi)
    st, ct = np.sin(theta), np.cos(theta)
    dirs = np.stack([np.outer(st, np.cos(phi)), np.outer(st, np.sin(phi)),
                     np.outer(ct, np.ones_like(phi))], axis=-1).reshape(-1, 3)   # [P, 3]
    wq = np.repeat(wg, n_phi) * (2 * math.pi / n_phi)                             # [P]
    pos = np.array([a.pos for a in atoms])
    RB = np.array([ATOM_FACTORS.get(a.element, _DEFAULT_FACTOR) for a in atoms])
    Plm = _sph_plm_table(LMAX, xg)                                                # [l, m, n_theta]
    # conj(Y_lm) on the grid, columns in seanindex order
    Yc = np.zeros((n_theta * n_phi, LMAX * LMAX), dtype=np.complex128)
    for l in range(LMAX):
        for m in range(-l, l + 1):
            ma = abs(m)
            plm = Plm[l, ma] * ((-1.0) ** ma if m < 0 else 1.0)
            val = np.outer(plm, np.exp(-1j * m * phi)).reshape(-1)
            Yc[:, seanindex0(l, m, LMAX)] = val
    dq = math.pi / rmax
    proj = dirs @ pos.T                                                           # [P, atoms]
    out = np.zeros((KMAX, LMAX * LMAX), dtype=np.complex128)
    for k in range(1, (kcount or KMAX) + 1):
        q = k * dq
        f = RB[:, 1] * np.exp(-0.5 * RB[:, 0] ** 2 * q * q)
        amp = np.exp(1j * q * proj) @ f
        I = (amp.real ** 2 + amp.imag ** 2) * wq
        out[k - 1] = I @ Yc
    return out


_SH_BASIS = None


def _sh_basis():
    """A small context that carries the stream and error state of structure_sh calls."""
    global _SH_BASIS
    if _SH_BASIS is None:
        from .api import calculate_basis
        _SH_BASIS = calculate_basis(2, 3, 4, 2)
    return _SH_BASIS


def atom_table(atoms: list) -> np.ndarray:
    """[n][5] rows (x, y, z, R, B) with the element's atom factor (structure.jl:8-16)."""
    return np.array([[*a.pos, *ATOM_FACTORS.get(a.element, _DEFAULT_FACTOR)] for a in atoms],
                    dtype=np.float64).reshape(-1, 5)


def structure_sh(molecules: list, LMAX: int, KMAX: int, rmax: float, route: str = "reference",
                 basis=None) -> dict:
    """SH coefficients of many molecules on the GPU (tp3_structure_sh), complex128
    [n_mol, KMAX, LMAX^2] in seanindex order.

    route "reference": the route of createSphericalHarmonicsStructure (structure.jl:125-134):
    density shells at r_k = k rmax / KMAX -> s2kit-semantics transform -> forward spherical
    Bessel transform -> absoluteSquare; returns {"density", "amplitude", "intensity"}.
    route "intensity": transform of |F(q_k)|^2 sampled on the same grid (intensityShell);
    returns {"intensity"}.  Amplitude and intensity shells sit at q_k = k pi / rmax."""
    from . import _lib
    b = basis or _sh_basis()
    code = {"reference": _lib.TP3_SH_REFERENCE, "intensity": _lib.TP3_SH_INTENSITY}[route]
    tabs = [atom_table(m) for m in molecules]
    atoms = np.ascontiguousarray(np.concatenate(tabs) if tabs else np.zeros((0, 5)))
    start = np.zeros(len(molecules) + 1, dtype=np.int32)
    start[1:] = np.cumsum([t.shape[0] for t in tabs])
    shape = (len(molecules), KMAX, LMAX * LMAX)
    outs = {k: np.zeros(shape, dtype=np.complex128) for k in
            (("density", "amplitude", "intensity") if code == _lib.TP3_SH_REFERENCE else ("intensity",))}
    ptr = lambda k: outs[k].ctypes.data if k in outs else None  # noqa: E731
    _lib.check(b._lib.tp3_structure_sh(b._ctx, atoms.ctypes.data, start.ctypes.data, len(molecules), LMAX, KMAX,
                                       float(rmax), code, ptr("density"), ptr("amplitude"), ptr("intensity")),
               b._ctx)
    return outs


def createSphericalHarmonicsStructure(pdb_path: str, LMAX: int, KMAX: int, rmax: float):
    """(density, fourierTransform, intensity) of a PDB structure as SphericalHarmonicsVolume
    objects, by the reference's route on the GPU (structure.jl:125-134): the density with
    rmax, the amplitude and intensity with rmax = qmax = pi KMAX / rmax."""
    from .api import SphericalHarmonicsVolume
    out = structure_sh([loadPDB(pdb_path)], LMAX, KMAX, rmax, route="reference")
    qmax = math.pi * KMAX / rmax
    return (SphericalHarmonicsVolume(out["density"][0], LMAX, KMAX, rmax),
            SphericalHarmonicsVolume(out["amplitude"][0], LMAX, KMAX, qmax),
            SphericalHarmonicsVolume(out["intensity"][0], LMAX, KMAX, qmax))


def tripletFactor(k1: int, k2: int, k3: int) -> float:
    """datagen.jl:166-174."""
    if k1 == k2 == k3:
        return 1.0
    if k1 == k2 or k1 == k3 or k2 == k3:
        return 3.0
    return 6.0


def raw_to_5d(c3_raw: np.ndarray, K: int, N: int) -> np.ndarray:
    """G x klength raw correlation -> N x 2N x K x K x K (correlations.jl:186-191)."""
    t = np.zeros((N, 2 * N, K, K, K), dtype=np.float64, order="F")
    i = 0
    for k1 in range(1, K + 1):
        for k2 in range(1, k1 + 1):
            for k3 in range(1, k2 + 1):
                t[:, :, k3 - 1, k2 - 1, k1 - 1] = c3_raw[:, i].reshape(N, 2 * N, order="F")
                i += 1
    return t


def poisson_histogram(c3_raw: np.ndarray, K: int, N: int, triplets: float, seed: int) -> np.ndarray:
    """Model c3 (G x klength) scaled to `triplets` counts and Poisson-sampled -> 5-D counts."""
    rng = np.random.default_rng(seed)
    p = np.maximum(np.asarray(c3_raw, dtype=np.float64), 0.0)
    lam = p * (triplets / p.sum())
    counts = rng.poisson(lam).astype(np.float64)
    return raw_to_5d(counts, K, N)


def loadHistograms(c3_full: np.ndarray, K3: int) -> np.ndarray:
    """c3 contract of loadHistograms (datagen.jl:445-468)."""
    NA, NB = c3_full.shape[0], c3_full.shape[1]
    if NA == NB:
        c3_full = np.concatenate([c3_full, c3_full], axis=1)
    c3_full = np.maximum(c3_full, 1e-30)
    c3 = c3_full[:, :, :K3, :K3, :K3]
    return np.asfortranarray(c3 / np.sum(np.abs(c3)))
