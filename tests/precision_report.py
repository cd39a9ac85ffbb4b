"""Precision of every evaluation mode against the FP64 oracle (needs a GPU).

    python tests/precision_report.py [--configs 1,2,4] [--rotations 1000] [--out FILE.json]

For each configuration (1: L=8 K=8 N=16 LMAX=9; 2: L=18 K=26 N=32 LMAX=25;
4: L=24 K=38 N=32 LMAX=25) a seeded synthetic molecule is expanded to intensity
coefficients and R random common rotations of it are scored.  A rotation applied to
every shell leaves c3 unchanged, so one FP64 oracle evaluation (C + OpenMP triple
products, FP64 l-triple contraction) is the exact answer for all R rotated inputs,
and each rotated input gives an independent sample of a mode's rounding error.
Reported per mode (plain FP32, BF16 hi/lo x3, TF32 hi/lo x3): max |c3 - c3_64| / max|c3_64|,
RMS error / RMS c3_64, relative L1, and the relative energy error against the FP64
Bayes energy of a 1e9-triplet Poisson histogram.  Configurations 1 and 2 also report
the relative L1 distance to the reference-form restatement (f32 tables, f64
accumulation) on the unrotated structure; at configuration 4 that form needs a
24.5 GB table and is skipped.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (ROOT, os.path.join(ROOT, "threephotons.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

CONFIGS = {
    1: dict(L=8, LMAX=9, K=8, N=16, KMAX=8, rmax=8.0),
    2: dict(L=18, LMAX=25, K=26, N=32, KMAX=38, rmax=38.0),
    4: dict(L=24, LMAX=25, K=38, N=32, KMAX=38, rmax=38.0),
}


def run_config(cfg_id: int, rotations: int, batch: int = 8) -> dict:
    import torch
    import tp3
    from oracle.basis import enumerate_basis, lt_form_F
    from oracle.c3 import energy_bayes
    from oracle.refcpu import triple_products_fast, RefCPU
    from oracle.sh import seanindex, wigner_D_sampled, random_rotation3
    from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms

    c = CONFIGS[cfg_id]
    L, LMAX, K, N = c["L"], c["LMAX"], c["K"], c["N"]
    out = {"config": cfg_id, **c, "rotations": rotations}
    t0 = time.time()
    coeff = intensity_coefficients(synthetic_molecule(327, seed=101), LMAX, c["KMAX"], c["rmax"])[:K]
    b = enumerate_basis(L, LMAX, N, K)
    T64 = triple_products_fast(b, coeff)
    F = lt_form_F(b)
    c3_64 = F @ T64.T                                        # [G, klength]
    hist = loadHistograms(poisson_histogram(c3_64, K, N, 1e9, seed=7), K)
    E64 = energy_bayes(c3_64, hist, K, N)
    out["oracle_seconds"] = time.time() - t0
    out["E64"] = E64
    if cfg_id in (1, 2):
        ref = RefCPU(L, LMAX, N, K)
        c3r = ref.c3(coeff)
        out["refform_vs_fp64_relL1"] = float(np.abs(c3r - c3_64).sum() / np.abs(c3_64).sum())
    # rotated inputs
    rng = np.random.default_rng(2024 + cfg_id)
    idx = {l: [seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)] for l in range(0, L + 1, 2)}
    rot = np.empty((rotations, K, LMAX * LMAX), dtype=np.complex128)
    for r in range(rotations):
        R = random_rotation3(rng)
        x = coeff.copy()
        for l in range(2, L + 1, 2):
            x[:, idx[l]] = coeff[:, idx[l]] @ wigner_D_sampled(l, R)
        rot[r] = x
    dev = torch.device("cuda")
    ref_dev = torch.from_numpy(np.ascontiguousarray(c3_64.T)).to(dev)      # [klength, G]
    cmax = float(ref_dev.abs().max())
    crms = float(ref_dev.pow(2).mean().sqrt())
    cl1 = float(ref_dev.abs().sum())
    basis = tp3.calculate_basis(L, LMAX, N, K)
    basis.set_histogram(hist)
    modes = {"plain_fp32": tp3.TP3_MODE_PLAIN_FP32, "tc_bf16x3": tp3.TP3_MODE_TC_BF16X3,
             "tc_tf32x3": tp3.TP3_MODE_TC_TF32X3}
    out["modes"] = {}
    for name, mode in modes.items():
        try:
            basis.set_mode(mode)
        except tp3.TP3Error as e:
            out["modes"][name] = {"unavailable": str(e)}
            continue
        klength, G = basis.klength, 2 * N * N
        d_c3 = torch.empty((batch, klength, G), dtype=torch.float32, device=dev)
        d_E = torch.empty(batch, dtype=torch.float64, device=dev)
        mx, rms, l1, eerr = [], [], [], []
        for r0 in range(0, rotations, batch):
            m = min(batch, rotations - r0)
            d_in = torch.from_numpy(np.ascontiguousarray(rot[r0:r0 + m]).view(np.float64)).to(dev)
            basis.c3_batch_device(m, d_in.data_ptr(), d_c3.data_ptr())
            basis.energy_batch_device(m, d_in.data_ptr(), d_E.data_ptr())
            basis.sync()
            for i in range(m):
                d = d_c3[i].double() - ref_dev
                mx.append(float(d.abs().max()) / cmax)
                rms.append(float(d.pow(2).mean().sqrt()) / crms)
                l1.append(float(d.abs().sum()) / cl1)
            eerr += [abs(float(e) - E64) / abs(E64) for e in d_E[:m].cpu().numpy()]
        mx, rms, l1, eerr = map(np.asarray, (mx, rms, l1, eerr))
        res = {"c3_max_err_over_max": float(mx.max()), "c3_rms_err_over_rms_mean": float(rms.mean()),
               "c3_rms_err_over_rms_max": float(rms.max()), "c3_relL1_max": float(l1.max()),
               "energy_rel_err_max": float(eerr.max()), "energy_rel_err_rms": float(np.sqrt((eerr ** 2).mean()))}
        if cfg_id in (1, 2):
            basis.set_mode(mode)
            c3u = basis.c3_raw(coeff).astype(np.float64)
            res["c3_relL1_vs_refform_unrotated"] = float(np.abs(c3u - c3r).sum() / np.abs(c3r).sum())
        out["modes"][name] = res
    basis.close()
    out["seconds"] = time.time() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", default="1,2,4")
    ap.add_argument("--rotations", type=int, default=1000)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    res = [run_config(int(cid), args.rotations) for cid in args.configs.split(",")]
    txt = json.dumps(res, indent=1)
    print(txt)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
